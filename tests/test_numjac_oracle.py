"""The restated Jacobian checker (tests/numjac_check.py, the reference's
numerical_jacobian in its bracketed form, Debug = -2) on the CPU oracle's
assembly: it flags exactly what the reference's own checker flagged on the
same golden problems and states (tests/golden/numjac_reference.json,
produced by running the reference), and it does flag a wrong Jacobian entry
planted in the oracle's output."""
import json
import os

import numpy as np
import pytest

import oracle
from tests import golden_cases as gc
from tests import numjac_check as nj

REF = os.path.join(gc.GOLDEN, "numjac_reference.json")


def _oracle_fill(o, plant=None):
    ija = o.ija()

    def fill(x):
        R, a, st = o.matrix_fill(x)
        assert st == 0
        A = nj.msr_to_dense(ija, a)
        if plant is not None:
            i, j, f = plant
            A[i, j] *= f
        return R, A
    return fill


def _layout(o, prob):
    return nj.Layout(prob, o.first_unknown(prob.mesh.num_nodes))


@pytest.mark.parametrize("name", ["cav2d_2x2", "cav2d_3x2_pert", "bfs2d_4x2_carreau",
                                  "bratu2d_4x4_pert", "channel2d_4x3_ibc"])
def test_checker_on_oracle_flags_what_the_reference_flagged(name):
    with open(REF) as f:
        ref = json.load(f)[name]
    g, case = gc.load(name)
    prob = nj.without_dirichlet(gc.problem_from_case(case))
    o = oracle.Oracle(prob)
    assert o.N == ref["columns"]
    flagged = nj.check(_layout(o, prob), _oracle_fill(o), g["x"])
    assert len(flagged) == len(ref["flagged"]) == 0, flagged[:5]


def test_checker_flags_a_jacobian_entry_planted_wrong_in_the_oracle():
    g, case = gc.load("cav2d_3x2_pert")
    prob = nj.without_dirichlet(gc.problem_from_case(case))
    o = oracle.Oracle(prob)
    R, A = _oracle_fill(o)(g["x"])
    # the largest off-diagonal entry, 10 % too large
    off = np.abs(A) * (~np.eye(o.N, dtype=bool))
    i, j = np.unravel_index(np.argmax(off), off.shape)
    flagged = nj.check(_layout(o, prob), _oracle_fill(o, (i, j, 1.1)), g["x"])
    assert ("bracket", int(i), int(j)) in flagged
