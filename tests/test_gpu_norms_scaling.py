"""Direct parity of two small steps of the Newton loop:

- row-sum scaling (row_sum_scaling_scale / row_sum_scale_MSR,
  src/sl_matrix_util.c:441,506) on the device, gb_row_sum_scale_device, on
  the reference's own assembled matrices (every golden fixture): the scale
  vector, the scaled residual and the scaled matrix equal the oracle's;
- the residual norms the Newton driver reports per step (L_oo, L_1, L_2 of
  the scaled residual, src/mm_sol_nonlinear.c:1451-1453 and
  L2_norm / L1_norm / Loo_norm :3177-3530) against the norms the reference
  itself printed when it solved the same golden problems, at the printed
  precision (two significant digits), and the same Newton step count.
"""
import re

import numpy as np
import pytest

import oracle
from goma_gb300.newton import GomaNewton
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu


def _csr_from_msr(gn, a_msr):
    rp, ci = gn.csr_pattern()
    N = gn.N
    rows = np.repeat(np.arange(N), np.diff(rp))
    k = np.arange(len(ci))
    off = np.where(ci == rows, -1, N + 1 + k - rows - (ci > rows))
    vals = np.where(ci == rows, a_msr[rows], a_msr[np.maximum(off, 0)])
    return vals


@pytest.mark.parametrize("name", gc.names())
def test_device_row_sum_scaling_matches_the_oracle_on_reference_matrices(name):
    import torch
    g, case = gc.load(name)
    prob = gc.problem_from_case(case)
    gn = GomaNewton(prob)
    o = oracle.Oracle(prob)
    a, R = g["a"], g["R"]
    a_s, R_s, s_ref = o.row_sum_scale(a, R)
    vals = torch.tensor(_csr_from_msr(gn, a), dtype=torch.float64, device="cuda")
    dR = torch.tensor(R, dtype=torch.float64, device="cuda")
    ds = torch.empty(gn.N, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    gn.scale_device(vals.data_ptr(), dR.data_ptr(), ds.data_ptr())
    gn.status()
    torch.cuda.synchronize()
    s = ds.cpu().numpy()
    assert np.abs(s - s_ref).max() <= 1e-14 * np.abs(s_ref).max()
    assert np.array_equal(np.sign(s), np.sign(s_ref))
    assert np.abs(dR.cpu().numpy() - R_s).max() <= 1e-14 * max(np.abs(R_s).max(), 1e-300)
    a_dev = gn.csr_to_msr(vals.data_ptr())
    assert gc.msr_row_scaled_error(o.ija(), a_dev, a_s) <= 1e-14


def _reference_norms(log):
    """(L_oo, L_1, L_2) of the scaled residual per Newton step, as printed."""
    out = []
    for line in str(log).splitlines():
        m = re.search(r"\[(\d+)\]\s+(\S+)\s+(\S+)\s+(\S+)", line)
        if m:
            out.append((int(m.group(1)), float(m.group(2)), float(m.group(3)),
                        float(m.group(4))))
    return out


def _printed_close(value, printed):
    """value rounds to printed at %7.1e (half a unit in the second digit)."""
    if printed == 0.0:
        return abs(value) < 5e-300
    e = np.floor(np.log10(abs(printed)))
    return abs(value - printed) <= 0.5 * 10.0 ** (e - 1) * 1.001


@pytest.mark.parametrize("name", gc.names("solve") + gc.names("solve", compact=True))
def test_newton_residual_norms_match_the_reference_log(name):
    g, case = gc.load(name)
    gn = GomaNewton(gc.problem_from_case(case))
    x0 = g["x0"] if "x0" in g else None
    x, conv, st = gn.solve_nonlinear_problem(x0, residual_tol=case.get("tol", 1e-11),
                                             linear_tol=1e-13, max_linear_its=3000,
                                             krylov_dim=60, max_newton=30)
    assert conv, st
    ref = _reference_norms(g["newton_log"])
    assert ref, "no norms in the reference's log"
    assert abs(st["newton_its"] - ref[-1][0]) <= 1
    first = ref[0][3]
    checked = 0
    for it, loo, l1, l2 in ref:
        if it >= len(st["residual_l2"]) or l2 < 1e-9 * max(first, 1.0):
            continue   # below this the printed digits are the linear solver's rounding
        assert _printed_close(st["residual_loo_steps"][it], loo), (it, loo)
        assert _printed_close(st["residual_l1"][it], l1), (it, l1)
        assert _printed_close(st["residual_l2"][it], l2), (it, l2)
        checked += 1
    assert checked >= 2
