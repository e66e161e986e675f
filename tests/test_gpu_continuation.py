"""Reynolds-number continuation of the Carreau channel: zeroth-order,
first-order (tangent) and learned initial guesses.  All three must reach
the same converged solutions (the Newton solve decides); the learned guess,
with the reference's predictor as fallback, must not need more Newton
iterations than the zeroth-order predictor it replaces."""
import numpy as np
import pytest

from goma_gb300 import problem as pb
from goma_gb300.continuation import continuation
from goma_gb300.newton import GomaNewton

pytestmark = pytest.mark.gpu

OPTS = dict(residual_tol=1e-10, linear_tol=1e-10, max_newton=30, max_linear_its=2000)


def _run(pred, nx=12, ny=4, steps=8):
    prob = pb.carreau_step_2d(nx, ny, 10.0)
    gn = GomaNewton(prob)
    recs, x = continuation(gn, 10.0, 200.0, steps, predictor=pred, newton_opts=OPTS,
                           learned_opts=dict(steps=300, batch=2048, lr=2e-3))
    return recs, x


def test_continuation_predictors_agree_and_learned_helps():
    """The network with only the zeroth-order fallback: every Newton
    iteration it saves is the network's doing."""
    rz, xz = _run("zeroth")
    rf, xf = _run("first")
    rl, xl = _run("learned")
    rlf, xlf = _run("learned+first")
    scale = np.abs(xz).max()
    for xo in (xf, xl, xlf):
        assert np.abs(xo - xz).max() <= 1e-8 * scale
    its = {name: sum(r["newton_its"] for r in recs[1:])
           for name, recs in (("zeroth", rz), ("first", rf), ("learned", rl),
                              ("learned+first", rlf))}
    print("newton iterations over the sweep:", its)
    print("learned-step guesses:", [r["guess"] for r in rl[1:]])
    assert its["first"] <= its["zeroth"]
    assert its["learned+first"] <= its["first"]
    # the network's own gain over the method without it
    assert any(r["guess"] == "learned" for r in rl[1:])
    assert its["learned"] < its["zeroth"]
