"""Reynolds-number continuation of the Carreau channel: zeroth-order,
first-order (tangent), secant and learned initial guesses.  All must reach
the same converged solutions (the Newton solve decides).  The learned guess
is the secant guess plus the network's curvature correction, with the plain
secant guess as its fallback, so what the network gains over the method
without it shows in the learned run against the secant run."""
import math

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
                           learned_opts=dict(steps=1500, batch=2048, lr=2e-3))
    return recs, x


def test_continuation_predictors_agree_and_learned_helps():
    runs = {p: _run(p) for p in ("zeroth", "first", "secant", "learned", "learned+first")}
    xz = runs["zeroth"][1]
    scale = np.abs(xz).max()
    for name, (_, xo) in runs.items():
        assert np.abs(xo - xz).max() <= 1e-8 * scale, name
    its = {n: sum(r["newton_its"] for r in recs[1:]) for n, (recs, _) in runs.items()}
    rl = runs["learned"][0]
    print("newton iterations over the sweep:", its)
    print("per-step Newton iterations:",
          {n: [r["newton_its"] for r in recs[1:]] for n, (recs, _) in runs.items()})
    print("learned-run guesses:", [r["guess"] for r in rl[1:]])
    print("learned-run candidate residuals:", [r["candidates"] for r in rl[1:]])
    assert its["first"] <= its["zeroth"]
    assert its["secant"] <= its["zeroth"]
    assert its["learned"] <= its["secant"]
    assert its["learned+first"] <= its["first"]
    # the network's own gain over the secant guess it corrects: wherever both
    # guesses were formed, the learned one's residual relative to the secant's
    ratios = [r["candidates"]["learned"] / r["candidates"]["secant"] for r in rl[1:]
              if "learned" in r["candidates"] and "secant" in r["candidates"]]
    print("learned / secant guess residual per step:", ["%.3g" % q for q in ratios])
    assert ratios, "the network never produced a guess"
    assert min(ratios) < 0.9
    gm = math.exp(sum(math.log(min(q, 1.0)) for q in ratios) / len(ratios))
    assert gm < 1.0
