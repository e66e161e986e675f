"""The continuation driver's host logic (goma_gb300/continuation.py, after
continue_problem, src/ac_conti.c:106) on a CPU stand-in for the Newton
solver: a diagonal cubic system R(x; lam) = x + c x^3 - lam b, solved by
Newton in numpy.  The stand-in fails a solve whose guess is farther than
`reach` from the solution, as a diverging Newton solve would, so step
halving (src/ac_conti.c:986-1045) can be exercised.  Checks: the parameter
schedule (uniform and log), the zeroth-order and secant guesses, halving
and its limit, the time budget, and the records."""
import numpy as np
import pytest

from goma_gb300.continuation import continuation


class CubicNewton:
    def __init__(self, n=40, reach=None):
        rng = np.random.default_rng(0)
        self.b = rng.uniform(0.5, 1.5, n)
        self.c = 0.3
        self.lam = 0.0
        self.N = n
        self.reach = reach
        self.guess_errors = []

    def dirichlet_init(self, x):
        return np.array(x, dtype=float)

    def exact(self, lam):
        x = np.zeros(self.N)
        for _ in range(60):
            x -= (x + self.c * x ** 3 - lam * self.b) / (1.0 + 3.0 * self.c * x ** 2)
        return x

    def solve_nonlinear_problem(self, x0=None, **opts):
        x = np.zeros(self.N) if x0 is None else np.array(x0, dtype=float)
        err = np.abs(x - self.exact(self.lam)).max()
        self.guess_errors.append((self.lam, err))
        st = {"newton_its": 0, "linear_its": 0, "factorizations": 0, "assemble_ms": 0.0,
              "scale_ms": 0.0, "factor_ms": 0.0, "solve_ms": 0.0, "total_ms": 0.0}
        if self.reach is not None and err > self.reach:
            return x, False, st
        for it in range(50):
            r = x + self.c * x ** 3 - self.lam * self.b
            if it > 0 and np.abs(r).max() < 1e-13:
                break
            x -= r / (1.0 + 3.0 * self.c * x ** 2)
            st["newton_its"] += 1
            st["linear_its"] += 1
            st["factorizations"] += 1
        return x, True, st


def set_lam(gn, lam):
    gn.lam = lam


@pytest.mark.parametrize("spacing", ["linear", "log"])
@pytest.mark.parametrize("predictor", ["zeroth", "secant"])
def test_sweep_reaches_the_end_point(predictor, spacing):
    gn = CubicNewton()
    recs, x = continuation(gn, 0.5, 4.0, 6, predictor=predictor, set_param=set_lam,
                           spacing=spacing)
    lams = [r["lam"] for r in recs]
    want = (np.linspace(0.5, 4.0, 7) if spacing == "linear"
            else np.exp(np.linspace(np.log(0.5), np.log(4.0), 7)))
    assert np.allclose(lams, want)
    assert np.abs(x - gn.exact(4.0)).max() < 1e-12
    assert recs[0]["guess"] == "initial"
    expected = ["zeroth"] * 6 if predictor == "zeroth" else ["zeroth"] + ["secant"] * 5
    assert [r["guess"] for r in recs[1:]] == expected
    assert all(r["halvings"] == 0 for r in recs[1:])


def test_secant_guesses_are_closer_than_zeroth():
    errs = {}
    for pred in ("zeroth", "secant"):
        gn = CubicNewton()
        continuation(gn, 0.5, 4.0, 8, predictor=pred, set_param=set_lam)
        errs[pred] = np.array([e for _, e in gn.guess_errors[2:]])  # steps with a secant
    assert np.all(errs["secant"] < 0.5 * errs["zeroth"])


def test_a_failed_step_is_halved_and_the_sweep_goes_on():
    gn = CubicNewton()
    full = np.abs(gn.exact(4.0) - gn.exact(0.5)).max()
    gn.reach = 0.6 * full  # the whole step fails, its halves succeed
    recs, x = continuation(gn, 0.5, 4.0, 1, predictor="zeroth", set_param=set_lam)
    assert np.abs(x - gn.exact(4.0)).max() < 1e-12
    assert recs[1]["halvings"] >= 1 and recs[1]["lam"] < 4.0
    assert recs[-1]["lam"] == 4.0
    lams = [r["lam"] for r in recs]
    assert np.all(np.diff(lams) > 0)


def test_too_many_halvings_raise():
    gn = CubicNewton()
    gn.reach = 1e-6
    with pytest.raises(RuntimeError, match="continuation step at lambda"):
        continuation(gn, 0.5, 4.0, 1, predictor="zeroth", x0=gn.exact(0.5), set_param=set_lam,
                     max_halvings=2)
    assert len(gn.guess_errors) == 1 + 3  # the start, the step and its two halvings


def test_time_budget_and_bad_predictor():
    gn = CubicNewton()
    recs, _ = continuation(gn, 0.5, 4.0, 5, set_param=set_lam, time_budget_s=0.0)
    assert len(recs) == 1
    with pytest.raises(ValueError):
        continuation(gn, 0.5, 4.0, 5, predictor="quadratic", set_param=set_lam)
