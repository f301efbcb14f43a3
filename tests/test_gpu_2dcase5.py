"""tests/testcase/2Dcase5 of the reference: 78,190 triangles, gray band, 32
directions, specular side walls.  Against the reference's own CPU code built
here (ref.npz, margin <= 1e-5, 40 outer iterations) and against the
reference's recorded GPU run (StaticBTESolver-2DM-1np.sol: 37 outer
iterations to margin < 1e-4, 4.78 s per outer iteration on the reference's
GPU, q0 = -1.29714e9)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _solve(sbte, c, **kw):
    prob = sbte.Problem(*c.args())
    ctx = sbte.Context(0).load(prob)
    st, rep = ctx.solve(**kw)
    res = ctx.result(st, rep)
    ctx.close()
    return res


PLAIN_2DCASE5 = pytest.mark.xfail(
    reason="the reference's right-Jacobi BiCGSTAB needs 560-1,100 iterations on this mesh's nearly pure "
           "advection systems (upwind graphs 560-810 levels deep) and the count of each system is decided by "
           "rounding (one part in 1e15 of the right-hand side moves it by hundreds: "
           "tests/test_bicgstab_sensitivity.py), so whether every system of a run stops within the reference's "
           "1,000 iterations is luck; on GB300 some do not and their last iterates stall the outer iteration "
           "near margin 1e10", strict=False)


@pytest.mark.parametrize("form_name,tol", [("FORM_SWEEP", 1e-6), pytest.param("FORM_PLAIN", 1e-6, marks=PLAIN_2DCASE5),
                                           ("FORM_MIXED", 1e-5)])
def test_2dcase5_matches_reference_build(sbte, get_case, form_name, tol):
    c = get_case("2Dcase5")
    res = _solve(sbte, c, max_iter=c.max_iter, tol=1e-5, form=getattr(sbte, form_name))
    assert res.status == 0
    assert res.report["n_iter"] == int(c.ref["n_iter"])
    assert rel_l2(res.T - 300, c.ref["T"] - 300) < tol
    np.testing.assert_allclose(res.q[[0, 3]], c.ref["q"][[0, 3]], rtol=tol)
    print(form_name, "ms per outer iteration", res.report["ms_total"] / res.report["n_iter"],
          "(the reference's GPU run: 4,780)")


def test_2dcase5_against_recorded_gpu_run(sbte, get_case):
    c = get_case("2Dcase5")
    res = _solve(sbte, c, max_iter=c.max_iter, tol=1e-4 * (1 - 1e-12), form=sbte.FORM_SWEEP)
    logged = c.meta["gpu_sol_margins"]
    assert len(res.margins) == len(logged)
    for a, b in zip(res.margins, logged):
        if b > 1.0:  # below ~1 the margins are differences at the inner-solver noise level
            assert abs(a - b) <= 1e-4 * b, (a, b)
    q = c.meta["gpu_sol_heat_flux"]
    assert abs(res.q[0] - q[0]) <= 1e-5 * abs(q[0])
    assert abs(res.q[3] - q[3]) <= 1e-5 * abs(q[3])


def test_2dcase5_anderson(sbte, get_case):
    """The plain iteration already converges fast here (40 steps, specular walls);
    Anderson mixing over T and the boundary-cell intensities must not slow it."""
    c = get_case("2Dcase5")
    res = _solve(sbte, c, max_iter=c.max_iter, tol=1e-5, form=sbte.FORM_SWEEP, accel=3, accel_every=8)
    assert res.status == 0 and res.report["n_iter"] <= int(c.ref["n_iter"]) + 2
    assert rel_l2(res.T - 300, c.ref["T"] - 300) < 1e-5
