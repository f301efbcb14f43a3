"""The upwind-sweep form (BTE_FORM_SWEEP): exact inner solves by level-ordered
forward substitution.  It solves the same systems as the reference's inner
solvers, so it reaches the same outer fixed point: relative L2 of T - T_ref
<= 1e-6 against the reference's own CPU code, same outer iteration counts."""
import numpy as np
import pytest

from conftest import SYNTH_CASES, TESTSH_CASES, rel_l2

pytestmark = pytest.mark.gpu


def _solve(sbte, c, **kw):
    p = sbte.Problem(*c.args())
    ctx = sbte.Context(0).load(p)
    st, rep = ctx.solve(**kw)
    res = ctx.result(st, rep)
    ctx.close()
    return res


@pytest.mark.parametrize("name", TESTSH_CASES + SYNTH_CASES + ["2Dcase2"])
def test_sweep_matches_reference_build(sbte, get_case, name):
    c = get_case(name)
    res = _solve(sbte, c, max_iter=c.max_iter, tol=1e-5, form=sbte.FORM_SWEEP)
    assert res.status == 0
    assert res.report["n_iter"] == int(c.ref["n_iter"])
    Tr = 0.0 if name in ("2DM1DG", "3DM1DG", "slab1d") else c.T_ref
    assert rel_l2(res.T - Tr, c.ref["T"] - Tr) < 1e-6
    q, qr = res.q, c.ref["q"]
    big = np.abs(qr) > 1e-3 * np.abs(qr).max()
    np.testing.assert_allclose(q[big], qr[big], rtol=1e-6)
    # exact inner solves: one sweep per system on these (acyclic) meshes
    assert res.report["inner_iterations"] == res.report["inner_solves"]


@pytest.mark.parametrize("name", ["2DM2DG", "3DM2DG", "3DM3DG"])
def test_sweep_matches_sol_logs(sbte, get_case, name):
    c = get_case(name)
    res = _solve(sbte, c, max_iter=c.max_iter, tol=1e-4 * (1 - 1e-12), form=sbte.FORM_SWEEP)
    logged = c.meta["sol_margins"]
    assert len(res.margins) == len(logged)
    q_logged = np.array(c.meta["sol_heat_flux"])
    big = np.abs(q_logged) > 1e-3 * np.abs(q_logged).max()
    np.testing.assert_allclose(res.q[big], q_logged[big], rtol=6e-6)


def test_sweep_with_cycles_matches_bicgstab(sbte, get_case):
    """Upwind graphs with cycles: lagged edges and repeated Gauss-Seidel sweeps.

    Flipping the stored normal of one side of an interior face makes both cells
    see that face as inflow for half of the directions (a 2-cycle)."""
    c = get_case("2DM2DG")
    p = sbte.Problem(*c.args())
    a = p.arrays()
    nbr, nrm = a["nbr"], a["normal"].copy()
    flipped = 0
    for cell in range(0, p.n_cell, 37):
        for f in range(p.n_face):
            if nbr[cell, f] >= 0:
                nrm[cell, f] *= -1.0
                flipped += 1
                break
    a["normal"] = nrm
    out = {}
    for form in (sbte.FORM_PLAIN, sbte.FORM_SWEEP):
        ctx = sbte.Context(0).set_arrays(a)
        st, rep = ctx.solve(max_iter=200, tol=1e-5, form=form)
        out[form] = (ctx.temperature(), rep.as_dict())
        ctx.close()
    Tp, rp = out[sbte.FORM_PLAIN]
    Ts, rs = out[sbte.FORM_SWEEP]
    assert flipped > 5
    assert rs["inner_iterations"] > rs["inner_solves"]  # some systems needed more than one sweep
    assert rs["n_iter"] == rp["n_iter"]
    assert rel_l2(Ts - 300, Tp - 300) < 1e-6
