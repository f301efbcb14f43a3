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


def _rewired(sbte, c, n_swaps=40, seed=0):
    """Geometry arrays whose upwind graphs have cycles.

    Planar meshes never do (interior-disjoint convex cells in the plane admit a
    translation order for every direction), so partners of interior face
    pairs are exchanged: (c1,f1)<->(c2,f2) and (c3,f3)<->(c4,f4) become
    (c1,f1)<->(c4,f4) and (c3,f3)<->(c2,f2), for faces with nearly the same
    normal and area so the flux stays conserved.  Every row keeps its own
    faces' areas and normals, so each system stays a diagonally dominant
    M-matrix of the reference's form; the long links close cycles."""
    p = sbte.Problem(*c.args())
    a = p.arrays()
    nbr = a["nbr"].copy()
    nrm, area = a["normal"], a["area"]
    rng = np.random.default_rng(seed)
    pairs = [(cc, f) for cc in range(p.n_cell) for f in range(p.n_face) if nbr[cc, f] > cc]
    back = lambda cc, f: int(np.nonzero(nbr[nbr[cc, f]] == cc)[0][0])
    used = set()
    for _ in range(200 * n_swaps):
        if len(used) >= 4 * n_swaps:
            break
        i, j = rng.choice(len(pairs), 2, replace=False)
        (c1, f1), (c3, f3) = pairs[i], pairs[j]
        if np.dot(nrm[c1, f1], nrm[c3, f3]) < 0.995 or abs(area[c1, f1] / area[c3, f3] - 1) > 0.05:
            continue
        c2, c4 = nbr[c1, f1], nbr[c3, f3]
        if len({c1, c2, c3, c4} & used) or len({c1, c2, c3, c4}) < 4:
            continue
        f2, f4 = back(c1, f1), back(c3, f3)
        nbr[c1, f1], nbr[c4, f4] = c4, c1
        nbr[c3, f3], nbr[c2, f2] = c2, c3
        used |= {c1, c2, c3, c4}
    a["nbr"] = nbr
    return a


def test_sweep_with_cycles_matches_bicgstab(sbte, get_case):
    """Cycles in the upwind graph: lagged edges and repeated Gauss-Seidel sweeps."""
    c = get_case("square16_b8")
    a = _rewired(sbte, c, n_swaps=10)
    out = {}
    for form in (sbte.FORM_PLAIN, sbte.FORM_SWEEP):
        ctx = sbte.Context(0).set_arrays(a)
        st, rep = ctx.solve(max_iter=3000, tol=1e-5, form=form)
        out[form] = (st, ctx.temperature(), rep.as_dict())
        ctx.close()
    sp, Tp, rp = out[sbte.FORM_PLAIN]
    ss, Ts, rs = out[sbte.FORM_SWEEP]
    assert sp == 0 and ss == 0, (sp, ss, rp, rs)
    assert rs["inner_iterations"] > rs["inner_solves"]  # some systems needed more than one sweep
    assert rs["inner_unconverged"] == 0
    assert rs["n_iter"] == rp["n_iter"]
    assert rel_l2(Ts - 300, Tp - 300) < 1e-6


@pytest.mark.parametrize("name", ["square16_b8", "3DM2DG", "square16_b8/cycles"])
def test_sweep_margin_placements_agree(sbte, get_case, monkeypatch, name):
    """The margin of an acyclic plan is summed either by the sweep (one more
    load and two FP64 operations per cell-system) or by k_reduce (e_prev read
    again); the autotuner times both.  Forced either way the temperatures agree
    to the bit, on 2D and 3D plans (two and three face slots), and the margins
    to rounding (the partials are grouped differently).  With lagged edges the
    reduction always sums it."""
    c = get_case(name.split("/")[0])
    runs = {}
    for placement in ("0", "1"):
        monkeypatch.setenv("BTE_SWEEP_MARGIN", placement)
        if name.endswith("/cycles"):
            ctx = sbte.Context(0).set_arrays(_rewired(sbte, c, n_swaps=10))
            st, rep = ctx.solve(max_iter=3000, tol=1e-5, form=sbte.FORM_SWEEP)
        else:
            ctx = sbte.Context(0).load(sbte.Problem(*c.args()))
            st, rep = ctx.solve(max_iter=c.max_iter, tol=1e-5, form=sbte.FORM_SWEEP)
        runs[placement] = (st, ctx.temperature(), ctx.margins(), rep.as_dict(), ctx.sweep_tuning())
        ctx.close()
    (s0, T0, m0, r0, t0), (s1, T1, m1, r1, t1) = runs["0"], runs["1"]
    assert s0 == 0 and s1 == 0
    assert r0["sweep_margin"] == 0 and r1["sweep_margin"] == (0 if name.endswith("/cycles") else 1), (r0, r1)
    # the autotuner's table (empty when the shape came from the per-process cache)
    for t in t0 + t1:
        assert t["ms"] > 0 and t["threads"] in (32, 64, 128, 256) and t["ring"] * t["group"] <= 4096
    assert r0["n_iter"] == r1["n_iter"] and r0["inner_iterations"] == r1["inner_iterations"]
    assert np.array_equal(T0, T1)
    np.testing.assert_allclose(m0, m1, rtol=1e-12, atol=0)



def _odd_slab(c):
    """slab1d with 101 cells: rows of the per-system arrays are padded to an even length."""
    args = list(c.args())
    args[0] = "101"
    return tuple(args)


@pytest.mark.parametrize("name,shape", [("square16_b8", None), ("square16_b8", "4,64"), ("2DM2DG", None),
                                        ("3DM2DG", None), ("cube5_b8", "4,64"), ("square16_b8/cycles", None),
                                        ("slab1d/odd", None), ("2Dcase5", None)])
def test_sweep_kernels_agree(sbte, get_case, monkeypatch, tmp_path, name, shape):
    """The sweep kernels compute the same x to the bit: the
    level-synchronous one, the same over levels split into slices of one
    position per thread, and the staged one (levels copied into shared memory
    ahead of use by bulk copies, right-hand side formed beforehand in level
    order).  Same temperatures, margins (summed by k_reduce here) and
    iteration counts, on 1D, 2D and 3D plans, with lagged edges, with an odd
    cell count, and with stages narrower than a level (shape 4,64: 32
    positions per stage)."""
    from staticbtesolver_gb300 import synth

    base = name.split("/")[0]
    if base.startswith("cube"):
        p = synth.make_problem(base, str(tmp_path))
        args, max_iter = (p.geo, p.bc_file, p.band_file, p.DM, p.num_theta, p.num_phi, p.T_ref, p.L_x, p.L_y,
                          p.L_z), 1000
    else:
        c = get_case(base)
        args, max_iter = (_odd_slab(c) if name.endswith("/odd") else c.args()), c.max_iter
    monkeypatch.setenv("BTE_SWEEP_MARGIN", "0")
    runs = {}
    if shape:
        monkeypatch.setenv("BTE_SWEEP_SHAPE", shape)
    for kernel in ("level", "staged", "split"):
        monkeypatch.setenv("BTE_SWEEP_KERNEL", kernel)
        if name.endswith("/cycles"):
            ctx = sbte.Context(0).set_arrays(_rewired(sbte, c, n_swaps=10))
            st, rep = ctx.solve(max_iter=3000, tol=1e-5, form=sbte.FORM_SWEEP)
        else:
            ctx = sbte.Context(0).load(sbte.Problem(*args))
            st, rep = ctx.solve(max_iter=max_iter, tol=1e-5, form=sbte.FORM_SWEEP)
        runs[kernel] = (st, ctx.temperature(), ctx.margins(), rep.as_dict(), ctx.sweep_tuning())
        ctx.close()
    s0, T0, m0, r0, t0 = runs["level"]
    for kid, kernel in ((1, "staged"), (2, "split")):
        s1, T1, m1, r1, t1 = runs[kernel]
        assert s0 == s1 and s0 in (0, 6)
        assert r0["sweep_kernel"] == 0 and r1["sweep_kernel"] == kid, (r0, r1)
        assert all(t["kernel"] == "level" for t in t0) and all(t["kernel"] == kernel for t in t1)
        if shape:
            assert all((t["group"], t["threads"]) == (4, 64) for t in t0 + t1)
        assert r0["n_iter"] == r1["n_iter"] and r0["inner_iterations"] == r1["inner_iterations"]
        assert np.array_equal(T0, T1), kernel
        assert np.array_equal(m0, m1), kernel


@pytest.mark.parametrize("name", ["square16_b8", "2DM2DG", "3DM2DG", "cube5_b8", "square16_b8/cycles", "slab1d/odd",
                                  "2Dcase5", "2Dcase5/global", "cube5_b8/global", "square100k"])
def test_device_level_order_matches_host(sbte, get_case, monkeypatch, tmp_path, name):
    """The sweep plan's level order built on the device (k_level_order: one
    block per direction, Kahn's waves, each wave sorted by cell index in
    shared memory; in-degrees in shared memory, or with /global in global
    memory, BTE_LEVEL_ORDER=global) is the host's (sweep_order.h,
    BTE_LEVEL_ORDER=host) entry for entry.  Directions whose upwind graph has
    a cycle are ordered on the host in both runs (they need the host's cycle
    breaking)."""
    from staticbtesolver_gb300 import synth

    base = name.split("/")[0]
    if base.startswith("cube") or base == "square100k":
        p = synth.make_problem(base, str(tmp_path))
        args = (p.geo, p.bc_file, p.band_file, p.DM, p.num_theta, p.num_phi, p.T_ref, p.L_x, p.L_y, p.L_z)
        c = None
    else:
        c = get_case(base)
        args = _odd_slab(c) if name.endswith("/odd") else c.args()
    orders, host_dirs = {}, {}
    for where in ("device", "host"):
        if where == "host":
            monkeypatch.setenv("BTE_LEVEL_ORDER", "host")
        elif name.endswith("/global"):
            monkeypatch.setenv("BTE_LEVEL_ORDER", "global")
        else:
            monkeypatch.delenv("BTE_LEVEL_ORDER", raising=False)
        if name.endswith("/cycles"):
            ctx = sbte.Context(0).set_arrays(_rewired(sbte, c, n_swaps=10))
        else:
            ctx = sbte.Context(0).load(sbte.Problem(*args))
        st, rep = ctx.solve(max_iter=2, tol=0.0, form=sbte.FORM_SWEEP)
        nd = ctx._dims[1]
        orders[where] = [ctx.level_order(d) for d in range(nd)]
        host_dirs[where] = rep.sweep_host_dirs
        ctx.close()
    assert host_dirs["host"] == nd
    if name.endswith("/cycles"):
        assert host_dirs["device"] > 0  # (here every direction's graph has a cycle)
    else:
        assert host_dirs["device"] == 0
    for d in range(nd):
        (pd, ld), (ph, lh) = orders["device"][d], orders["host"][d]
        assert np.array_equal(pd, ph), d
        assert np.array_equal(ld, lh), d
        assert np.array_equal(np.sort(pd), np.arange(len(pd)))
