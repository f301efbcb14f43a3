"""Diffusion-synthetic acceleration of the outer iteration (bte_options.dsa), on the GPU.

The correction changes how fast the source iteration reaches its fixed point,
not which fixed point: every test compares with the unaccelerated iteration
of the same form (parity-pinned to the oracle per outer iteration elsewhere)
run to a much tighter margin, or with the reference's own results.
Tolerances: relative L2 of T - T_ref <= 1e-8 against the unaccelerated
field converged to margin 1e-13 when the accelerated one stops at 1e-11 (both
FP64 sweeps; the low-order solve is FP32 but only accelerates; it also
amplifies the rounding noise of T differences, which sets a margin floor near
1e-10 on 100k-cell meshes), and <= 1e-5 at the reference's margin
1e-5 stop (the unaccelerated iteration itself is that far from its limit on
slowly converging cases).  The low-order solve itself is checked against a
SciPy direct solve of the same operator.
"""
import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _square(tmp_path, n, n_band, side, name="sq"):
    from staticbtesolver_gb300 import synth

    geo = str(tmp_path / f"{name}.mphtxt")
    synth.write_mphtxt(geo, synth.square_mesh(n))
    synth.write_band_file(str(tmp_path / f"{name}.band"), synth.debye_bands(n_band))
    synth.write_bc_file(str(tmp_path / f"{name}.bc"), [(0, 1, 301.0), (1, 2, 300.0), (2, 1, 299.0), (3, 2, 300.0)])
    return (geo, str(tmp_path / f"{name}.bc"), str(tmp_path / f"{name}.band"), 2, 8, 8, 300.0, side, side, 0.0)


def _lo_operator(oracle_mod, args):
    from oracle.dsa import coefficients, fixed_faces, read_bands, read_bc_rows

    o = oracle_mod.Oracle(*args)
    g, q = o.geometry(), o.quadrature()
    fixed = fixed_faces(g["nbr"], read_bc_rows(args[1]))
    W = coefficients(g, q, read_bands(args[2]), fixed, o.dim, 0.25).T.copy()
    nb = np.where(g["nbr"].T >= 0, g["nbr"].T, -1).astype(np.int32)
    return nb, W, g["volume"]


def _matrix(nb, W):
    import scipy.sparse as sp

    F, n = W.shape
    m = nb >= 0
    rows = np.broadcast_to(np.arange(n), (F, n))
    return (sp.csr_matrix((-W[m], (rows[m], nb[m])), shape=(n, n)) + sp.diags(W.sum(0))).tocsc()


def test_low_order_solve_matches_direct_solve(sbte, oracle_mod, tmp_path):
    import scipy.sparse.linalg as spla

    args = _square(tmp_path, 40, 8, 1e-5)
    nb, W, vol = _lo_operator(oracle_mod, args)
    A = _matrix(nb, W)
    rng = np.random.default_rng(7)
    b = vol * (rng.standard_normal(len(vol)) + 0.5)
    x_ref = spla.spsolve(A, b)
    dinv = 1.0 / np.sqrt(A.diagonal())
    # the solve stops on the preconditioned residual sqrt(r.M^-1 r), within a
    # few times the plain one; FP32 vectors: the true residual follows the
    # recurrence's down to ~1e-4 (the correction only needs ~1e-3; the outer
    # iteration is FP64)
    for tol in (1e-3, 1e-4):
        x, it, rr = sbte.dsa_solve(nb, W, b, tol=tol, maxit=5000)
        assert 0 < it < 5000 and rr <= tol
        res = np.linalg.norm(dinv * (b - A @ x)) / np.linalg.norm(dinv * b)
        assert res <= max(6 * tol, 1e-3), (tol, res)
        if tol == 1e-4:
            assert rel_l2(x, x_ref) < 1e-2
    # deterministic: a second call gives the same bits
    x2, it2, _ = sbte.dsa_solve(nb, W, b, tol=1e-4, maxit=5000)
    assert it2 == it and np.array_equal(x2, x)
    # zero right-hand side: zero correction, no iteration
    x0, it0, _ = sbte.dsa_solve(nb, W, np.zeros_like(b), tol=1e-5)
    assert it0 == 0 and not x0.any()


def test_low_order_solve_rejects_asymmetric_operator(sbte, oracle_mod, tmp_path):
    args = _square(tmp_path, 6, 2, 1e-5)
    nb, W, vol = _lo_operator(oracle_mod, args)
    W2 = W.copy()
    k = np.argwhere(nb >= 0)[0]
    W2[k[0], k[1]] *= 1.5
    with pytest.raises(sbte.BteError):
        sbte.dsa_solve(nb, W2, vol)
    nb2 = nb.copy()
    nb2[k[0], k[1]] = len(vol)  # out of range
    with pytest.raises(sbte.BteError):
        sbte.dsa_solve(nb2, W, vol)


def _run(sbte, args, **kw):
    p = sbte.Problem(*args)
    ctx = sbte.Context(0).load(p)
    st, rep = ctx.solve(**kw)
    res = ctx.result(st, rep)
    ctx.close()
    return res


@pytest.mark.parametrize("form", ["SWEEP", "PLAIN"])
def test_dsa_reaches_the_plain_fixed_point_moderately_diffusive(sbte, tmp_path, form):
    """A 1e-6 m square (Knudsen numbers 1e-3 .. 0.8): the unaccelerated source
    iteration needs ~3,000 outer iterations; with dsa a few tens, to the same field."""
    args = _square(tmp_path, 12, 8, 1e-6)
    fm = getattr(sbte, "FORM_" + form)
    ref = _run(sbte, args, max_iter=20000, tol=1e-13, form=sbte.FORM_SWEEP)
    assert ref.report["converged"] and ref.report["n_iter"] > 1500
    tight = _run(sbte, args, max_iter=200, tol=1e-11, form=fm, dsa=True, dsa_tol=1e-4)
    assert tight.report["converged"] and tight.report["n_iter"] <= 60, tight.report["n_iter"]
    assert tight.report["dsa_solves"] == tight.report["n_iter"] - 1
    assert rel_l2(tight.T - 300.0, ref.T - 300.0) < 1e-8
    std = _run(sbte, args, max_iter=200, tol=1e-5, form=fm, dsa=True)
    assert std.status == 0 and std.report["n_iter"] <= 30
    assert rel_l2(std.T - 300.0, ref.T - 300.0) < 1e-5
    big = np.abs(ref.q) > 1e-3 * np.abs(ref.q).max()
    np.testing.assert_allclose(std.q[big], ref.q[big], rtol=1e-4)


def test_dsa_on_ballistic_golden_case(sbte, get_case):
    """The reference's ballistic 2DM2DG case (specular side walls): dsa may
    help little there, but it must land on the same field."""
    c = get_case("2DM2DG")
    ref = _run(sbte, c.args(), max_iter=5000, tol=1e-13, form=sbte.FORM_SWEEP)
    res = _run(sbte, c.args(), max_iter=5000, tol=1e-11, form=sbte.FORM_SWEEP, dsa=True, dsa_tol=1e-4)
    assert res.report["converged"] and ref.report["converged"]
    assert rel_l2(res.T - 300.0, ref.T - 300.0) < 1e-8
    assert res.report["n_iter"] <= ref.report["n_iter"]
    std = _run(sbte, c.args(), max_iter=c.max_iter, tol=1e-5, form=sbte.FORM_SWEEP, dsa=True)
    assert rel_l2(std.T - 300.0, c.ref["T"] - 300.0) < 1e-5


def test_dsa_with_anderson(sbte, tmp_path):
    args = _square(tmp_path, 12, 8, 1e-6)
    ref = _run(sbte, args, max_iter=20000, tol=1e-13, form=sbte.FORM_SWEEP)
    res = _run(sbte, args, max_iter=200, tol=1e-12, form=sbte.FORM_SWEEP, dsa=True, accel=3, accel_every=4)
    assert res.report["converged"]
    assert rel_l2(res.T - 300.0, ref.T - 300.0) < 1e-7


def test_dsa_is_bitwise_reproducible(sbte, tmp_path):
    args = _square(tmp_path, 12, 8, 1e-6)
    a = _run(sbte, args, max_iter=40, tol=1e-9, form=sbte.FORM_SWEEP, dsa=True)
    b = _run(sbte, args, max_iter=40, tol=1e-9, form=sbte.FORM_SWEEP, dsa=True)
    assert np.array_equal(a.T, b.T) and np.array_equal(a.margins, b.margins)
    assert a.report["dsa_iterations"] == b.report["dsa_iterations"] > 0


def _diffusive_fixture(name="square12_b8"):
    import json
    import os

    from conftest import GOLDEN

    d = os.path.join(GOLDEN, "diffusive", name)
    meta = json.load(open(os.path.join(d, "expected.json")))
    ref = dict(np.load(os.path.join(d, "ref.npz")))
    args = (os.path.join(d, "mesh.mphtxt"), os.path.join(d, "inputbc.dat"), os.path.join(d, "band.dat"), meta["DM"],
            meta["num_theta"], meta["num_phi"], meta["T_ref"], meta["side"], meta["side"], 0.0)
    return args, meta, ref


DIFFUSIVE = ["square12_b8", "squarepores"]


@pytest.mark.parametrize("name", DIFFUSIVE)
def test_dsa_matches_oracle_fixed_point(sbte, name):
    """tests/golden/diffusive/<name>: the oracle's own outer iterations,
    interleaved with a CPU diffusion correction, reach the iteration's fixed
    point (certified by one more plain oracle step); the GPU's accelerated
    solve lands on it.  squarepores has three circular pores with diffuse
    walls: inner walls, a non-convex domain, aggregates cut by the pores."""
    args, meta, ref = _diffusive_fixture(name)
    assert ref["cert_dT"] < 1e-11
    tight = _run(sbte, args, max_iter=200, tol=1e-11, form=sbte.FORM_SWEEP, dsa=True, dsa_tol=1e-4)
    assert tight.report["converged"]
    assert rel_l2(tight.T - 300.0, ref["T_fixed"] - 300.0) < 1e-8
    big = np.abs(ref["q_fixed"]) > 1e-3 * np.abs(ref["q_fixed"]).max()
    np.testing.assert_allclose(tight.q[big], ref["q_fixed"][big], rtol=1e-7)
    std = _run(sbte, args, max_iter=200, tol=1e-5, form=sbte.FORM_SWEEP, dsa=True)
    assert std.status == 0 and std.report["n_iter"] <= 30
    assert rel_l2(std.T - 300.0, ref["T_fixed"] - 300.0) < 1e-5


@pytest.mark.parametrize("name", DIFFUSIVE)
def test_plain_iteration_matches_reference_build_on_long_run(sbte, name):
    """The same fixture run by the reference's own CPU solver: its plain
    iteration stops at margin <= 1e-5 after thousands of outer iterations,
    still ~5e-5 from the fixed point.  The GPU's unaccelerated iteration
    reproduces that run (same count, same field), and the accelerated one is
    closer to the fixed point than the reference's own answer."""
    args, meta, ref = _diffusive_fixture(name)
    if "T_refbuild" not in ref:
        pytest.skip("fixture made without the reference build")
    n_ref = int(ref["n_iter_refbuild"])
    plain = _run(sbte, args, max_iter=n_ref + 100, tol=1e-5, form=sbte.FORM_SWEEP)
    assert plain.status == 0
    assert abs(plain.report["n_iter"] - n_ref) <= 1
    assert rel_l2(plain.T - 300.0, ref["T_refbuild"] - 300.0) < 1e-6
    d_ref = rel_l2(ref["T_refbuild"] - 300.0, ref["T_fixed"] - 300.0)
    acc = _run(sbte, args, max_iter=200, tol=1e-5, form=sbte.FORM_SWEEP, dsa=True)
    assert rel_l2(acc.T - 300.0, ref["T_fixed"] - 300.0) < d_ref


@pytest.mark.parametrize("form", ["SWEEP", "PLAIN"])
def test_porous_square_first_iterations_match_oracle(sbte, form):
    """tests/golden/diffusive/squarepores: three circular pores with diffuse
    walls (inner walls, a non-convex domain).  The first five plain outer
    iterations match the oracle's (its GMRES inner solves stop at 1e-9)."""
    args, meta, ref = _diffusive_fixture("squarepores")
    res = _run(sbte, args, max_iter=5, tol=0.0, form=getattr(sbte, "FORM_" + form))
    assert res.report["n_iter"] == 5
    assert rel_l2(res.T - 300.0, ref["T_it5"] - 300.0) < 1e-7
    np.testing.assert_allclose(res.margins, ref["margins_it5"], rtol=1e-6)
    big = np.abs(ref["q_it5"]) > 1e-3 * np.abs(ref["q_it5"]).max()
    np.testing.assert_allclose(res.q[big], ref["q_it5"][big], rtol=1e-6)


def test_square100k_reaches_oracle_fixed_point(sbte, tmp_path):
    """The diffusive workload at full size (1e-4 m square, 100,352 triangles,
    20 bands x 32 directions): the reference's source iteration contracts by
    ~1.3e-5 per outer iteration there (~870,000 iterations to its stop); with
    the correction the sweep form stops at margin <= 1e-5 within 15 outer
    iterations, within 1e-6 (relative L2 of T - T_ref) of the oracle's fixed
    point (tests/golden/full/square100k.npz) and its heat fluxes within 1e-5 of
    the largest.
    The plain iteration is still ~94 % of the way from T_ref to it after 200."""
    from staticbtesolver_gb300 import synth

    fx = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "full", "square100k.npz"))
    p = synth.make_problem("square100k", str(tmp_path))
    synth.write_band_file(p.band_file, {k: fx["band_" + k] for k in ("vg", "tau", "C", "Lr")})
    args = (p.geo, p.bc_file, p.band_file, p.DM, p.num_theta, p.num_phi, p.T_ref, p.L_x, p.L_y, p.L_z)
    acc = _run(sbte, args, max_iter=100, tol=1e-5, form=sbte.FORM_SWEEP, dsa=True)
    assert acc.status == 0 and acc.report["n_iter"] <= 15
    err = rel_l2(acc.T - p.T_ref, fx["T"] - p.T_ref)
    assert err < 1e-6, err
    # (the adiabatic walls' net fluxes are near-cancellations ~3e-3 of the
    # isothermal walls': the bar is relative to the largest flux)
    np.testing.assert_allclose(acc.q, fx["q"], rtol=0, atol=1e-5 * np.abs(fx["q"]).max())
    plain = _run(sbte, args, max_iter=200, tol=1e-5, form=sbte.FORM_SWEEP)
    assert plain.status == 6  # max_iter reached
    assert rel_l2(plain.T - p.T_ref, fx["T"] - p.T_ref) > 0.5


@pytest.mark.parametrize("form", ["PLAIN", "MIXED"])
def test_square100k_krylov_forms_with_dsa(sbte, tmp_path, form):
    """The Krylov forms under the correction on the full diffusive square:
    both stop at margin <= 1e-5 within 15 outer iterations, within 1e-5 of
    the oracle's fixed point.  The correction amplifies an inner solve's
    error by up to 1 / (1 - rho) (~1e5 here), so the mixed form's inner
    solves run to 1e-11 under it (at the default 1e-9 its margins cycle
    between 1e-2 and 20 and never stop)."""
    from staticbtesolver_gb300 import synth

    fx = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "full", "square100k.npz"))
    p = synth.make_problem("square100k", str(tmp_path))
    synth.write_band_file(p.band_file, {k: fx["band_" + k] for k in ("vg", "tau", "C", "Lr")})
    args = (p.geo, p.bc_file, p.band_file, p.DM, p.num_theta, p.num_phi, p.T_ref, p.L_x, p.L_y, p.L_z)
    res = _run(sbte, args, max_iter=40, tol=1e-5, form=getattr(sbte, "FORM_" + form), dsa=True)
    assert res.status == 0 and res.report["n_iter"] <= 15, (res.status, res.report["n_iter"])
    err = rel_l2(res.T - p.T_ref, fx["T"] - p.T_ref)
    assert err < 1e-5, err
