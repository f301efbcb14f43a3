"""Kernel-level parity: the C-ABI BiCGSTAB on one CSR system (the reference's
BICGSTAB boundary, src/bicgstab.hpp:65,96,138) against the oracle's restatement."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,band,direction", [("2DM2DG", 0, 5), ("3DM3DG", 0, 77), ("square10_b40", 39, 3),
                                                 ("cube4_b2", 1, 100), ("2DM1DG", 0, 2)])
def test_csr_bicgstab_matches_oracle(sbte, oracle_mod, get_case, name, band, direction):
    c = get_case(name)
    o = oracle_mod.Oracle(*c.args())
    rng = np.random.default_rng(1)
    e_prev = rng.uniform(0, 1e4, size=(o.n_band, o.n_dir, o.n_cell))
    ebar = rng.uniform(0, 1e4, size=(o.n_cell, o.n_band))
    rp, ci, v, b = o.assemble(band, direction, e_prev, ebar)
    xo, ito, co = oracle_mod.bicgstab_csr(rp, ci, v, b, 1000, 1e-9)
    xg, itg, cg = sbte.bicgstab_csr(rp, ci, v, b, 1000, 1e-9)
    assert cg == co
    if o.dim > 1:
        assert abs(itg - ito) <= 1
        assert np.linalg.norm(xg - xo) <= 1e-9 * np.linalg.norm(xo)
    else:
        # single-entry right-hand side: rounding-dependent BiCGSTAB paths (see test_gpu_parity)
        assert abs(itg - ito) <= 0.1 * ito
        assert np.linalg.norm(xg - xo) <= 1e-6 * np.linalg.norm(xo)
    # residual of the GPU answer, checked with the oracle's matrix
    A = np.zeros((o.n_cell, o.n_cell))
    for r in range(o.n_cell):
        A[r, ci[rp[r]:rp[r + 1]]] = v[rp[r]:rp[r + 1]]
    assert np.linalg.norm(b - A @ xg) <= 2e-9 * np.linalg.norm(b)


def test_csr_zero_rhs_and_multi_chunk_bidiagonal(sbte, oracle_mod):
    n = 3000  # three 1024-cell chunks: exercises the cross-block dot products
    rng = np.random.default_rng(4)
    rows, cols, vals = [], [], []
    for r in range(n):
        if r > 0:
            rows.append(r); cols.append(r - 1); vals.append(-rng.uniform(0.2, 0.9))
        rows.append(r); cols.append(r); vals.append(rng.uniform(1.0, 2.0))
    rp = np.searchsorted(np.array(rows), np.arange(n + 1)).astype(np.int32)
    ci, v = np.array(cols, np.int32), np.array(vals)
    x, it, conv = sbte.bicgstab_csr(rp, ci, v, np.zeros(n))
    assert conv and it == 0 and not x.any()
    b = rng.uniform(-1, 1, n)
    xg, itg, cg = sbte.bicgstab_csr(rp, ci, v, b)
    xo, ito, co = oracle_mod.bicgstab_csr(rp, ci, v, b)
    assert cg and co and abs(itg - ito) <= 1
    assert np.linalg.norm(xg - xo) <= 1e-9 * np.linalg.norm(xo)


def test_csr_maxit_reports_unconverged(sbte, oracle_mod, get_case):
    c = get_case("2DM2DG")
    o = oracle_mod.Oracle(*c.args())
    e_prev = np.ones((o.n_band, o.n_dir, o.n_cell))
    rp, ci, v, b = o.assemble(0, 3, e_prev, np.ones((o.n_cell, o.n_band)))
    x, it, conv = sbte.bicgstab_csr(rp, ci, v, b, maxit=1, tol=1e-14)
    assert not conv and it == 1


@pytest.mark.parametrize("name,form_name,kw", [("square16_b8", "FORM_PLAIN", {}), ("square16_b8", "FORM_MIXED", {}),
                                               ("3DM2DG", "FORM_PLAIN", {}), ("cube4_b2", "FORM_MIXED", {}),
                                               ("square10_b40", "FORM_PLAIN", {"plain_cycles": 3, "inner_maxit": 40})])
def test_persistent_bicgstab_matches_phase_kernels(sbte, get_case, monkeypatch, name, form_name, kw):
    """The Krylov forms' BiCGSTAB as one persistent launch per batch
    (BTE_KRYLOV=persistent: one block per system, the phase bodies chunk by
    chunk) and as one launch per phase (the default: the host checking every 8
    iterations) give the same x to the bit: the same temperatures, margins and
    inner iteration counts, in FP64 (PLAIN, also with the best-iterate limit of
    plain_cycles) and FP32 (MIXED)."""
    c = get_case(name)
    runs = {}
    for mode in ("persistent", "phase"):
        if mode == "persistent":
            monkeypatch.setenv("BTE_KRYLOV", "persistent")
        else:
            monkeypatch.delenv("BTE_KRYLOV", raising=False)
        ctx = sbte.Context(0).load(sbte.Problem(*c.args()))
        st, rep = ctx.solve(max_iter=c.max_iter, tol=1e-5, form=getattr(sbte, form_name), profile=True, **kw)
        runs[mode] = (st, ctx.temperature(), ctx.margins(), rep.as_dict(), ctx.kernel_stats())
        ctx.close()
    (s0, T0, m0, r0, k0), (s1, T1, m1, r1, k1) = runs["persistent"], runs["phase"]
    assert s0 == s1
    assert k0["bicg_persistent"]["launches"] > 0 and k0["bicg_p_update"]["launches"] == 0
    assert k1["bicg_persistent"]["launches"] == 0 and k1["bicg_p_update"]["launches"] > 0
    assert r0["inner_iterations"] == r1["inner_iterations"] and r0["inner_unconverged"] == r1["inner_unconverged"]
    assert np.array_equal(T0, T1)
    assert np.array_equal(m0, m1)
