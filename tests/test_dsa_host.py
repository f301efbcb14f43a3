"""The low-order operator of the diffusion-synthetic acceleration
(staticbtesolver_gb300/csrc/dsa_setup.h), on the CPU.

The header is plain C++; it is compiled here into a small shared library and
checked against a NumPy restatement of the same face coefficients on meshes
read by the oracle (the reference's geometry and quadrature):
  W_f = (A_f / Omega_tot) sum_b Lr_b L_b (G_f + beta L_b q_f / delta_f) / sum_b Lr_b,
G_f = 1/2 sum_d |S_d.n_f|, q_f = sum_d (S_d.n_f)(s_d.n_f), delta_f the
centroid distance across the face (dim/(dim+1) (V_c + V_nb) / A_f; a wall
face uses V_c alone).  The operator must be symmetric, hold exactly the
isothermal (and unnamed) wall faces, and have zero row sums away from them.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "staticbtesolver_gb300", "csrc", "dsa_setup.h")

SRC = r'''
#include "%s"
extern "C" int dsa_c(int dim, int n, int F, const int* nbr, const double* area, const double* normal,
                     const double* volume, int nd, const double* s, const double* S, double om, int nb,
                     const double* vg, const double* tau, const double* Lr, const char* fixed, double beta,
                     double* W, int* nbo, double* diag) {
    std::vector<char> fx(fixed, fixed + (size_t)n * F);
    bte::DsaCoefficients co;
    bte::dsa_coefficients(dim, n, F, nbr, area, normal, volume, nd, s, S, om, nb, vg, tau, Lr, fx, beta, co);
    std::copy(co.W.begin(), co.W.end(), W);
    std::copy(co.nb.begin(), co.nb.end(), nbo);
    std::copy(co.diag.begin(), co.diag.end(), diag);
    return co.n_dirichlet;
}
extern "C" void order_c(int n, int F, const int* nbr, int leaf, int* out) {
    std::vector<int> o;
    bte::locality_order(n, F, nbr, leaf, o);
    std::copy(o.begin(), o.end(), out);
}
extern "C" void hilbert_c(int dim, int n, const double* cen, int* out) {
    std::vector<int> o;
    bte::hilbert_order(dim, n, cen, o);
    std::copy(o.begin(), o.end(), out);
}
extern "C" unsigned long long hkey_c(int dim, int b, unsigned x0, unsigned x1, unsigned x2) {
    unsigned x[3] = {x0, x1, x2};
    return bte::hilbert_key(x, dim, b);
}
extern "C" int coarse_c(int n, int F, const int* nb, const double* w, int nblk, int per, double* ac, int* geo,
                        int* need_ptr, int* need) {
    bte::DsaCoarse co;
    bte::dsa_coarse(n, F, nb, w, nblk, per, co);
    std::copy(co.ac.begin(), co.ac.end(), ac);
    geo[0] = co.chunk; geo[1] = co.seg;
    std::copy(co.need_ptr.begin(), co.need_ptr.end(), need_ptr);
    std::copy(co.need.begin(), co.need.end(), need);
    return co.n_agg;
}
'''


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    d = tmp_path_factory.mktemp("dsa_setup")
    src = d / "dsa.cpp"
    src.write_text(SRC % HEADER)
    out = d / "libdsa.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", str(out), str(src)], check=True)
    L = C.CDLL(str(out))
    L.dsa_c.restype = C.c_int
    L.hkey_c.restype = C.c_ulonglong
    L.hkey_c.argtypes = [C.c_int, C.c_int, C.c_uint, C.c_uint, C.c_uint]
    return L


from oracle.dsa import coefficients, fixed_faces, read_bands as bands_of, read_bc_rows as bc_rows  # noqa: E402


def restated(g, q, bands, fixed, dim, beta):
    return coefficients(g, q, bands, fixed, dim, beta)


def run(lib, o, bands, rows, beta=0.25):
    g, q = o.geometry(), o.quadrature()
    n, F = g["nbr"].shape
    fixed = fixed_faces(g["nbr"], rows)
    W, nbo, diag = np.zeros(F * n), np.zeros(F * n, np.int32), np.zeros(n)
    f64 = lambda a: np.ascontiguousarray(a, np.float64).ctypes.data_as(C.c_void_p)
    nbr = np.ascontiguousarray(g["nbr"], np.int32)
    fx = np.ascontiguousarray(fixed, np.int8)
    nd = lib.dsa_c(o.dim, n, F, nbr.ctypes.data_as(C.c_void_p), f64(g["area"]), f64(g["normal"]), f64(g["volume"]),
                   o.n_dir, f64(q["s"]), f64(q["S"]), C.c_double(q["solid_angle"]), len(bands["vg"]),
                   f64(bands["vg"]), f64(bands["tau"]), f64(bands["Lr"]), fx.ctypes.data_as(C.c_void_p),
                   C.c_double(beta), W.ctypes.data_as(C.c_void_p), nbo.ctypes.data_as(C.c_void_p),
                   diag.ctypes.data_as(C.c_void_p))
    return g, q, fixed, W.reshape(F, n), nbo.reshape(F, n), diag, nd


@pytest.mark.parametrize("name", ["square10_b40", "2DM2DG", "cube4_b2"])
def test_coefficients_match_restatement(lib, oracle_mod, get_case, name):
    case = get_case(name)
    o = oracle_mod.Oracle(*case.args())
    bands, rows = bands_of(case.band), bc_rows(case.bc)
    for beta in (0.0, 0.25):
        g, q, fixed, W, nbo, diag, nd = run(lib, o, bands, rows, beta)
        ref = restated(g, q, bands, fixed, o.dim, beta).T  # [F][n]
        np.testing.assert_allclose(W, ref, rtol=1e-12, atol=0)
        assert nd == int(fixed.sum())
        # couplings only through interior faces, to the face's neighbour
        nbr = g["nbr"].T
        assert np.array_equal(nbo, np.where(nbr >= 0, nbr, -1))
        np.testing.assert_allclose(diag, W.sum(0), rtol=1e-14)


@pytest.mark.parametrize("name", ["square10_b40", "cube4_b2"])
def test_operator_is_symmetric_and_conservative(lib, oracle_mod, get_case, name):
    import scipy.sparse as sp

    case = get_case(name)
    o = oracle_mod.Oracle(*case.args())
    g, q, fixed, W, nbo, diag, nd = run(lib, o, bands_of(case.band), bc_rows(case.bc))
    F, n = W.shape
    m = nbo >= 0
    cols = np.where(m, nbo, 0)
    rows = np.broadcast_to(np.arange(n), (F, n))
    A = sp.csr_matrix((-W[m], (rows[m], cols[m])), shape=(n, n)) + sp.diags(diag)
    assert abs(A - A.T).max() == 0.0  # each face evaluated once, stored on both sides
    # zero row sums except in cells with a fixed-temperature wall face
    walls = (np.where(nbo < 0, W, 0.0)).sum(0)
    np.testing.assert_allclose(np.asarray(A.sum(1)).ravel(), walls, atol=1e-12 * diag.max())
    assert nd > 0 and (walls > 0).sum() > 0
    # positive definite with at least one wall held fixed
    ev = np.linalg.eigvalsh(A.toarray()) if n <= 2000 else None
    if ev is not None:
        assert ev.min() > 0


def test_adiabatic_walls_carry_no_term(lib, oracle_mod, get_case):
    """Diffuse (2) and specular (31) walls are adiabatic: no wall coefficient."""
    case = get_case("2DM2DG")
    o = oracle_mod.Oracle(*case.args())
    rows = bc_rows(case.bc)
    g, q, fixed, W, nbo, diag, nd = run(lib, o, bands_of(case.band), rows)
    nbr = g["nbr"].T
    types = {-e - 1: t for e, t, _ in rows}
    for code, t in types.items():
        sel = nbr == code
        if t == 1:
            assert (W[sel] > 0).all()
        else:
            assert (W[sel] == 0).all()


def _scaled_permuted(lib, o, case, nblk, per):
    """The low-order operator scaled to unit diagonal in the locality order, as the solve holds it."""
    g, q, fixed, W, nbo, diag, nd = run(lib, o, bands_of(case.band), bc_rows(case.bc))
    F, n = W.shape
    cm = np.ascontiguousarray(np.where((nbo >= 0) & (W > 0), nbo, -1).T, np.int32)  # [n][F]
    order = np.zeros(n, np.int32)
    lib.order_c(n, F, cm.ctypes.data_as(C.c_void_p), max(8, n // (nblk * per) // 2), order.ctypes.data_as(C.c_void_p))
    pos = np.argsort(order)
    dsc = 1.0 / np.sqrt(diag)
    nbp = np.full((F, n), -1, np.int32)
    wp = np.zeros((F, n))
    for f in range(F):
        c = order
        m = nbo[f, c] >= 0
        nbp[f, m] = pos[nbo[f, c][m]]
        wp[f, m] = W[f, c][m] * dsc[c][m] * dsc[nbo[f, c][m]]
    return order, pos, nbp, wp


@pytest.mark.parametrize("name", ["square16_b8", "cube4_b2"])
def test_locality_order_and_coarse_operator(lib, oracle_mod, get_case, name):
    import scipy.sparse as sp

    case = get_case(name)
    o = oracle_mod.Oracle(*case.args())
    nblk, per = 8, 4
    order, pos, nbp, wp = _scaled_permuted(lib, o, case, nblk, per)
    F, n = wp.shape
    assert np.array_equal(np.sort(order), np.arange(n))
    m = nblk * per
    ac = np.zeros(m * m)
    geo = np.zeros(2, np.int32)
    need_ptr = np.zeros(nblk + 1, np.int32)
    need = np.zeros(m * nblk, np.int32)
    f64p = lambda a: np.ascontiguousarray(a).ctypes.data_as(C.c_void_p)
    got = lib.coarse_c(n, F, f64p(nbp), f64p(wp), nblk, per, ac.ctypes.data_as(C.c_void_p),
                       geo.ctypes.data_as(C.c_void_p), need_ptr.ctypes.data_as(C.c_void_p),
                       need.ctypes.data_as(C.c_void_p))
    assert got == m
    chunk, seg = int(geo[0]), int(geo[1])
    agg = (np.arange(n) // chunk) * per + (np.arange(n) - (np.arange(n) // chunk) * chunk) // seg
    rows = np.broadcast_to(np.arange(n), (F, n))
    msk = nbp >= 0
    A = (sp.csr_matrix((-wp[msk], (rows[msk], nbp[msk])), shape=(n, n)) + sp.eye(n)).toarray()
    P = np.zeros((n, m))
    P[np.arange(n), agg] = 1.0
    Ac = P.T @ A @ P
    empty = P.sum(0) == 0
    Ac[empty, empty] = 1.0
    np.testing.assert_allclose(ac.reshape(m, m), Ac, rtol=0, atol=1e-12)
    # the device inverts it by Gauss-Jordan steps without pivoting (k_gj_step):
    # the same steps in NumPy reach the inverse of this positive definite matrix
    G = ac.reshape(m, m).copy()
    for k in range(m):
        rp = 1.0 / G[k, k]
        col, row = G[:, k].copy(), G[k, :].copy()
        G = G - np.outer(col, row * rp)
        G[k, :] = row * rp
        G[:, k] = -col * rp
        G[k, k] = rp
    np.testing.assert_allclose(G @ Ac, np.eye(m), atol=1e-9)
    # every block's list holds the aggregates of its cells and of their neighbours
    for k in range(nblk):
        lst = set(need[need_ptr[k]:need_ptr[k + 1]].tolist())
        cells = np.arange(k * chunk, min(n, (k + 1) * chunk))
        want = set(agg[cells].tolist()) | set(agg[nbp[:, cells][nbp[:, cells] >= 0]].tolist())
        assert lst == want
    # compact aggregates: many couplings stay inside an aggregate
    inside = (agg[rows[msk]] == agg[nbp[msk]]).mean()
    assert inside > 0.4, inside  # a random numbering keeps ~1/32 inside


def _hilbert_keys(q, b):
    """NumPy restatement of the transpose algorithm (J. Skilling, AIP Conf.
    Proc. 707 (2004) 381) for integer points q [n][dim] < 2^b."""
    x = [q[:, i].astype(np.uint64) for i in range(q.shape[1])]
    dim = len(x)
    Q = 1 << (b - 1)
    while Q > 1:
        low = np.uint64(Q - 1)
        for i in range(dim):
            hit = (x[i] & np.uint64(Q)) != 0
            t = (x[0] ^ x[i]) & low
            x0 = np.where(hit, x[0] ^ low, x[0] ^ t)
            if i > 0:
                x[i] = np.where(hit, x[i], x[i] ^ t)
            x[0] = x0
        Q >>= 1
    for i in range(1, dim):
        x[i] = x[i] ^ x[i - 1]
    t = np.zeros_like(x[0])
    Q = 1 << (b - 1)
    while Q > 1:
        t = np.where((x[dim - 1] & np.uint64(Q)) != 0, t ^ np.uint64(Q - 1), t)
        Q >>= 1
    x = [xi ^ t for xi in x]
    key = np.zeros_like(x[0])
    for q_ in range(b - 1, -1, -1):
        for i in range(dim):
            key = (key << np.uint64(1)) | ((x[i] >> np.uint64(q_)) & np.uint64(1))
    return key


@pytest.mark.parametrize("dim,b", [(2, 4), (3, 3)])
def test_hilbert_key_walks_grid_neighbours(lib, dim, b):
    """Sorted by key, the cells of a 2^b grid form a path of unit steps that
    visits every cell once (the defining property of the curve)."""
    side = 1 << b
    pts = np.stack(np.meshgrid(*[np.arange(side)] * dim, indexing="ij"), -1).reshape(-1, dim)
    keys = np.array([lib.hkey_c(dim, b, *(list(map(int, p)) + [0] * (3 - dim))) for p in pts], np.uint64)
    assert np.array_equal(np.sort(keys), np.arange(side ** dim, dtype=np.uint64))
    path = pts[np.argsort(keys)]
    assert (np.abs(np.diff(path, axis=0)).sum(1) == 1).all()
    np.testing.assert_array_equal(_hilbert_keys(pts, b), keys)


@pytest.mark.parametrize("dim", [2, 3])
def test_hilbert_order_matches_restatement(lib, dim):
    """hilbert_order on 70,000 random centroids (host threads and radix
    passes) equals a stable sort of the restated keys, ties by cell index."""
    rng = np.random.default_rng(dim)
    n = 70000
    cen = np.zeros((n, 3))
    cen[:, :dim] = rng.uniform(-1e-6, 3e-6, (n, dim))
    cen[:, 0] *= 0.5  # a box longer in y: one scale for every axis
    cen[100:200] = cen[5000]  # ties
    out = np.zeros(n, np.int32)
    lib.hilbert_c(dim, n, cen.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p))
    b = 21
    lo = cen[:, :dim].min(0)
    ext = (cen[:, :dim].max(0) - lo).max()
    steps = float(1 << b)
    q = np.minimum(np.maximum((cen[:, :dim] - lo) * (steps / ext), 0.0), steps - 1).astype(np.uint64)
    want = np.argsort(_hilbert_keys(q, b), kind="stable")
    np.testing.assert_array_equal(out, want)


def test_coarse_operator_on_host_threads(lib):
    """dsa_coarse on a 30,000-cell operator (above the size it forms on host
    threads): the coarse matrix P^T A P and every block's need list equal a
    serial NumPy restatement."""
    rng = np.random.default_rng(5)
    n, F, nblk, per = 30000, 3, 16, 4
    nb = np.full((F, n), -1, np.int32)
    w = np.zeros((F, n))
    for f, off in enumerate((1, 97, 5003)):
        has = rng.random(n) < 0.9
        nb[f, has] = (np.arange(n)[has] + off) % n
        w[f, has] = rng.uniform(0.1, 1.0, has.sum())
    m = nblk * per
    ac = np.zeros(m * m)
    geo = np.zeros(2, np.int32)
    need_ptr = np.zeros(nblk + 1, np.int32)
    need = np.zeros(m * nblk, np.int32)
    ptr = lambda a: np.ascontiguousarray(a).ctypes.data_as(C.c_void_p)
    got = lib.coarse_c(n, F, ptr(nb), ptr(w), nblk, per, ac.ctypes.data_as(C.c_void_p), geo.ctypes.data_as(C.c_void_p),
                       need_ptr.ctypes.data_as(C.c_void_p), need.ctypes.data_as(C.c_void_p))
    assert got == m
    chunk, seg = int(geo[0]), int(geo[1])
    k = np.arange(n) // chunk
    agg = k * per + (np.arange(n) - k * chunk) // seg
    want = np.zeros((m, m))
    for c in range(n):
        J = agg[c]
        want[J, J] += 1.0
        for f in range(F):
            if nb[f, c] >= 0:
                want[J, agg[nb[f, c]]] -= w[f, c]
    np.testing.assert_array_equal(ac.reshape(m, m), want)
    for b in range(nblk):
        cells = np.arange(b * chunk, min(n, (b + 1) * chunk))
        lst = sorted(set(agg[cells].tolist()) | set(agg[nb[:, cells][nb[:, cells] >= 0]].tolist()))
        assert need[need_ptr[b]:need_ptr[b + 1]].tolist() == lst
