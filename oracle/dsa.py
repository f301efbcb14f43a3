"""Diffusion-corrected fixed points of the restated source iteration (TEST INFRASTRUCTURE ONLY).

The reference's source iteration (src/StaticBTESolver.cpp:690-808, restated in
oracle/bte_oracle.cpp) converges geometrically; in the diffusive regime its
error shrinks by ~1e-6 per outer iteration, so the oracle cannot reach its
fixed point by iterating.  ``fixed_point`` reaches the same fixed point by
interleaving the oracle's own outer iterations (``Oracle.step``: GMRES(30) +
ILU(0) per system, exactly the restated reference) with a low-order diffusion
correction solved by SciPy on the CPU.  The fixed point is unique and every
correction vanishes there, so the result is the reference iteration's limit;
``certify`` checks it by one more uncorrected oracle step.

``operator`` restates the low-order face coefficients of
staticbtesolver_gb300/csrc/dsa_setup.h in NumPy (the CPU tests compare the two).
Nothing in the product imports this module.
"""
from __future__ import annotations

import numpy as np


def read_bands(path):
    a = np.atleast_2d(np.loadtxt(path))
    return dict(vg=a[:, 0], tau=a[:, 1], C=a[:, 2], Lr=a[:, 3])


def read_bc_rows(path):
    """(entity, type, T) rows of a boundary-condition file (src/BTEBoundaryCondition.cpp:7-23)."""
    rows = []
    for line in open(path).read().splitlines()[1:]:
        parts = line.split()
        if len(parts) >= 3 and not line.lstrip().startswith("#"):
            rows.append((int(parts[0]), int(parts[1]), float(parts[2])))
    return rows


def fixed_faces(nbr, rows):
    """Wall faces held at a fixed temperature: isothermal rows and boundary codes no row names."""
    named = {-e - 1: t for e, t, _ in rows}
    return np.array([[x < 0 and named.get(int(x), 1) == 1 for x in r] for r in nbr])


def coefficients(g, q, bands, fixed, dim, beta=0.25):
    """W[c][f] of the low-order operator:
    W_f = (A_f / Omega_tot) sum_b Lr_b L_b (G_f + beta L_b q_f / delta_f) / sum_b Lr_b."""
    nbr, area, normal, vol = g["nbr"], g["area"], g["normal"], g["volume"]
    s, S, om = q["s"], q["S"], q["solid_angle"]
    G = S if dim > 1 else s
    w = bands["Lr"] / bands["Lr"].sum()
    lam = bands["vg"] * bands["tau"]
    a1, a2 = np.sum(w * lam), np.sum(w * lam * lam)
    gn = np.einsum("dk,cfk->cfd", G, normal)
    sn = np.einsum("dk,cfk->cfd", s, normal)
    gabs = 0.5 * np.abs(gn).sum(-1)
    qq = (gn * sn).sum(-1)
    h = dim / (dim + 1.0)
    nbc = np.where(nbr >= 0, nbr, 0)
    delta = np.where(nbr >= 0, h * (vol[:, None] + vol[nbc]) / area, h * vol[:, None] / area)
    coef = area / om * (gabs * a1 + beta * a2 * qq / delta)
    return np.where((nbr >= 0) | fixed, coef, 0.0)


def operator(g, q, bands, fixed, dim, beta=0.25):
    """The low-order operator as a SciPy CSC matrix (symmetrised the way
    dsa_setup.h stores each interior face once on both sides)."""
    import scipy.sparse as sp

    W = coefficients(g, q, bands, fixed, dim, beta)
    nbr = g["nbr"]
    n, F = nbr.shape
    rows = np.repeat(np.arange(n), F)
    m = (nbr >= 0).ravel()
    A = sp.csr_matrix((-W.ravel()[m], (rows[m], nbr.ravel()[m])), shape=(n, n))
    A = 0.5 * (A + A.T)
    diag = -np.asarray(A.sum(1)).ravel() + np.where(nbr < 0, W, 0.0).sum(1)
    return (A + sp.diags(diag)).tocsc()


def fixed_point(o, band_file, bc_file, tol=1e-13, max_iter=200, beta=0.25, threads=0, inner_tol=1e-12, log=None,
                stall=8, stall_tol=1e-8):
    """Run the oracle's outer iteration with a diffusion correction after every
    step until the margin (the reference's, between consecutive transport
    iterates) is <= tol.  Returns (T, e, margins); T and e are the transport
    iterate's (no correction applied to them).  On large meshes the
    correction amplifies the rounding noise of successive temperatures and the
    margin levels off (near 1e-10 at 1e5 cells): once it is <= stall_tol and
    has not reached a new low for `stall` iterations, the iterate with the
    smallest margin is returned."""
    import scipy.sparse.linalg as spla

    g, q = o.geometry(), o.quadrature()
    bands = read_bands(band_file)
    fixed = fixed_faces(g["nbr"], read_bc_rows(bc_file))
    lu = spla.splu(operator(g, q, bands, fixed, o.dim, beta))
    vol = g["volume"]
    shift = bands["C"] / q["solid_angle"]
    bcells = np.flatnonzero((g["nbr"] < 0).any(1))
    T_ref = q["T_ref"]
    e = np.zeros((o.n_band, o.n_dir, o.n_cell))
    T = np.full(o.n_cell, T_ref)
    margins = []
    best = (np.inf, -1, None, None)
    for k in range(max_iter):
        e_new, Th, m = o.step(e, T, threads=threads, inner_tol=inner_tol)
        margins.append(m)
        if log:
            log(k, m)
        if m <= tol:
            return Th, e_new, np.array(margins)
        if m < best[0]:
            best = (m, k, Th.copy(), e_new.copy())
        elif best[0] <= stall_tol and k - best[1] >= stall:
            return best[2], best[3], np.array(margins[: best[1] + 1])
        x = lu.solve(vol * (Th - T))
        T = Th + x
        e = e_new
        e[:, :, bcells] += shift[:, None, None] * x[bcells][None, None, :]
    raise RuntimeError(f"no fixed point within {max_iter} corrected iterations (last margin {margins[-1]:.3e})")


def certify(o, e, T, threads=0, inner_tol=1e-12):
    """One uncorrected oracle step from a converged state: returns
    (margin, relative change of T - T_ref) -- both at rounding level for a fixed point."""
    T_ref = o.quadrature()["T_ref"]
    _, T1, m = o.step(e, T, threads=threads, inner_tol=inner_tol, want_energy=False)
    return m, float(np.linalg.norm(T1 - T) / np.linalg.norm(T - T_ref))
