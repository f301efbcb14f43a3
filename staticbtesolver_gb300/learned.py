"""Learned acceleration of the outer source iteration.

The source iteration (src/StaticBTESolver.cpp:707-804) converges
geometrically and slowly when the dominant bands are diffusive.  A small
per-cell MLP (the kernels live in csrc/bte_mlp.cuh) looks at a cell's last
four outer temperatures and its geometry and predicts the converged
equilibrium temperature; every few iterations the solver jumps there and the
plain iteration continues to the same margin.  This module

* computes the features exactly as the device kernel k_accel_features does
  (the network learns a correction to each cell's Aitken estimate),
* generates training data from the solver's own iterate histories on seeded
  synthetic problems (bte_options.keep_history),
* trains the network with the project's GPU kernels (bte_mlp_train), and
* loads / saves the trained parameters (data/mlp_accel.npy).
"""
from __future__ import annotations

import ctypes as C
import os
import tempfile

import numpy as np

from . import synth

NPARAM = 34305
CLIP = 64.0
CORR = 8.0  # the learned correction is clipped to +-CORR (as in k_accel_apply)
EVERY = 6  # outer iterations between extrapolations used with the committed weights
DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
WEIGHTS = os.path.join(DATA, "mlp_accel.npy")


def init_params(seed: int = 0) -> np.ndarray:
    """He-initialised weights, zero biases, in the flat layout of include/bte_cuda.h."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM, np.float32)
    o = 0
    for fan_in, fan_out in ((8, 128), (128, 128), (128, 128), (128, 1)):
        n = fan_in * fan_out
        p[o:o + n] = rng.normal(0, np.sqrt(2.0 / fan_in), n).astype(np.float32)
        o += n + fan_out  # skip the bias block
    return p


def feature_geometry(arrays: dict) -> dict:
    """Per-problem constants of the features (as bte_solve computes them)."""
    cen, V = arrays["centroid"], arrays["volume"]
    b, c = arrays["bands"], arrays["bcs"]
    lr = np.asarray(b["Lr"], float)
    kn_num = float(np.sum(lr * np.asarray(b["vg"]) * np.asarray(b["tau"])) / np.sum(lr))
    dT = float(np.max(np.abs(np.asarray(c["T"], float) - arrays["T_ref"]))) if len(c["T"]) else 0.0
    span = lambda a: (a.min(), a.max() - a.min())
    (xmin, xs), (ymin, ys) = span(cen[:, 0]), span(cen[:, 1])
    return dict(vmean=V.mean(), xmin=xmin, xspan=xs, ymin=ymin, yspan=ys, kn_num=kn_num, inv_dim=1.0 / arrays["dim"],
                T_ref=arrays["T_ref"], dT=dT if dT > 0 else 1.0, centroid=cen, volume=V)


def aitken_norm(d1, d2, s):
    """Per-cell Aitken estimate of the remaining change in units of s (as aitken_norm in bte_mlp.cuh)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(d2 != 0.0, d1 / np.where(d2 != 0.0, d2, 1.0), 0.0)
        ok = (r > 0.0) & (r < 1.0)
        a = np.where(ok, d1 * r / np.where(ok, 1.0 - r, 1.0) / s, 0.0)
    return np.clip(a, -CLIP, CLIP)


def features(t0, t1, t2, t3, fg: dict):
    """Features [n][8] (float32), scale s [n] and Aitken estimate A [n] from T_k .. T_{k-3}."""
    d1, d2, d3 = t0 - t1, t1 - t2, t2 - t3
    s = np.abs(d1) + np.abs(d2) + np.abs(d3) + 1e-300
    A = aitken_norm(d1, d2, s)
    cen, V = fg["centroid"], fg["volume"]
    f = np.empty((len(t0), 8))
    f[:, 0], f[:, 1], f[:, 2] = d1 / s, d2 / s, d3 / s
    f[:, 3] = A / CLIP
    f[:, 4] = (cen[:, 0] - fg["xmin"]) / fg["xspan"] if fg["xspan"] > 0 else 0.0
    f[:, 5] = (cen[:, 1] - fg["ymin"]) / fg["yspan"] if fg["yspan"] > 0 else 0.0
    f[:, 6] = np.log(V / fg["vmean"])
    f[:, 7] = np.log10(fg["kn_num"] / V ** fg["inv_dim"])
    return f.astype(np.float32), s, A


def jump_rows(margins, every: int = EVERY, tol: float = 1e-5):
    """Outer iterations at which bte_solve extrapolated, and those after which it
    restored the state before a jump (its rule, replayed from the margins): from
    iteration 3 on, every `every` iterations; `every`-1 iterations after a jump
    the jump is undone, and extrapolation stops, unless the margin is below the
    margin at the jump.
    Returns (jumps, reverts): rows after which the field changed discontinuously."""
    on, last, m_at, jumps, reverts = True, -1, 0.0, [], []
    for it, m in enumerate(margins):
        if not np.isfinite(m) or m <= tol:
            break
        if on and last >= 0 and it == last + every - 1 and not (m < m_at):
            on = False
            reverts.append(it)
        if on and it >= 3 and (last < 0 or it - last >= every):
            jumps.append(it)
            last, m_at = it, m
    return jumps, reverts


def samples_from_history(hist: np.ndarray, fg: dict, every: int = 2, rng=None, max_rows: int = 0, jumps=()):
    """(X, Y) pairs from one solve's temperature history (rows = outer iterations).

    Target: the correction to the Aitken estimate, clip(clip((T* - T_k) / s, +-64) - A, +-8),
    with T* = the last (converged) row.  Row j of a run that extrapolated (or restored
    its state) after iteration j is followed by a discontinuity, so windows
    T_{k-3} .. T_k with such a j in [k-3, k-1] are skipped."""
    T_star = hist[-1]
    jset = set(int(j) for j in jumps)
    X, Y = [], []
    for k in range(3, len(hist) - 1, every):
        if any(j in jset for j in range(k - 3, k)):
            continue
        f, s, A = features(hist[k], hist[k - 1], hist[k - 2], hist[k - 3], fg)
        y = np.clip(np.clip((T_star - hist[k]) / s, -CLIP, CLIP) - A, -CORR, CORR).astype(np.float32)
        X.append(f)
        Y.append(y)
    if not X:
        return np.zeros((0, 8), np.float32), np.zeros(0, np.float32)
    X, Y = np.concatenate(X), np.concatenate(Y)
    if max_rows and len(Y) > max_rows:
        rng = rng or np.random.default_rng(0)
        sel = rng.choice(len(Y), max_rows, replace=False)
        X, Y = X[sel], Y[sel]
    return X, Y


def mirrored(X, Y):
    """The same samples with T reflected about T_ref: the difference features and the
    Aitken feature change sign and so does the target (doubles the data, makes the fit odd)."""
    Xm = X.copy()
    Xm[:, :4] *= -1.0
    return np.concatenate([X, Xm]), np.concatenate([Y, -Y])


def training_problems(n: int, seed: int = 7, cell_range=(40, 101)):
    """Seeded 2D problems around the 1e-7 m square: size, bands, walls and wall
    temperatures vary (side log-uniform in [3e-8, 3e-7] m, 40-100 cells per side,
    20 or 40 bands, diffuse or specular side walls, 0.5-5 K between the ends)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        side = float(np.exp(rng.uniform(np.log(3e-8), np.log(3e-7))))
        cells = int(rng.integers(*cell_range))
        bands = int(rng.choice([20, 40]))
        wall = int(rng.choice([2, 31]))
        dT = float(rng.uniform(0.5, 5.0))
        out.append(dict(side=side, cells=cells, bands=bands, wall=wall, dT=dT, seed=int(rng.integers(1 << 30))))
    return out


def write_problem(spec: dict, out_dir: str) -> synth.Problem:
    os.makedirs(out_dir, exist_ok=True)
    geo = os.path.join(out_dir, "mesh.mphtxt")
    band = os.path.join(out_dir, "band.dat")
    bc = os.path.join(out_dir, "bc.dat")
    synth.write_mphtxt(geo, synth.square_mesh(spec["cells"], seed=spec["seed"]))
    synth.write_band_file(band, synth.debye_bands(spec["bands"]))
    half = spec["dT"] / 2
    synth.write_bc_file(bc, [(0, 1, 300.0 + half), (1, spec["wall"], 300.0), (2, 1, 300.0 - half),
                             (3, spec["wall"], 300.0)])
    return synth.Problem("train", geo, band, bc, 2, 8, 8, 300.0, 20000, spec["side"], spec["side"], 0.0)


def generate(specs, max_rows_per_problem: int = 40000, device: int = 0, seed: int = 0, accel: int = 0,
             params=None, accel_every: int = EVERY):
    """Run each problem with the sweep form keeping the T history; return X, Y, info.
    accel = 2 (Aitken) or 1 (learned, `params`) records the trajectories the
    accelerator itself produces, so the network is trained on the states it meets."""
    import staticbtesolver_gb300 as S

    rng = np.random.default_rng(seed)
    Xs, Ys, info = [], [], []
    with tempfile.TemporaryDirectory() as tmp:
        for i, spec in enumerate(specs):
            p = write_problem(spec, os.path.join(tmp, str(i)))
            prob = S.Problem(p.geo, p.bc_file, p.band_file, p.DM, p.num_theta, p.num_phi, p.T_ref, p.L_x, p.L_y, p.L_z)
            ctx = S.Context(device).load(prob)
            if accel == 1:
                ctx.set_mlp(params)
            st, rep = ctx.solve(max_iter=p.max_iter, tol=1e-5, form=S.FORM_SWEEP, keep_history=True, accel=accel,
                                accel_every=accel_every)
            hist = ctx.history()
            jumps, reverts = jump_rows(ctx.margins(), accel_every) if accel else ([], [])
            ctx.close()
            assert (len(jumps), len(reverts)) == (rep.accel_steps, rep.accel_reverts), (jumps, reverts, rep.as_dict())
            X, Y = samples_from_history(hist, feature_geometry(prob.arrays()), rng=rng, max_rows=max_rows_per_problem,
                                        jumps=jumps + reverts)
            Xs.append(X)
            Ys.append(Y)
            info.append(dict(spec, n_iter=rep.n_iter, accel=accel, jumps=rep.accel_steps, reverts=rep.accel_reverts))
    return np.concatenate(Xs), np.concatenate(Ys), info


def train(X, Y, steps=3000, batch=4096, lr=1e-3, seed=0, params=None):
    """Adam on the GPU with the project's kernels (bte_mlp_train)."""
    import staticbtesolver_gb300 as S

    L, _ = S._load()
    p = init_params(seed) if params is None else np.array(params, np.float32)
    loss = np.zeros(steps, np.float32)
    X = np.ascontiguousarray(X, np.float32)
    Y = np.ascontiguousarray(Y, np.float32)
    st = L.bte_mlp_train(X.ctypes.data_as(C.c_void_p), Y.ctypes.data_as(C.c_void_p), len(Y), steps, batch,
                         C.c_float(lr), C.c_uint(seed), p.ctypes.data_as(C.c_void_p), loss.ctypes.data_as(C.c_void_p))
    if st != 0:
        raise S.BteError(st, L.bte_last_error(None).decode())
    return p, loss


def predict(params, X):
    """MLP outputs on the GPU (bte_mlp_predict)."""
    import staticbtesolver_gb300 as S

    L, _ = S._load()
    X = np.ascontiguousarray(X, np.float32)
    p = np.ascontiguousarray(params, np.float32)
    y = np.zeros(len(X), np.float32)
    st = L.bte_mlp_predict(X.ctypes.data_as(C.c_void_p), len(X), p.ctypes.data_as(C.c_void_p),
                           y.ctypes.data_as(C.c_void_p))
    if st != 0:
        raise S.BteError(st, L.bte_last_error(None).decode())
    return y


def shrink(params, X_val, Y_val):
    """Scale the output layer by lam = clip(<t, y> / <y, y>, 0, 1) fitted on held-out rows,
    so the correction is only as large as it predicts well.  Returns (params, lam)."""
    y = np.clip(predict(params, X_val).astype(np.float64), -CORR, CORR)
    lam = float(np.clip(np.dot(Y_val, y) / max(np.dot(y, y), 1e-30), 0.0, 1.0))
    return scaled(params, lam), lam


def scaled(params, lam):
    """The network with its output (last layer weights and bias) multiplied by lam."""
    p = np.array(params, np.float32)
    p[NPARAM - 129:] *= lam
    return p


def select_scale(params, specs, lams=(0.0, 0.25, 0.5, 0.75, 1.0), accel_every: int = EVERY, device: int = 0):
    """Pick the output scale by what it does: total outer iterations to margin <= 1e-5 of
    learned-accelerated solves on held-out problems, for each lam (lam = 0 is the Aitken
    extrapolation itself).  Returns (params scaled by the best lam, {lam: iterations})."""
    import staticbtesolver_gb300 as S

    totals = {}
    with tempfile.TemporaryDirectory() as tmp:
        probs = []
        for i, spec in enumerate(specs):
            p = write_problem(spec, os.path.join(tmp, str(i)))
            probs.append((S.Problem(p.geo, p.bc_file, p.band_file, p.DM, p.num_theta, p.num_phi, p.T_ref, p.L_x,
                                    p.L_y, p.L_z), p.max_iter))
        for lam in lams:
            tot = 0
            for prob, max_iter in probs:
                ctx = S.Context(device).load(prob)
                ctx.set_mlp(scaled(params, lam))
                st, rep = ctx.solve(max_iter=max_iter, tol=1e-5, form=S.FORM_SWEEP, accel=1, accel_every=accel_every)
                ctx.close()
                tot += rep.n_iter if st == 0 else 10 * max_iter
            totals[float(lam)] = tot
    best = min(totals, key=lambda k: (totals[k], k))
    return scaled(params, best), totals


def load(path: str = WEIGHTS) -> np.ndarray:
    return np.load(path).astype(np.float32)
