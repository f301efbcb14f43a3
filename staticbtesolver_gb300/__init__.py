"""GB300-native steady-state phonon BTE solve (the hot path of yuchengs/StaticBTESolver).

Python front end over the two in-tree native libraries:
  * ``libbte_cuda.so`` -- hand-written sm_103a kernels behind the C ABI of
    include/bte_cuda.h (assembly, batched BiCGSTAB, reductions, heat flux);
  * ``libstaticbtesolver_gb300.so`` -- the reference's C++ API
    (StaticBTESolver / BTEMesh / BTEBand / BTEBoundaryCondition) and the C
    entry points of include/sbte.h that read the reference's input files and
    run its preprocessing.

There is no CPU fallback: every solve runs on the GPU through the C ABI, and
a missing library or device raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import _build

__all__ = ["build", "Problem", "Context", "Options", "Report", "StaticBTESolver", "bicgstab_csr", "dsa_solve",
           "FORM_PLAIN", "FORM_MIXED", "FORM_SWEEP", "BteError", "lib_paths"]

FORM_PLAIN = 0
FORM_MIXED = 1
FORM_SWEEP = 2

STATUS = {0: "ok", 1: "invalid argument", 2: "call out of order", 3: "CUDA error", 4: "out of device memory",
          5: "unsupported boundary condition", 6: "not converged", 7: "non-finite value", 8: "no CUDA device"}
NOT_CONVERGED = 6

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")

ITER_CB = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_double, C.c_double)


class BteError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {msg}")


class Options(C.Structure):
    _fields_ = [("max_iter", C.c_int), ("tol", C.c_double), ("form", C.c_int), ("inner_tol", C.c_double),
                ("inner_maxit", C.c_int), ("batch_systems", C.c_int), ("on_iteration", ITER_CB),
                ("user", C.c_void_p), ("profile", C.c_int), ("accel", C.c_int), ("accel_every", C.c_int),
                ("keep_history", C.c_int), ("dsa", C.c_int), ("dsa_tol", C.c_double), ("dsa_maxit", C.c_int),
                ("plain_cycles", C.c_int)]


class KernelStat(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_longlong), ("ms", C.c_double), ("bytes", C.c_double)]


class Report(C.Structure):
    _fields_ = [("n_iter", C.c_int), ("converged", C.c_int), ("final_margin", C.c_double),
                ("inner_solves", C.c_longlong), ("inner_iterations", C.c_longlong),
                ("inner_unconverged", C.c_longlong), ("refinements", C.c_longlong), ("ms_total", C.c_double),
                ("ms_rhs", C.c_double), ("ms_inner", C.c_double), ("ms_reduce", C.c_double),
                ("kernel_launches", C.c_longlong), ("sweep_group", C.c_int), ("sweep_threads", C.c_int),
                ("accel_steps", C.c_int), ("accel_reverts", C.c_int), ("sweep_ring", C.c_int),
                ("sweep_margin", C.c_int), ("dsa_solves", C.c_int), ("dsa_iterations", C.c_longlong),
                ("ms_dsa", C.c_double), ("sweep_kernel", C.c_int),
                ("ms_host_setup", C.c_double), ("ms_host_plan", C.c_double), ("ms_host_order", C.c_double),
                ("ms_host_dsa", C.c_double),
                ("ms_wall", C.c_double), ("sweep_host_dirs", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_cuda = None
_host = None


def build(force: bool = False) -> None:
    _build.build(force=force)


def lib_paths():
    return _build.LIB_CUDA, _build.LIB_HOST, _build.BTECMD


def _load():
    global _cuda, _host
    if _cuda is not None:
        return _cuda, _host
    for p in (_build.LIB_CUDA, _build.LIB_HOST):
        if not os.path.exists(p):
            raise ImportError(f"native library {p} is missing; run staticbtesolver_gb300.build()")
    L = C.CDLL(_build.LIB_CUDA, mode=C.RTLD_GLOBAL)
    vp = C.c_void_p
    L.bte_default_options.argtypes = [C.POINTER(Options)]
    L.bte_status_string.restype = C.c_char_p
    L.bte_status_string.argtypes = [C.c_int]
    L.bte_last_error.restype = C.c_char_p
    L.bte_last_error.argtypes = [vp]
    L.bte_create.argtypes = [C.POINTER(vp), C.c_int]
    L.bte_destroy.argtypes = [vp]
    L.bte_set_geometry.argtypes = [vp, C.c_int, C.c_int, C.c_int, _ip, _dp, _dp, _dp]
    L.bte_set_quadrature.argtypes = [vp, C.c_int, _dp, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double]
    L.bte_set_bands.argtypes = [vp, C.c_int, _dp, _dp, _dp, _dp]
    L.bte_set_bcs.argtypes = [vp, C.c_int, _ip, _ip, _dp]
    L.bte_solve.argtypes = [vp, C.POINTER(Options), C.POINTER(Report)]
    L.bte_get_temperature.argtypes = [vp, _dp]
    L.bte_get_band_temperature.argtypes = [vp, _dp]
    L.bte_get_heat_flux.argtypes = [vp, _dp, C.c_void_p]
    L.bte_get_energy.argtypes = [vp, _dp]
    L.bte_get_margins.argtypes = [vp, C.c_void_p, C.c_int, C.POINTER(C.c_int)]
    for fn in ("bte_set_mlp", "bte_set_centroids", "bte_get_history", "bte_mlp_predict", "bte_mlp_gradient",
               "bte_mlp_train"):
        getattr(L, fn).restype = C.c_int
    L.bte_set_mlp.argtypes = [vp, C.c_void_p]
    L.bte_set_centroids.argtypes = [vp, _dp]
    L.bte_get_history.argtypes = [vp, C.c_void_p, C.c_int, C.POINTER(C.c_int)]
    L.bte_mlp_predict.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    L.bte_mlp_gradient.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
    L.bte_mlp_train.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_uint, C.c_void_p,
                                C.c_void_p]
    L.bte_mlp_param_count.restype = C.c_int
    L.bte_get_kernel_stats.argtypes = [vp, C.c_void_p, C.c_int, C.POINTER(C.c_int)]
    L.bte_get_kernel_stats.restype = C.c_int
    L.bte_get_sweep_tuning.argtypes = [vp, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                       C.POINTER(C.c_int)]
    L.bte_get_sweep_tuning.restype = C.c_int
    L.bte_get_level_order.argtypes = [vp, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_int)]
    L.bte_get_level_order.restype = C.c_int
    L.bte_bicgstab_csr.argtypes = [C.c_int, _ip, _ip, _dp, C.c_int, _dp, _dp, C.c_int, C.c_double,
                                   C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.bte_dsa_solve.argtypes = [C.c_int, C.c_int, _ip, _dp, _dp, _dp, C.c_double, C.c_int, C.POINTER(C.c_int),
                                C.POINTER(C.c_double)]
    for fn in ("bte_create", "bte_destroy", "bte_set_geometry", "bte_set_quadrature", "bte_set_bands",
               "bte_set_bcs", "bte_solve", "bte_get_temperature", "bte_get_band_temperature", "bte_get_heat_flux",
               "bte_get_energy", "bte_get_margins", "bte_bicgstab_csr", "bte_dsa_solve"):
        getattr(L, fn).restype = C.c_int
    H = C.CDLL(_build.LIB_HOST)
    H.sbte_open.restype = vp
    H.sbte_open.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                            C.c_double, C.c_double]
    H.sbte_error.restype = C.c_char_p
    H.sbte_close.argtypes = [vp]
    H.sbte_counts.argtypes = [vp, _ip]
    H.sbte_quadrature.argtypes = [vp, _dp, _dp, _dp, _dp]
    H.sbte_geometry.argtypes = [vp, _dp, _dp, _dp, _dp, _ip]
    H.sbte_bands.argtypes = [vp, _dp, _dp, _dp, _dp]
    H.sbte_bcs.argtypes = [vp, _ip, _ip, _dp]
    H.sbte_upload.restype = C.c_int
    H.sbte_upload.argtypes = [vp, vp]
    H.sbte_write_tempcell.restype = C.c_int
    H.sbte_write_tempcell.argtypes = [C.c_char_p, C.c_int, C.c_int, _dp, _dp, C.c_double, C.c_double, C.c_double]
    _cuda, _host = L, H
    return L, H


def default_options(**kw) -> Options:
    L, _ = _load()
    o = Options()
    L.bte_default_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class Problem:
    """A problem read from the reference's input files and preprocessed on the host.

    Mirrors what BTEcmd builds from -g/-m/-b/-d/-t/-p/-T/-x/-y/-z.
    """

    def __init__(self, geo, bc_file, band_file, DM, num_theta, num_phi, T_ref=300.0, L_x=0.0, L_y=0.0, L_z=0.0):
        _, H = _load()
        self._h = H.sbte_open(str(geo).encode(), str(bc_file).encode(), str(band_file).encode(), int(DM),
                              int(num_theta), int(num_phi), float(T_ref), float(L_x), float(L_y), float(L_z))
        if not self._h:
            raise BteError(1, H.sbte_error().decode())
        c = np.zeros(6, np.int32)
        H.sbte_counts(self._h, c)
        self.n_cell, self.n_dir, self.n_band, self.n_face, self.n_bc, self.dim = map(int, c)
        self.DM, self.num_theta, self.num_phi = int(DM), int(num_theta), int(num_phi)

    def close(self):
        if getattr(self, "_h", None):
            _host.sbte_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def quadrature(self):
        nd = self.n_dir
        s, S, w, sc = np.zeros(3 * nd), np.zeros(3 * nd), np.zeros(nd), np.zeros(5)
        _host.sbte_quadrature(self._h, s, S, w, sc)
        return dict(s=s.reshape(nd, 3), S=S.reshape(nd, 3), omega=w, solid_angle=sc[0], T_ref=sc[1],
                    wfactor=sc[2], ms_quadrature=sc[3], ms_geometry=sc[4])

    def geometry(self):
        n, nf = self.n_cell, self.n_face
        vol, cen, area = np.zeros(n), np.zeros(3 * n), np.zeros(n * nf)
        nrm, nbr = np.zeros(3 * n * nf), np.zeros(n * nf, np.int32)
        _host.sbte_geometry(self._h, vol, cen, area, nrm, nbr)
        return dict(volume=vol, centroid=cen.reshape(n, 3), area=area.reshape(n, nf),
                    normal=nrm.reshape(n, nf, 3), nbr=nbr.reshape(n, nf))

    def bands(self):
        nb = self.n_band
        a = [np.zeros(nb) for _ in range(4)]
        _host.sbte_bands(self._h, *a)
        return dict(vg=a[0], tau=a[1], C=a[2], Lr=a[3])

    def bcs(self):
        k = max(self.n_bc, 1)
        idx, typ, T = np.zeros(k, np.int32), np.zeros(k, np.int32), np.zeros(k)
        _host.sbte_bcs(self._h, idx, typ, T)
        return dict(index=idx[: self.n_bc], type=typ[: self.n_bc], T=T[: self.n_bc])

    def arrays(self):
        """Everything the C ABI takes, as host arrays (for bte_set_* calls)."""
        q, g = self.quadrature(), self.geometry()
        return dict(dim=self.dim, n_cell=self.n_cell, n_face=self.n_face, n_dir=self.n_dir, DM=self.DM,
                    num_theta=self.num_theta, num_phi=self.num_phi, **g, **q, bands=self.bands(), bcs=self.bcs())


@dataclass
class Result:
    T: np.ndarray
    Tb: np.ndarray
    q: np.ndarray
    q_band: np.ndarray
    margins: np.ndarray
    report: dict
    status: int


class Context:
    """One bte_ctx: a device, a stream and the resident problem."""

    def __init__(self, device: int = 0):
        L, _ = _load()
        h = C.c_void_p()
        st = L.bte_create(C.byref(h), int(device))
        if st != 0:
            raise BteError(st, L.bte_last_error(None).decode())
        self._h = h
        self._dims = None

    def close(self):
        if getattr(self, "_h", None):
            _cuda.bte_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, what=""):
        if st != 0:
            raise BteError(st, (what + ": " if what else "") + _cuda.bte_last_error(self._h).decode())

    def load(self, problem: Problem):
        self._check(_host.sbte_upload(problem._h, self._h), "upload")
        self._dims = (problem.n_cell, problem.n_dir, problem.n_band, problem.n_bc)
        return self

    def set_arrays(self, a: dict):
        """bte_set_* from host arrays (as returned by Problem.arrays())."""
        L = _cuda
        f64 = lambda x: np.ascontiguousarray(x, np.float64).ravel()
        i32 = lambda x: np.ascontiguousarray(x, np.int32).ravel()
        self._check(L.bte_set_geometry(self._h, a["dim"], a["n_cell"], a["n_face"], i32(a["nbr"]), f64(a["area"]),
                                       f64(a["normal"]), f64(a["volume"])), "geometry")
        nb_dm = a.get("DM"), a.get("num_theta"), a.get("num_phi")
        self._check(L.bte_set_quadrature(self._h, a["n_dir"], f64(a["s"]), f64(a["S"]), f64(a["omega"]), *nb_dm,
                                         float(a["solid_angle"]), float(a["T_ref"])), "quadrature")
        b = a["bands"]
        self._check(L.bte_set_bands(self._h, len(b["vg"]), f64(b["vg"]), f64(b["tau"]), f64(b["C"]), f64(b["Lr"])),
                    "bands")
        c = a["bcs"]
        n_bc = len(c["index"])
        self._check(L.bte_set_bcs(self._h, n_bc, i32(c["index"]) if n_bc else np.zeros(1, np.int32),
                                  i32(c["type"]) if n_bc else np.zeros(1, np.int32),
                                  f64(c["T"]) if n_bc else np.zeros(1)), "bcs")
        if "centroid" in a:
            self._check(L.bte_set_centroids(self._h, f64(a["centroid"])), "centroids")
        self._dims = (a["n_cell"], a["n_dir"], len(b["vg"]), n_bc)
        return self

    def set_mlp(self, params):
        p = np.ascontiguousarray(params, np.float32)
        self._check(_cuda.bte_set_mlp(self._h, p.ctypes.data_as(C.c_void_p)), "set_mlp")
        return self

    def history(self):
        k = C.c_int(0)
        _cuda.bte_get_history(self._h, None, 0, C.byref(k))
        h = np.zeros((k.value, self._dims[0]))
        _cuda.bte_get_history(self._h, h.ctypes.data_as(C.c_void_p), k.value, C.byref(k))
        return h

    def solve(self, max_iter=1000, tol=1e-5, form=FORM_PLAIN, inner_tol=1e-9, inner_maxit=1000,
              batch_systems=0, on_iteration=None, raise_on_not_converged=False, profile=False, accel=0,
              accel_every=8, keep_history=False, dsa=False, dsa_tol=0.0, dsa_maxit=0, plain_cycles=0):
        o = default_options(max_iter=int(max_iter), tol=float(tol), form=int(form), inner_tol=float(inner_tol),
                            inner_maxit=int(inner_maxit), batch_systems=int(batch_systems), profile=int(profile),
                            accel=int(accel), accel_every=int(accel_every), keep_history=int(bool(keep_history)),
                            dsa=int(bool(dsa)), dsa_tol=float(dsa_tol), dsa_maxit=int(dsa_maxit),
                            plain_cycles=int(plain_cycles))
        cb = None
        if on_iteration is not None:
            cb = ITER_CB(lambda _u, it, m, ms: on_iteration(it, m, ms))
            o.on_iteration = cb
        rep = Report()
        st = _cuda.bte_solve(self._h, C.byref(o), C.byref(rep))
        if st != 0 and not (st == NOT_CONVERGED and not raise_on_not_converged):
            self._check(st, "solve")
        return st, rep

    def temperature(self):
        T = np.zeros(self._dims[0])
        self._check(_cuda.bte_get_temperature(self._h, T))
        return T

    def band_temperature(self):
        n, _, nb, _ = self._dims
        Tb = np.zeros(n * nb)
        self._check(_cuda.bte_get_band_temperature(self._h, Tb))
        return Tb.reshape(n, nb)

    def heat_flux(self):
        _, _, nb, nbc = self._dims
        q, qb = np.zeros(max(nbc, 1)), np.zeros(max(nbc * nb, 1))
        self._check(_cuda.bte_get_heat_flux(self._h, q, qb.ctypes.data_as(C.c_void_p)))
        return q[:nbc], qb[: nbc * nb].reshape(nbc, nb)

    def energy(self):
        n, nd, nb, _ = self._dims
        e = np.zeros(nb * nd * n)
        self._check(_cuda.bte_get_energy(self._h, e))
        return e.reshape(nb, nd, n)

    def kernel_stats(self):
        arr = (KernelStat * 32)()
        n = C.c_int(0)
        self._check(_cuda.bte_get_kernel_stats(self._h, C.cast(arr, C.c_void_p), 32, C.byref(n)))
        return {arr[i].name.decode(): dict(launches=arr[i].launches, ms=arr[i].ms, bytes=arr[i].bytes)
                for i in range(n.value)}

    def sweep_tuning(self):
        """The sweep autotuner's candidates on this context's plan, as dicts
        (bands and threads per block, ring positions per band, kernel "level",
        "staged" or "split", milliseconds); empty when the shape came from the
        per-process cache."""
        n = C.c_int(0)
        self._check(_cuda.bte_get_sweep_tuning(self._h, None, None, None, None, None, 0, C.byref(n)))
        m = n.value
        cols = [np.zeros(max(m, 1), np.int32) for _ in range(4)] + [np.zeros(max(m, 1), np.float32)]
        self._check(_cuda.bte_get_sweep_tuning(self._h, *[c.ctypes.data_as(C.c_void_p) for c in cols], m,
                                               C.byref(n)))
        return [dict(group=int(cols[0][k]), threads=int(cols[1][k]), ring=int(cols[2][k]),
                     kernel=("level", "staged", "split")[int(cols[3][k])], ms=float(cols[4][k])) for k in range(m)]

    def level_order(self, d):
        """The sweep plan's level order of direction d: (cells in order, level starts then n)."""
        n = self._dims[0]
        perm = np.zeros(n, np.int32)
        lvl = np.zeros(n + 1, np.int32)
        k = C.c_int(0)
        self._check(_cuda.bte_get_level_order(self._h, int(d), perm.ctypes.data_as(C.c_void_p),
                                              lvl.ctypes.data_as(C.c_void_p), n + 1, C.byref(k)))
        return perm, lvl[:k.value + 1].copy()

    def margins(self):
        k = C.c_int(0)
        _cuda.bte_get_margins(self._h, None, 0, C.byref(k))
        m = np.zeros(max(k.value, 1))
        _cuda.bte_get_margins(self._h, m.ctypes.data_as(C.c_void_p), k.value, C.byref(k))
        return m[: k.value]

    def result(self, st, rep) -> Result:
        q, qb = self.heat_flux()
        return Result(T=self.temperature(), Tb=self.band_temperature(), q=q, q_band=qb, margins=self.margins(),
                      report=rep.as_dict(), status=st)


def write_tempcell(path, centroid, T, dim, L):
    """T at the cell centroids in the reference's Tempcell.dat format
    (src/StaticBTESolver.cpp:818-831): "x/L_x y/L_y [z/L_z] T" per cell."""
    _, H = _load()
    cen = np.ascontiguousarray(centroid, np.float64).reshape(-1, 3)
    T = np.ascontiguousarray(T, np.float64)
    if len(T) != len(cen):
        raise BteError(1, "write_tempcell: centroid and T sizes differ")
    st = H.sbte_write_tempcell(str(path).encode(), len(T), int(dim), cen, T,
                               *map(float, L))
    if st != 0:
        raise BteError(st, H.sbte_error().decode())


class StaticBTESolver:
    """Python mirror of the reference's StaticBTESolver (ctor, setParam, solve) on file inputs."""

    def __init__(self, geo, bc_file, band_file, L_x=0.0, L_y=0.0, L_z=0.0, device=0):
        self._files = (geo, bc_file, band_file)
        self._L = (L_x, L_y, L_z)
        self._param = (3, 4, 4, 300.0)
        self._device = device
        self.result = None

    def setParam(self, DM, num_theta, num_phi, T_ref):
        self._param = (DM, num_theta, num_phi, T_ref)

    def solve(self, max_iter, tol=1e-5, form=FORM_PLAIN, inner_tol=1e-9, on_iteration=None) -> Result:
        p = Problem(*self._files, *self._param, *self._L)
        ctx = Context(self._device).load(p)
        st, rep = ctx.solve(max_iter=max_iter, tol=tol, form=form, inner_tol=inner_tol, on_iteration=on_iteration)
        self.result = ctx.result(st, rep)
        self._geometry = (p.arrays()["centroid"], p.dim)
        ctx.close()
        return self.result

    def writeTempcell(self, path="Tempcell.dat"):
        if self.result is None:
            raise BteError(2, "writeTempcell: solve first")
        write_tempcell(path, self._geometry[0], self.result.T, self._geometry[1], self._L)


def dsa_solve(nb, W, b, tol=1e-6, maxit=4000):
    """The low-order diffusion solve of the dsa option on the GPU (bte_dsa_solve):
    nb[f][c] neighbour (-1 none / wall), W[f][c] >= 0 symmetric couplings, b[n];
    returns (x, iterations, relative residual of the Jacobi-scaled system)."""
    L, _ = _load()
    nb = np.ascontiguousarray(nb, np.int32)
    W = np.ascontiguousarray(W, np.float64)
    F, n = nb.shape
    x = np.zeros(n)
    it, rr = C.c_int(0), C.c_double(0.0)
    st = L.bte_dsa_solve(n, F, nb.ravel(), W.ravel(), np.ascontiguousarray(b, np.float64), x, float(tol), int(maxit),
                         C.byref(it), C.byref(rr))
    if st != 0:
        raise BteError(st, L.bte_last_error(None).decode())
    return x, it.value, rr.value


def bicgstab_csr(rowptr, col, val, b, maxit=1000, tol=1e-9):
    """The reference's BICGSTAB(n, maxit, tol).init(...).solve(x) on one CSR system (GPU)."""
    L, _ = _load()
    n = len(rowptr) - 1
    x = np.zeros(n)
    it, conv = C.c_int(0), C.c_int(0)
    st = L.bte_bicgstab_csr(n, np.ascontiguousarray(rowptr, np.int32), np.ascontiguousarray(col, np.int32),
                            np.ascontiguousarray(val, np.float64), int(len(col)), np.ascontiguousarray(b, np.float64),
                            x, int(maxit), float(tol), C.byref(it), C.byref(conv))
    if st != 0:
        raise BteError(st, "bte_bicgstab_csr")
    return x, it.value, bool(conv.value)
