"""ctypes front end to the oracle (TEST INFRASTRUCTURE ONLY).

The oracle is a CPU restatement of the reference's DOM-FVM phonon BTE source
iteration (oracle/bte_oracle.cpp), used by tests/, by ``__graft_entry__.smoke()``
and by bench.py's CPU-baseline leg as the checker.  The product never imports
this module.  ``RefSolver`` wraps the reference's own CPU code compiled from
its sources against the shims in oracle/shim (oracle/Makefile ``ref``); it only
exists on machines where the reference sources were present at build time.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libbte_ref.so")
REF_BIN_PATH = os.path.join(HERE, "_ref", "BTEcmd_ref")
# Where the reference's sources are mounted, when they are (the recipes that
# compile them read it from STATICBTESOLVER_REFERENCE; the GPU hosts have none).
REFERENCE_ROOT = os.environ.get("STATICBTESOLVER_REFERENCE", "/root/reference")

INNER_GMRES_ILU0 = 0
INNER_BICGSTAB = 1

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lp = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")

_lib = None


def build(quiet: bool = True) -> None:
    """Compile the oracle restatement (oracle/_build/liboracle.so)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


def build_reference(ref_root: str = REFERENCE_ROOT) -> bool:
    """Compile the reference's own CPU solver into oracle/_ref (if its sources exist)."""
    if not os.path.isdir(os.path.join(ref_root, "src")):
        return False
    out = subprocess.run(["make", "-C", HERE, "ref", f"REF={ref_root}"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference build failed:\n" + out.stdout + out.stderr)
    return True


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.oracle_open.restype = C.c_void_p
        L.oracle_open.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int,
                                  C.c_double, C.c_double, C.c_double, C.c_double]
        L.oracle_close.argtypes = [C.c_void_p]
        L.oracle_counts.argtypes = [C.c_void_p, _ip]
        L.oracle_quadrature.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
        L.oracle_geometry.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _ip]
        L.oracle_run.restype = C.c_int
        L.oracle_run.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int,
                                 C.c_longlong]
        L.oracle_step.restype = C.c_double
        L.oracle_step.argtypes = [C.c_void_p, _dp, _dp, C.c_int, C.c_double, C.c_int, C.c_void_p, _dp]
        L.oracle_temperature.argtypes = [C.c_void_p, _dp]
        L.oracle_band_temperature.argtypes = [C.c_void_p, _dp]
        L.oracle_heat_flux.argtypes = [C.c_void_p, _dp, _dp]
        L.oracle_margins.restype = C.c_int
        L.oracle_margins.argtypes = [C.c_void_p, _dp, C.c_int]
        L.oracle_energy.argtypes = [C.c_void_p, _dp]
        L.oracle_inner_stats.argtypes = [C.c_void_p, _lp, _dp]
        L.oracle_assemble.restype = C.c_int
        L.oracle_assemble.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, _dp]
        for name in ("oracle_bicgstab_csr", "oracle_gmres_csr"):
            f = getattr(L, name)
            f.restype = C.c_int
            f.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp, C.c_int, C.c_double, C.POINTER(C.c_int)]
        _lib = L
    return _lib


@dataclass
class Result:
    T: np.ndarray
    q: np.ndarray
    q_band: np.ndarray
    margins: np.ndarray
    n_iter: int
    Tb: np.ndarray | None = None
    e: np.ndarray | None = None
    inner: dict = field(default_factory=dict)


class Oracle:
    """One problem (mesh, bands, boundary conditions, angular parameters)."""

    def __init__(self, geo, bc_file, band_file, DM, num_theta, num_phi, T_ref=300.0,
                 L_x=0.0, L_y=0.0, L_z=0.0):
        L = lib()
        self._h = L.oracle_open(str(geo).encode(), str(bc_file).encode(), str(band_file).encode(),
                                DM, num_theta, num_phi, T_ref, L_x, L_y, L_z)
        if not self._h:
            raise FileNotFoundError(f"oracle could not read {geo}, {bc_file}, {band_file}")
        c = np.zeros(6, np.int32)
        L.oracle_counts(self._h, c)
        self.n_cell, self.n_dir, self.n_band, self.n_face, self.n_bc, self.dim = map(int, c)

    def close(self):
        if self._h:
            lib().oracle_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def quadrature(self):
        nd = self.n_dir
        s, S, w, sc = np.zeros(3 * nd), np.zeros(3 * nd), np.zeros(nd), np.zeros(3)
        lib().oracle_quadrature(self._h, s, S, w, sc)
        return dict(s=s.reshape(nd, 3), S=S.reshape(nd, 3), omega=w, solid_angle=sc[0],
                    wfactor=sc[1], T_ref=sc[2])

    def geometry(self):
        n, nf = self.n_cell, self.n_face
        vol, cen = np.zeros(n), np.zeros(3 * n)
        area, nrm, nbr = np.zeros(n * nf), np.zeros(3 * n * nf), np.zeros(n * nf, np.int32)
        lib().oracle_geometry(self._h, vol, cen, area, nrm, nbr)
        return dict(volume=vol, centroid=cen.reshape(n, 3), area=area.reshape(n, nf),
                    normal=nrm.reshape(n, nf, 3), nbr=nbr.reshape(n, nf))

    def run(self, max_iter=1000, outer_tol=1e-5, inner=INNER_GMRES_ILU0, inner_tol=1e-9,
            threads=0, max_systems=0, want_energy=False) -> Result:
        L = lib()
        it = L.oracle_run(self._h, max_iter, outer_tol, inner, inner_tol, threads, max_systems)
        T = np.zeros(self.n_cell)
        L.oracle_temperature(self._h, T)
        Tb = np.zeros(self.n_cell * self.n_band)
        L.oracle_band_temperature(self._h, Tb)
        q, qb = np.zeros(self.n_bc), np.zeros(self.n_bc * self.n_band)
        L.oracle_heat_flux(self._h, q, qb)
        m = np.zeros(max(it, 1))
        L.oracle_margins(self._h, m, len(m))
        st, sec = np.zeros(3, np.int64), np.zeros(1)
        L.oracle_inner_stats(self._h, st, sec)
        e = None
        if want_energy:
            e = np.zeros(self.n_band * self.n_dir * self.n_cell)
            L.oracle_energy(self._h, e)
            e = e.reshape(self.n_band, self.n_dir, self.n_cell)
        return Result(T=T, q=q, q_band=qb.reshape(self.n_bc, self.n_band), margins=m[:it], n_iter=it,
                      Tb=Tb.reshape(self.n_cell, self.n_band), e=e,
                      inner=dict(solves=int(st[0]), iterations=int(st[1]), unconverged=int(st[2]),
                                 seconds=float(sec[0])))

    def step(self, e_prev, T_src, inner=INNER_GMRES_ILU0, inner_tol=1e-9, threads=0, want_energy=True):
        """One outer iteration of the reference's source iteration from a given
        state (e_prev [n_band][n_dir][n_cell], source temperature T_src [n_cell]).
        Returns (e, T, margin); e is None unless want_energy."""
        e_prev = np.ascontiguousarray(e_prev, np.float64).reshape(-1)
        T_src = np.ascontiguousarray(T_src, np.float64)
        T = np.zeros(self.n_cell)
        e = np.zeros(self.n_band * self.n_dir * self.n_cell) if want_energy else None
        m = lib().oracle_step(self._h, e_prev, T_src, inner, inner_tol, threads,
                              e.ctypes.data_as(C.c_void_p) if e is not None else None, T)
        if e is not None:
            e = e.reshape(self.n_band, self.n_dir, self.n_cell)
        return e, T, float(m)

    def heat_flux(self):
        """Heat flux of the last run or step."""
        q, qb = np.zeros(self.n_bc), np.zeros(self.n_bc * self.n_band)
        lib().oracle_heat_flux(self._h, q, qb)
        return q, qb.reshape(self.n_bc, self.n_band)

    def assemble(self, band, direction, e_prev, ebar):
        n, nf = self.n_cell, self.n_face
        rowptr = np.zeros(n + 1, np.int32)
        col = np.zeros(nf * n + 1, np.int32)
        val = np.zeros(nf * n + 1)
        rhs = np.zeros(n)
        nnz = lib().oracle_assemble(self._h, band, direction, np.ascontiguousarray(e_prev, np.float64),
                                    np.ascontiguousarray(ebar, np.float64), rowptr, col, val, rhs)
        return rowptr, col[:nnz].copy(), val[:nnz].copy(), rhs


def bicgstab_csr(rowptr, col, val, b, maxit=1000, tol=1e-9):
    n = len(rowptr) - 1
    x = np.zeros(n)
    conv = C.c_int(0)
    it = lib().oracle_bicgstab_csr(n, np.ascontiguousarray(rowptr, np.int32), np.ascontiguousarray(col, np.int32),
                                   np.ascontiguousarray(val, np.float64), np.ascontiguousarray(b, np.float64),
                                   x, maxit, tol, C.byref(conv))
    return x, it, bool(conv.value)


def gmres_csr(rowptr, col, val, b, maxit=1000, rtol=1e-9):
    n = len(rowptr) - 1
    x = np.zeros(n)
    conv = C.c_int(0)
    it = lib().oracle_gmres_csr(n, np.ascontiguousarray(rowptr, np.int32), np.ascontiguousarray(col, np.int32),
                                np.ascontiguousarray(val, np.float64), np.ascontiguousarray(b, np.float64),
                                x, maxit, rtol, C.byref(conv))
    return x, it, bool(conv.value)


class RefSolver:
    """The reference's own CPU solver (compiled here from its sources), via ref_harness.cpp."""

    _L = None

    @classmethod
    def available(cls) -> bool:
        return os.path.exists(REF_LIB_PATH)

    @classmethod
    def _lib(cls):
        if cls._L is None:
            L = C.CDLL(REF_LIB_PATH)
            L.ref_solve.restype = C.c_int
            L.ref_solve.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int,
                                    C.c_double, C.c_int, C.c_double, C.c_double, C.c_double,
                                    _dp, C.c_int, _dp, C.c_int, _dp, C.c_int, _dp, C.c_int, _ip, _lp]
            cls._L = L
        return cls._L

    @classmethod
    def solve(cls, geo, bc_file, band_file, DM, num_theta, num_phi, T_ref=300.0, max_iter=1000,
              L_x=0.0, L_y=0.0, L_z=0.0, max_cells=2_000_000) -> Result:
        L = cls._lib()
        T = np.zeros(max_cells)
        q, qb, m = np.zeros(64), np.zeros(64 * 64), np.zeros(max(max_iter, 1))
        counts, inner = np.zeros(5, np.int32), np.zeros(3, np.int64)
        rc = L.ref_solve(str(geo).encode(), str(bc_file).encode(), str(band_file).encode(), DM,
                         num_theta, num_phi, T_ref, max_iter, L_x, L_y, L_z, T, len(T), q, len(q),
                         qb, len(qb), m, len(m), counts, inner)
        if rc != 0:
            raise RuntimeError(f"reference solve failed: {rc}")
        n_cell, n_iter, n_bc, n_band = (int(v) for v in counts[:4])
        return Result(T=T[:n_cell].copy(), q=q[:n_bc].copy(),
                      q_band=qb[: n_bc * n_band].reshape(n_bc, n_band).copy(),
                      margins=m[:n_iter].copy(), n_iter=n_iter,
                      inner=dict(solves=int(inner[0]), iterations=int(inner[1]), unconverged=int(inner[2])))
