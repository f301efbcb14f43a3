"""Regenerate tests/golden/full/<name>.npz: a full-size synthetic workload solved by the oracle.

The oracle (oracle/bte_oracle.cpp, the reference's CPU algorithm: ILU(0)-GMRES inner
solves, margin <= 1e-5 as in src/StaticBTESolver.cpp:798) runs the whole source
iteration on the workload that the benchmark times.  The fixture keeps the cell
temperatures, the heat flux per boundary and per band, the margin trajectory, and
SHA-256 hashes of the generated mesh / band / boundary files so a test can check
that the generator still writes the same problem.

square20k takes about 40 minutes on 8 host threads.

square100k (--fixed-point): in the diffusive regime the source iteration's
error shrinks by ~1e-6 per outer iteration, so the oracle reaches the
iteration's fixed point through oracle/dsa.py instead (its own outer
iterations interleaved with a CPU diffusion correction), and certifies it by
one more uncorrected outer iteration; the fixture also keeps that
certificate.

cube200k (--iterations 2): the first outer iterations of the 3D configuration
(196,608 tetrahedra x 5,120 systems; a full solve is days of CPU time): the
fixture keeps T at every 4th cell, the sum of e over the cells of every
(band, direction) system, the margins and the heat flux after them.

cube15_b8: a converged solve of a 20,250-tetrahedron cube (8 bands x 128
directions), the 3D converged parity case.

Usage:  python tests/golden/full/make_full.py [square20k] [--threads 8]
        python tests/golden/full/make_full.py cube15_b8
        python tests/golden/full/make_full.py square100k --fixed-point
        python tests/golden/full/make_full.py cube200k --iterations 2
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, ROOT)

from oracle.oracle import Oracle  # noqa: E402
from staticbtesolver_gb300 import synth  # noqa: E402


def file_hashes(p) -> dict:
    return {k: hashlib.sha256(open(getattr(p, k), "rb").read()).hexdigest() for k in ("geo", "band_file", "bc_file")}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("name", nargs="?", default="square20k")
    ap.add_argument("--threads", type=int, default=8)
    ap.add_argument("--max-iter", type=int, default=1000)
    ap.add_argument("--fixed-point", action="store_true")
    ap.add_argument("--iterations", type=int, default=0)
    a = ap.parse_args()
    if a.fixed_point:
        return fixed_point(a)
    if a.iterations:
        return early(a)
    with tempfile.TemporaryDirectory() as tmp:
        p = synth.make_problem(a.name, tmp)
        h = file_hashes(p)
        o = Oracle(p.geo, p.bc_file, p.band_file, p.DM, p.num_theta, p.num_phi, p.T_ref, p.L_x, p.L_y, p.L_z)
        t = time.time()
        r = o.run(a.max_iter, 1e-5, threads=a.threads)
        el = time.time() - t
    print(a.name, "outer iterations", r.n_iter, "seconds", round(el, 1), "q", r.q)
    bands = synth.debye_bands(len(r.q_band[0]))  # see early(): kept so other hosts solve the same inputs
    np.savez_compressed(os.path.join(HERE, f"{a.name}.npz"), T=r.T, q=r.q, q_band=r.q_band, margins=r.margins,
                        n_iter=r.n_iter, seconds=el, inner_iterations=r.inner["iterations"], hashes=json.dumps(h),
                        band_vg=bands["vg"], band_tau=bands["tau"], band_C=bands["C"], band_Lr=bands["Lr"])


def early(a) -> None:
    with tempfile.TemporaryDirectory() as tmp:
        p = synth.make_problem(a.name, tmp)
        h = file_hashes(p)
        o = Oracle(p.geo, p.bc_file, p.band_file, p.DM, p.num_theta, p.num_phi, p.T_ref, p.L_x, p.L_y, p.L_z)
        t = time.time()
        r = o.run(a.iterations, 0.0, threads=a.threads, want_energy=True)
        el = time.time() - t
    e_sums = r.e.sum(axis=2)  # [n_band][n_dir]
    print(a.name, "outer iterations", r.n_iter, "seconds", round(el, 1), "margins", r.margins, "q", r.q)
    # the band values themselves: NumPy's exp/expm1 differ in the last bit
    # across CPU architectures, so another host regenerates them from these
    bands = synth.debye_bands(len(r.q_band[0]))
    np.savez_compressed(os.path.join(HERE, f"{a.name}_it{a.iterations}.npz"), T_every4=r.T[::4], T_sum=r.T.sum(),
                        band_vg=bands["vg"], band_tau=bands["tau"], band_C=bands["C"], band_Lr=bands["Lr"],
                        T_sq=np.sum((r.T - p.T_ref) ** 2), e_sums=e_sums, q=r.q, q_band=r.q_band,
                        margins=r.margins, n_iter=r.n_iter, seconds=el, hashes=json.dumps(h))


def fixed_point(a) -> None:
    from oracle import dsa

    with tempfile.TemporaryDirectory() as tmp:
        p = synth.make_problem(a.name, tmp)
        h = file_hashes(p)
        o = Oracle(p.geo, p.bc_file, p.band_file, p.DM, p.num_theta, p.num_phi, p.T_ref, p.L_x, p.L_y, p.L_z)
        t = time.time()
        T, e, m = dsa.fixed_point(o, p.band_file, p.bc_file, tol=1e-11, threads=a.threads,
                                  log=lambda k, mk: print(f"  corrected iteration {k}: margin {mk:.3e}", flush=True))
        q, q_band = o.heat_flux()
        el = time.time() - t
        cert_margin, cert_dT = dsa.certify(o, e, T, threads=a.threads)
    print(a.name, "corrected outer iterations", len(m), "seconds", round(el, 1), "certificate", cert_margin, cert_dT,
          "q", q)
    np.savez_compressed(os.path.join(HERE, f"{a.name}.npz"), T=T, q=q, q_band=q_band, margins=m, n_iter=len(m),
                        seconds=el, cert_margin=cert_margin, cert_dT=cert_dT, hashes=json.dumps(h))


if __name__ == "__main__":
    main()
