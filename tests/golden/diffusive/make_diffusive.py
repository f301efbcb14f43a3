"""Regenerate the diffusive-regime fixtures (run where the reference is mounted).

The reference's source iteration (src/StaticBTESolver.cpp:690-808) slows down
as the mean free paths shrink against the domain; these fixtures pin where it
ends up on such problems, so the GPU's diffusion-synthetic acceleration can be
checked against it:

  * square12_b8: a 1e-6 m square, 2 x 12^2 jittered-Delaunay triangles, 8 bands
    of the synthetic dispersion (Knudsen numbers ~1e-3 .. 0.8), left/right
    isothermal 301/299 K, top/bottom diffuse.  The reference's own CPU solver
    compiled here (oracle/Makefile `ref`) runs its plain iteration to its own
    stop (margin <= 1e-5, ~thousands of outer iterations) -> T_refbuild; the
    oracle restatement reaches the iteration's limit through oracle/dsa.py
    (its own outer iterations interleaved with a SciPy diffusion correction)
    -> T_fixed, certified by one more uncorrected oracle step.
  * squarepores: the same on a 1e-6 m square with three circular pores
    (synth.make_problem("squarepores"): 3,925 triangles, pore walls diffuse,
    entity 4), a non-convex domain with inner walls.  The reference build
    (compiled at -O0) did not reach its stop within an hour here, so this
    fixture holds the oracle's fixed point and the oracle's own first five
    plain outer iterations (T_it5, margins_it5) instead of the build's run.

Usage:  python tests/golden/diffusive/make_diffusive.py [name ...]
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, ROOT)

from oracle import dsa as D  # noqa: E402
from oracle import oracle as O  # noqa: E402
from staticbtesolver_gb300 import synth  # noqa: E402

WALLS = [(0, 1, 301.0), (1, 2, 300.0), (2, 1, 299.0), (3, 2, 300.0)]
PORES = ((0.3, 0.3, 0.12), (0.68, 0.42, 0.15), (0.4, 0.75, 0.1))  # as synth's squarepores
CASES = {"square12_b8": dict(n=12, bands=8, side=1e-6),
         "squarepores": dict(n=48, bands=8, side=1e-6, pores=PORES, rows=WALLS + [(4, 2, 300.0)], refbuild=False)}


def make(name, n, bands, side, pores=(), rows=WALLS, refbuild=True):
    d = os.path.join(HERE, name)
    os.makedirs(d, exist_ok=True)
    geo = os.path.join(d, "mesh.mphtxt")
    synth.write_mphtxt(geo, synth.square_mesh(n, pores=pores))
    synth.write_band_file(os.path.join(d, "band.dat"), synth.debye_bands(bands))
    synth.write_bc_file(os.path.join(d, "inputbc.dat"), rows)
    args = (geo, os.path.join(d, "inputbc.dat"), os.path.join(d, "band.dat"), 2, 8, 8, 300.0, side, side, 0.0)
    o = O.Oracle(*args)
    t0 = time.time()
    T_fp, e_fp, m_fp = D.fixed_point(o, args[2], args[1], tol=1e-13)
    q_fp, _ = o.heat_flux()
    cert_margin, cert_dT = D.certify(o, e_fp, T_fp)
    t_fp = time.time() - t0
    print(f"{name}: fixed point in {len(m_fp)} corrected oracle iterations ({t_fp:.1f} s); "
          f"one more plain step: margin {cert_margin:.2e}, |dT|/|T-Tref| {cert_dT:.2e}", flush=True)
    early = {}
    if not refbuild:  # the oracle's own first plain outer iterations
        o5 = O.Oracle(*args)
        r5 = o5.run(5, 0.0)
        early = dict(T_it5=r5.T, margins_it5=r5.margins, q_it5=r5.q)
    r = None
    if refbuild and O.RefSolver.available():
        t0 = time.time()
        r = O.RefSolver.solve(*args[:7], max_iter=100000, L_x=side, L_y=side, L_z=0.0)
        dist = float(np.linalg.norm(r.T - T_fp) / np.linalg.norm(T_fp - 300.0))
        print(f"{name}: reference build stops after {r.n_iter} plain iterations ({time.time() - t0:.1f} s), "
              f"rel L2(T - T_ref) from the fixed point {dist:.2e}", flush=True)
    np.savez_compressed(os.path.join(d, "ref.npz"), T_fixed=T_fp, q_fixed=q_fp, margins_fixed=m_fp,
                        cert_margin=cert_margin, cert_dT=cert_dT, **early,
                        **({} if r is None else dict(T_refbuild=r.T, q_refbuild=r.q, n_iter_refbuild=r.n_iter,
                                                     margins_refbuild=r.margins)))
    json.dump(dict(name=name, n=n, bands=bands, side=side, DM=2, num_theta=8, num_phi=8, T_ref=300.0,
                   corrected_iterations=len(m_fp), cert_margin=cert_margin, cert_dT=cert_dT,
                   n_iter_refbuild=None if r is None else int(r.n_iter)),
              open(os.path.join(d, "expected.json"), "w"), indent=1)


def main():
    O.build()
    for name, kw in CASES.items():
        if len(sys.argv) > 1 and name not in sys.argv[1:]:
            continue
        make(name, **kw)


if __name__ == "__main__":
    main()
