"""Regenerate the golden fixtures under tests/golden/ (run where the reference is mounted).

Sources, all from the reference or from the reference's own code run here:
  * the five regression cases of the reference's test.sh (tests/{2DM1DG,3DM1DG,
    2DM2DG,3DM2DG,3DM3DG}): their input files are copied, and their recorded
    logs (*.sol) are parsed into expected.json (margin trajectory and heat
    flux per boundary, 6 significant digits; those logs stop at margin < 1e-4);
  * tests/testcase/2Dcase5 (78,190-cell mesh, gray band, specular side walls):
    mesh (gzipped), bands, boundary file, and its recorded GPU log;
  * tests/testcase/2Dcase2 (11,630-cell mesh): mesh (gzipped), bands and both
    recorded logs (GPU BiCGSTAB and CPU GMRES).  Those logs were made with
    specular (type 31) side walls at L = 1e-8 m: with the type-2 file shipped
    beside them (inputbc_2D.dat) the second margin is 2.14e10, with type 31 it
    is 6.00575e10 as logged, so the fixture's inputbc.dat uses type 31;
  * small seeded synthetic problems written by staticbtesolver_gb300.synth;
  * for every case, the temperature field, heat fluxes and margins of the
    reference's own CPU solver compiled here from its sources
    (oracle/Makefile `ref`, margin <= 1e-5 as in src/StaticBTESolver.cpp:798)
    -> ref.npz.

Usage:  python tests/golden/make_golden.py [--reference DIR]   (default: $STATICBTESOLVER_REFERENCE)
"""
from __future__ import annotations

import argparse
import gzip
import json
import os
import re
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from staticbtesolver_gb300 import synth  # noqa: E402

# name -> (mesh or 1D cell count, DM, num_theta, num_phi, L_x, L_y, L_z, max_iter), from test.sh:6-22
TESTSH = {
    "3DM3DG": ("mesh.mphtxt", 3, 4, 4, 1e-8, 1e-8, 1e-8, 1000),
    "3DM2DG": ("mesh.mphtxt", 3, 4, 4, 1e-8, 1e-8, 0.0, 1000),
    "3DM1DG": ("100", 3, 8, 1, 1e-8, 0.0, 0.0, 1000),
    "2DM2DG": ("mesh.mphtxt", 2, 8, 8, 1e-8, 1e-8, 0.0, 10000),
    "2DM1DG": ("100", 2, 8, 1, 1e-8, 0.0, 0.0, 10000),
}
SYNTH = ["square10_b40", "cube4_b2", "slab1d", "square16_b8"]


def parse_sol(path):
    margins, q = [], {}
    for line in open(path):
        m = re.search(r"Iteration #(\d+)\s+Margin per band per cell: (\S+)", line)
        if m:
            margins.append(float(m.group(2)))
        m = re.search(r"heat flux of Boundary Condition #(\d+): (\S+)", line)
        if m:
            q[int(m.group(1))] = float(m.group(2))
    return margins, [q[k] for k in sorted(q)]


def run_ref(case_dir, geo, bc, band, DM, nt, np_, Lx, Ly, Lz, max_iter):
    r = O.RefSolver.solve(geo, bc, band, DM, nt, np_, 300.0, max_iter, Lx, Ly, Lz)
    np.savez_compressed(os.path.join(case_dir, "ref.npz"), T=r.T, q=r.q, q_band=r.q_band, margins=r.margins,
                        n_iter=r.n_iter)
    return r


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=O.REFERENCE_ROOT)
    ap.add_argument("--only", default="", help="comma-separated case names")
    args = ap.parse_args()
    only = set(filter(None, args.only.split(",")))
    want = lambda n: not only or n in only
    ref = args.reference
    O.build()
    if not O.build_reference(ref):
        raise SystemExit("reference sources not found")
    for name, (geo, DM, nt, np_, Lx, Ly, Lz, max_iter) in TESTSH.items():
        if not want(name):
            continue
        src = os.path.join(ref, "tests", name)
        dst = os.path.join(HERE, name)
        os.makedirs(dst, exist_ok=True)
        for f in ("band.dat", "inputbc.dat") + (("mesh.mphtxt",) if geo.endswith(".mphtxt") else ()):
            shutil.copyfile(os.path.join(src, f), os.path.join(dst, f))
        margins, q = parse_sol(os.path.join(src, f"{name}.sol"))
        meta = dict(source=f"tests/{name}/{name}.sol", geo=geo, DM=DM, num_theta=nt, num_phi=np_, L_x=Lx, L_y=Ly,
                    L_z=Lz, max_iter=max_iter, T_ref=300.0, sol_margins=margins, sol_heat_flux=q,
                    sol_stop="first margin below 1e-4")
        g = os.path.join(dst, geo) if geo.endswith(".mphtxt") else geo
        r = run_ref(dst, g, os.path.join(dst, "inputbc.dat"), os.path.join(dst, "band.dat"), DM, nt, np_, Lx, Ly, Lz,
                    max_iter)
        meta["ref_n_iter"] = int(r.n_iter)
        json.dump(meta, open(os.path.join(dst, "expected.json"), "w"), indent=1)
        print(name, "ref iters", r.n_iter, "q", r.q)
    # 2Dcase2, 2Dcase5
    if want("2Dcase2"):
        case_2dcase2(ref)
    if want("2Dcase5"):
        case_2dcase5(ref)
    for name in SYNTH:
        if want(name):
            case_synth(name)


def case_2dcase2(ref):
    src = os.path.join(ref, "tests", "testcase", "2Dcase2")
    dst = os.path.join(HERE, "2Dcase2")
    os.makedirs(dst, exist_ok=True)
    with open(os.path.join(src, "2D_12000.mphtxt"), "rb") as fi, gzip.open(os.path.join(dst, "mesh.mphtxt.gz"), "wb") as fo:
        fo.write(fi.read())
    with open(os.path.join(dst, "inputbc.dat"), "w") as f:
        f.write("4 #number of boundaries\n\n#boundary index, type, temperature (side walls specular, see make_golden.py)\n"
                "0 1 301\n1 31 300\n2 31 300\n3 1 300\n")
    shutil.copyfile(os.path.join(src, "Input-dispersion-relation-fp.dat"), os.path.join(dst, "band.dat"))
    gm, gq = parse_sol(os.path.join(src, "StaticBTESolver-2DM-1np.sol"))
    cm, cq = parse_sol(os.path.join(src, "StaticBTESolver-2DM-1np-cpu-gmres.sol"))
    meta = dict(source="tests/testcase/2Dcase2", DM=2, num_theta=8, num_phi=8, L_x=1e-8, L_y=1e-8, L_z=0.0,
                max_iter=1000, T_ref=300.0, gpu_sol_margins=gm, gpu_sol_heat_flux=gq, cpu_sol_margins=cm,
                cpu_sol_heat_flux=cq, sol_stop="first margin below 1e-4")
    tmp = os.path.join(dst, "mesh.mphtxt")
    shutil.copyfile(os.path.join(src, "2D_12000.mphtxt"), tmp)
    r = run_ref(dst, tmp, os.path.join(dst, "inputbc.dat"), os.path.join(dst, "band.dat"), 2, 8, 8, 1e-8, 1e-8, 0.0,
                1000)
    os.remove(tmp)
    meta["ref_n_iter"] = int(r.n_iter)
    json.dump(meta, open(os.path.join(dst, "expected.json"), "w"), indent=1)
    print("2Dcase2 ref iters", r.n_iter, "q", r.q)


def case_2dcase5(ref):
    """tests/testcase/2Dcase5: 78,190 triangles, gray band, specular side walls as in
    its inputbc_2D.dat; its GPU log pins the margins (stop below 1e-4) and q."""
    src = os.path.join(ref, "tests", "testcase", "2Dcase5")
    dst = os.path.join(HERE, "2Dcase5")
    os.makedirs(dst, exist_ok=True)
    with open(os.path.join(src, "2D_78000.mphtxt"), "rb") as fi, gzip.open(os.path.join(dst, "mesh.mphtxt.gz"), "wb") as fo:
        fo.write(fi.read())
    shutil.copyfile(os.path.join(src, "inputbc_2D.dat"), os.path.join(dst, "inputbc.dat"))
    shutil.copyfile(os.path.join(src, "Input-dispersion-relation-fp.dat"), os.path.join(dst, "band.dat"))
    gm, gq = parse_sol(os.path.join(src, "StaticBTESolver-2DM-1np.sol"))
    meta = dict(source="tests/testcase/2Dcase5", DM=2, num_theta=8, num_phi=8, L_x=1e-8, L_y=1e-8, L_z=0.0,
                max_iter=1000, T_ref=300.0, gpu_sol_margins=gm, gpu_sol_heat_flux=gq,
                sol_stop="first margin below 1e-4")
    tmp = os.path.join(dst, "mesh.mphtxt")
    shutil.copyfile(os.path.join(src, "2D_78000.mphtxt"), tmp)
    r = run_ref(dst, tmp, os.path.join(dst, "inputbc.dat"), os.path.join(dst, "band.dat"), 2, 8, 8, 1e-8, 1e-8, 0.0,
                1000)
    os.remove(tmp)
    meta["ref_n_iter"] = int(r.n_iter)
    json.dump(meta, open(os.path.join(dst, "expected.json"), "w"), indent=1)
    print("2Dcase5 ref iters", r.n_iter, "q", r.q)


def case_synth(name):
    if True:
        dst = os.path.join(HERE, "synth", name)
        p = synth.make_problem(name, dst)
        geo = p.geo if p.geo.endswith(".mphtxt") else p.geo
        r = run_ref(dst, geo, p.bc_file, p.band_file, p.DM, p.num_theta, p.num_phi, p.L_x, p.L_y, p.L_z, p.max_iter)
        meta = p.args()
        for k in ("geo", "band_file", "bc_file"):
            if meta[k].endswith((".mphtxt", ".dat")):
                meta[k] = os.path.basename(meta[k])
        meta["ref_n_iter"] = int(r.n_iter)
        json.dump(meta, open(os.path.join(dst, "expected.json"), "w"), indent=1)
        print(name, "ref iters", r.n_iter, "q", r.q)


if __name__ == "__main__":
    main()
