"""In-tree build of the native libraries (no cmake; one nvcc TU, host TUs in parallel).

Outputs (git-ignored) in staticbtesolver_gb300/_build/:
  libbte_cuda.so                 sm_103a kernels + the C ABI of include/bte_cuda.h
  libstaticbtesolver_gb300.so    the StaticBTESolver C++ API and include/sbte.h
  BTEcmd                         the command-line tool
"""
from __future__ import annotations

import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
OUT = os.path.join(PKG, "_build")
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_SOURCES = ["utility.cpp", "io.cpp", "prepare.cpp", "StaticBTESolver.cpp", "sbte_c.cpp", "BTEMain.cpp"]

LIB_CUDA = os.path.join(OUT, "libbte_cuda.so")
LIB_HOST = os.path.join(OUT, "libstaticbtesolver_gb300.so")
BTECMD = os.path.join(OUT, "BTEcmd")


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run_all(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for c in cmds]
    errs = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errs.append(" ".join(c) + "\n" + out)
    if errs:
        raise RuntimeError("build failed:\n" + "\n\n".join(errs))


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> None:
    os.makedirs(OUT, exist_ok=True)
    cuda_deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "bte_cuda.h")]
    host_deps = [os.path.join(HOST, f) for f in os.listdir(HOST)] + [
        os.path.join(INCLUDE, f) for f in ("bte_cuda.h", "sbte.h")] + [
        os.path.join(INCLUDE, "StaticBTESolver", f) for f in os.listdir(os.path.join(INCLUDE, "StaticBTESolver"))]
    nvcc = _nvcc()
    cmds = []
    objs = []
    if force or _stale(LIB_CUDA, cuda_deps):
        cmds.append([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                     "-Xptxas", "-warn-spills", "-o", LIB_CUDA, os.path.join(CSRC, "bte_api.cu")])
    need_host = force or _stale(LIB_HOST, host_deps) or _stale(BTECMD, host_deps)
    if need_host:
        for src in HOST_SOURCES:
            obj = os.path.join(OUT, src.replace(".cpp", ".o"))
            objs.append(obj)
            cmds.append(["g++", "-std=c++17", "-O2", "-fPIC", "-Wall", "-c", os.path.join(HOST, src), "-o", obj])
    if cmds:
        _run_all(cmds)
    if need_host or force:
        _run_all([["g++", "-shared", "-o", LIB_HOST, *objs, "-L" + OUT, "-lbte_cuda", "-Wl,-rpath,$ORIGIN"]])
        _run_all([["g++", "-std=c++17", "-O2", "-o", BTECMD, os.path.join(HOST, "BTEcmd.cpp"), "-L" + OUT,
                   "-lstaticbtesolver_gb300", "-lbte_cuda", "-Wl,-rpath,$ORIGIN"]])
    if verbose:
        print("built", LIB_CUDA, LIB_HOST, BTECMD)


if __name__ == "__main__":
    build(force=True, verbose=True)
