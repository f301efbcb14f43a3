"""The C ABI library loads and exports every entry point its headers declare.

No compute call is made here: these run on machines without a GPU.
"""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b((?:bte|sbte)_[a-z_0-9]+)\s*\(", text)))


def _exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


@pytest.mark.parametrize("header,lib_index", [("bte_cuda.h", 0), ("sbte.h", 1)])
def test_every_declared_symbol_is_exported(sbte, header, lib_index):
    lib = sbte.lib_paths()[lib_index]
    names = _declared(header)
    assert names, header
    exported = _exported(lib)
    if header == "sbte.h":
        names = [n for n in names if n.startswith("sbte_")]
    missing = [n for n in names if n not in exported]
    assert not missing, missing


def test_libraries_load(sbte):
    L, H = sbte._load()
    assert L.bte_status_string(0) == b"ok"
    assert L.bte_status_string(6).startswith(b"outer iteration")


def test_default_options_match_reference(sbte):
    o = sbte.default_options()
    assert o.max_iter == 10000 and o.tol == 1e-5 and o.inner_tol == 1e-9 and o.inner_maxit == 1000
    assert o.form == sbte.FORM_PLAIN


def test_csr_entry_rejects_bad_arguments_before_touching_a_device(sbte):
    import numpy as np
    L, _ = sbte._load()
    rp = np.array([0, 1, 3], np.int32)
    ci = np.array([0, 5, 1], np.int32)  # column 5 out of range
    v = np.ones(3)
    x = np.zeros(2)
    st = L.bte_bicgstab_csr(2, rp, ci, v, 3, np.ones(2), x, 10, 1e-9, None, None)
    assert st == 1


def test_create_without_device_reports_status(sbte):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    L, _ = sbte._load()
    h = ctypes.c_void_p()
    st = L.bte_create(ctypes.byref(h), 0)
    assert st in (3, 8)
    assert L.bte_last_error(None)
