"""The allocation-free entry point bte_bicgstab_csr_noalloc.

Some callers cannot allocate device memory: their device memory belongs to
another allocator with a fixed budget (a framework's caching pool, an
application embedding this library), or they must not trigger the device-wide
synchronisation that cudaMalloc/cudaFree imply in the middle of their stream
work.  This entry point takes device inputs and outputs from the caller and
keeps all of its scratch in one static device array.  Here device buffers come
from torch (the caller's allocator), the results are compared with the
allocating entry point bte_bicgstab_csr on the same systems, on two calls in a
row (the second call must not see the first call's leftovers).  This file is
collected last so that a stop at the first failure has already run every
other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bidiagonal(n, seed):
    rng = np.random.default_rng(seed)
    rows, cols, vals = [], [], []
    for r in range(n):
        if r > 0:
            rows.append(r); cols.append(r - 1); vals.append(-rng.uniform(0.2, 0.9))
        rows.append(r); cols.append(r); vals.append(rng.uniform(1.0, 2.0))
        if r + 7 < n and r % 5 == 0:
            rows.append(r); cols.append(r + 7); vals.append(-rng.uniform(0.0, 0.1))
    order = np.lexsort((cols, rows))
    rows, cols, vals = np.array(rows)[order], np.array(cols, np.int32)[order], np.array(vals)[order]
    rp = np.searchsorted(rows, np.arange(n + 1)).astype(np.int32)
    return rp, cols, vals, rng.uniform(-1, 1, n)


def _noalloc(sbte, rp, ci, v, b, maxit=1000, tol=1e-9, free_memory=None):
    """One call through the C ABI on torch-owned device buffers.  free_memory
    (a list) receives the device's free bytes right before and right after
    the call itself."""
    import torch

    L, _ = sbte._load()
    f = L.bte_bicgstab_csr_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_double,
                  C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    dev = torch.device("cuda", 0)
    t_rp, t_ci = torch.from_numpy(rp).to(dev), torch.from_numpy(ci).to(dev)
    t_v, t_b = torch.from_numpy(v).to(dev), torch.from_numpy(b).to(dev)
    t_x = torch.full((len(b),), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    it, conv = C.c_int(0), C.c_int(0)
    torch.cuda.synchronize(dev)
    if free_memory is not None:
        free_memory.append(torch.cuda.mem_get_info(dev)[0])
    st = f(len(b), t_rp.data_ptr(), t_ci.data_ptr(), t_v.data_ptr(), len(ci), t_b.data_ptr(), t_x.data_ptr(),
           maxit, tol, C.c_void_p(stream), C.byref(it), C.byref(conv))
    torch.cuda.synchronize(dev)
    if free_memory is not None:
        free_memory.append(torch.cuda.mem_get_info(dev)[0])
    return st, t_x.cpu().numpy(), it.value, bool(conv.value)


def test_noalloc_matches_allocating_entry_on_two_calls(sbte):
    for n, seed in ((3000, 1), (1800, 2)):  # second call: smaller system, different values
        rp, ci, v, b = _bidiagonal(n, seed)
        st, x_na, it_na, conv_na = _noalloc(sbte, rp, ci, v, b)
        x_ref, it_ref, conv_ref = sbte.bicgstab_csr(rp, ci, v, b)
        assert st == 0
        assert conv_na and conv_ref
        assert it_na == it_ref
        assert np.linalg.norm(x_na - x_ref) <= 1e-12 * np.linalg.norm(x_ref)


def test_noalloc_call_allocates_no_device_memory(sbte):
    rp, ci, v, b = _bidiagonal(4000, 4)
    _noalloc(sbte, rp, ci, v, b)  # the first call on the device loads the module
    free = []
    st, x, _, conv = _noalloc(sbte, rp, ci, v, b, free_memory=free)
    assert st == 0 and conv
    assert free[0] == free[1], free


def test_noalloc_rejects_oversize_and_bad_csr(sbte):
    L, _ = sbte._load()
    rp, ci, v, b = _bidiagonal(100, 3)
    st, _, _, _ = _noalloc(sbte, rp, ci, v, b, maxit=10 ** 6)
    assert st == 1 and b"maxit" in L.bte_last_error(None)
    bad = ci.copy()
    bad[5] = 100  # column out of range
    st, _, _, _ = _noalloc(sbte, rp, bad, v, b)
    assert st == 1 and b"malformed" in L.bte_last_error(None)
    dec = rp.copy()
    dec[10], dec[11] = dec[11], dec[10]  # row pointers decrease
    assert dec[11] < dec[10]
    st, _, _, _ = _noalloc(sbte, dec, ci, v, b)
    assert st == 1 and b"malformed" in L.bte_last_error(None)
    short = rp.copy()
    short[-1] -= 1  # rowptr[n] != nnz
    st, _, _, _ = _noalloc(sbte, short, ci, v, b)
    assert st == 1 and b"malformed" in L.bte_last_error(None)
    # a good call after the rejected ones still matches the allocating entry
    st, x_na, _, _ = _noalloc(sbte, rp, ci, v, b)
    x_ref, _, _ = sbte.bicgstab_csr(rp, ci, v, b)
    assert st == 0 and np.linalg.norm(x_na - x_ref) <= 1e-12 * np.linalg.norm(x_ref)
    big = 1 << 18
    f = L.bte_bicgstab_csr_noalloc
    st = f(big + 1, None, None, None, 0, None, None, 10, 1e-9, None, None, None)
    assert st == 1 and b"262144" in L.bte_last_error(None)
