"""The sweep plan's level order (staticbtesolver_gb300/csrc/sweep_order.h), on the CPU.

The header is plain C++; it is compiled here into a small shared library and
checked against a Python restatement of the same waves of Kahn's algorithm:
levels are the cells whose upstream cells are all in earlier levels, each
level in index order.  Acyclic upwind graphs (every planar mesh) give no
lagged edge and an order in which every inflow neighbour comes first; a cyclic
graph starts a level with the unprocessed cell of fewest unresolved inflow
edges and lags exactly those edges.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "staticbtesolver_gb300", "csrc", "sweep_order.h")

SRC = r'''
#include "%s"
extern "C" int level_order_c(int n, int F, const unsigned char* mask, const int* nbr, int* perm, int* lvl,
                             int* lagged) {
    std::vector<int> p, l, g;
    bte::level_order(n, F, mask, nbr, p, l, g);
    std::copy(p.begin(), p.end(), perm);
    std::copy(l.begin(), l.end(), lvl);
    std::copy(g.begin(), g.end(), lagged);
    return (int)l.size();
}
'''


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    d = tmp_path_factory.mktemp("sweep_order")
    src = d / "so.cpp"
    src.write_text(SRC % HEADER)
    out = d / "libso.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", str(out), str(src)], check=True)
    L = C.CDLL(str(out))
    L.level_order_c.restype = C.c_int
    return L


def run(lib, mask, nbr):
    n, F = nbr.shape
    perm = np.zeros(n, np.int32)
    lvl = np.zeros(n + 1, np.int32)
    lag = np.zeros(F * n, np.int32)
    m = np.ascontiguousarray(mask, np.uint8)
    nb = np.ascontiguousarray(nbr, np.int32)
    k = lib.level_order_c(n, F, m.ctypes.data_as(C.c_void_p), nb.ctypes.data_as(C.c_void_p),
                          perm.ctypes.data_as(C.c_void_p), lvl.ctypes.data_as(C.c_void_p),
                          lag.ctypes.data_as(C.c_void_p))
    return perm, lvl[:k], lag.reshape(F, n)


def waves(mask, nbr):
    """Kahn's algorithm in waves, acyclic graphs: level = cells all of whose
    inflow neighbours are placed, in index order."""
    n, F = nbr.shape
    up = [[int(nbr[c, f]) for f in range(F) if mask[c] >> f & 1] for c in range(n)]
    placed = np.zeros(n, bool)
    perm, lvl = [], []
    while len(perm) < n:
        wave = [c for c in range(n) if not placed[c] and all(placed[u] for u in up[c])]
        assert wave, "cyclic"
        lvl.append(len(perm))
        perm += wave
        placed[wave] = True
    lvl.append(n)
    return np.array(perm), np.array(lvl)


def triangle_masks(sbte, get_case, name, dirs):
    c = get_case(name)
    p = sbte.Problem(*c.args())
    g, q = p.geometry(), p.quadrature()
    n, F = p.n_cell, p.n_face
    nbr = g["nbr"].reshape(n, F).astype(np.int32)
    nrm = g["normal"].reshape(n, F, 3)
    s = q["s"].reshape(-1, 3)
    for d in dirs:
        inflow = (nrm @ s[d] < 0) & (nbr >= 0)
        yield (inflow * (1 << np.arange(F))).sum(1).astype(np.uint8), nbr


@pytest.mark.parametrize("name", ["square10_b40", "cube4_b2", "2DM2DG"])
def test_level_order_matches_waves(sbte, get_case, lib, name):
    for mask, nbr in triangle_masks(sbte, get_case, name, dirs=range(0, 8, 3)):
        perm, lvl, lag = run(lib, mask, nbr)
        wp, wl = waves(mask, nbr)
        np.testing.assert_array_equal(perm, wp)
        np.testing.assert_array_equal(lvl, wl)
        assert not lag.any()
        # every inflow neighbour sits on an earlier level
        level = np.empty(len(perm), int)
        for k in range(len(lvl) - 1):
            level[perm[lvl[k]:lvl[k + 1]]] = k
        n, F = nbr.shape
        for c in range(n):
            for f in range(F):
                if mask[c] >> f & 1:
                    assert level[nbr[c, f]] < level[c]


def test_level_order_lags_one_edge_per_cycle(lib):
    """Six cells in a ring, each fed by its predecessor: no cell is free, so
    cell 0 (fewest unresolved edges, lowest index) starts alone, its edge from
    cell 5 is lagged, and the rest follow one per level."""
    n = 6
    nbr = np.array([[(c - 1) % n, (c + 1) % n] for c in range(n)], np.int32)
    mask = np.full(n, 1, np.uint8)  # face 0 (from the predecessor) is inflow
    perm, lvl, lag = run(lib, mask, nbr)
    np.testing.assert_array_equal(perm, np.arange(n))
    np.testing.assert_array_equal(lvl, np.arange(n + 1))
    assert lag.sum() == 1 and lag[0, 0] == 1


def test_level_order_two_cycles_and_a_tail(lib):
    """Two disjoint 3-cycles feeding a tail cell: one lagged edge per cycle,
    and the tail comes after both."""
    # cells 0-1-2 cycle, 3-4-5 cycle, 6 fed by 2 and 5; F = 2 faces per cell
    nbr = np.array([[2, 6], [0, 2], [1, 0], [5, 6], [3, 5], [4, 3], [2, 5]], np.int32)
    mask = np.array([1, 1, 1, 1, 1, 1, 3], np.uint8)
    perm, lvl, lag = run(lib, mask, nbr)
    assert sorted(perm.tolist()) == list(range(7))
    assert perm[-1] == 6
    assert lag.sum() == 2
    pos = np.empty(7, int)
    pos[perm] = np.arange(7)
    for c in range(7):
        for f in range(2):
            if mask[c] >> f & 1 and not lag[f, c]:
                assert pos[nbr[c, f]] < pos[c]
