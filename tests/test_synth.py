"""Seeded synthetic inputs: deterministic, valid meshes, formats the reference reads."""
import numpy as np

from staticbtesolver_gb300 import synth


def test_square_mesh_is_valid_and_deterministic():
    a = synth.square_mesh(60, seed=7)
    b = synth.square_mesh(60, seed=7)
    np.testing.assert_array_equal(a["tri"], b["tri"])
    np.testing.assert_array_equal(a["points"], b["points"])
    P, T = a["points"], a["tri"]
    area = 0.5 * ((P[T[:, 1], 0] - P[T[:, 0], 0]) * (P[T[:, 2], 1] - P[T[:, 0], 1])
                  - (P[T[:, 1], 1] - P[T[:, 0], 1]) * (P[T[:, 2], 0] - P[T[:, 0], 0]))
    assert (area > 0).all()
    assert abs(area.sum() - 1.0) < 1e-12
    # every edge is shared by 2 triangles or lies on the boundary list
    edges = {}
    for t in T:
        for k in range(3):
            e = tuple(sorted((t[k], t[(k + 1) % 3])))
            edges[e] = edges.get(e, 0) + 1
    bnd = {tuple(sorted(s)) for s in a["seg"]}
    for e, n in edges.items():
        assert n == 2 or (n == 1 and e in bnd)
    assert len(bnd) == 4 * 60


def test_square_mesh_is_delaunay():
    m = synth.square_mesh(10, seed=3)
    P, T = m["points"], m["tri"]
    for t in T[:50]:
        a, b, c = P[t]
        inside = [synth._incircle(*a, *b, *c, *P[v]) for v in range(len(P)) if v not in t]
        assert max(inside) <= 1e-12


def test_cube_mesh_is_valid():
    m = synth.cube_mesh(4, seed=5)
    P, T = m["points"], m["tet"]
    a, b, c, d = (P[T[:, k]] for k in range(4))
    vol = np.abs(np.einsum("ij,ij->i", np.cross(b - a, c - a), d - a)) / 6
    assert (vol > 0).all()
    assert abs(vol.sum() - 1.0) < 1e-12
    assert len(T) == 6 * 4 ** 3
    assert set(np.unique(m["tri_ent"])) == {0, 1, 2, 3, 4, 5}


def test_pore_carving():
    m = synth.cube_mesh(8, seed=5, pore_radius=0.2)
    assert 6 in set(np.unique(m["tri_ent"]))
    assert len(m["tet"]) < 6 * 8 ** 3


def test_square_pores():
    """Circular pores in the square: positive triangles, every edge shared by
    two triangles or listed as boundary, each pore wall (entity 4) a closed
    loop (every wall vertex on exactly two wall edges), no unused point."""
    pores = ((0.3, 0.3, 0.12), (0.68, 0.42, 0.15), (0.4, 0.75, 0.1))
    m = synth.square_mesh(48, pores=pores)
    P, T = m["points"], m["tri"]
    area = 0.5 * ((P[T[:, 1], 0] - P[T[:, 0], 0]) * (P[T[:, 2], 1] - P[T[:, 0], 1])
                  - (P[T[:, 1], 1] - P[T[:, 0], 1]) * (P[T[:, 2], 0] - P[T[:, 0], 0]))
    assert (area > 0).all()
    holes = sum(np.pi * r * r for _, _, r in pores)
    assert abs(area.sum() - (1.0 - holes)) < 0.02
    edges = {}
    for t in T:
        for k in range(3):
            e = tuple(sorted((int(t[k]), int(t[(k + 1) % 3]))))
            edges[e] = edges.get(e, 0) + 1
    bnd = {tuple(sorted(map(int, s))) for s in m["seg"]}
    assert all(n == 2 or (n == 1 and e in bnd) for e, n in edges.items())
    assert all(edges.get(e) == 1 for e in bnd)
    wall = m["seg"][m["seg_ent"] == 4]
    assert len(wall) > 0
    deg = np.bincount(wall.ravel(), minlength=len(P))
    assert set(np.unique(deg[deg > 0])) == {2}
    assert len(np.unique(T.ravel())) == len(P)


def test_debye_bands():
    b = synth.debye_bands(40)
    assert abs(b["C"].sum() - 1.627e6) < 1e-6
    assert abs(b["Lr"].sum() - 1.0) < 1e-12
    assert b["tau"].min() >= 1e-12 * (1 - 1e-12) and b["tau"].max() <= 1e-10 * (1 + 1e-12)
    assert abs(b["tau"][-1] - 1e-12) < 1e-24
    assert b["vg"][0] == 8000.0 and abs(b["vg"][-1] - 2000.0) < 1e-9
