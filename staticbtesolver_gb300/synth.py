"""Seeded synthetic inputs for the phonon BTE solve.

The reference measures nothing on public data; its workloads are meshes, band
files and boundary-condition files.  This module writes all three in the exact
formats the reference's readers accept (src/BTEMesh.cpp:7-130 for COMSOL
``.mphtxt``, src/BTEBand.cpp:8-26, src/BTEBoundaryCondition.cpp:7-23) so the
same files drive the reference build, the oracle and this package.

Meshes are on the unit square / unit cube; the physical size comes from the
``L_x/L_y/L_z`` scale factors, as with the reference's ``-x -y -z`` flags.

* 2D: a jittered (n+1) x (n+1) point grid (interior points moved by
  U(-j, j) h in x and y, edge points slide along their edge, corners fixed),
  triangulated and then made Delaunay by Lawson edge flips.  Boundary
  entities 0..3 = left, bottom, right, top; optional circular pores (the
  triangles whose centroid lies inside are removed), whose walls are
  entity 4.
* 3D: a jittered (n+1)^3 lattice, each cube split into the 6 Kuhn tetrahedra
  (conforming across cubes), with a positive-volume guard; optional
  cylindrical pore along z (cells whose centroid lies inside are removed and
  the new faces get their own entity).  Entities: 0 x=0, 1 y=0, 2 z=0,
  3 z=1, 4 y=1, 5 x=1, 6 pore wall.
* Bands: omega_i uniform midpoints in (0, omega_max]; group velocity linear
  from 8000 to 2000 m/s, decreasing with omega; tau = 1e-10 (omega_max /
  (10 omega))^2 clamped to [1e-12, 1e-10]; C_i proportional to the
  Bose-Einstein derivative hbar omega df/dT times the Debye density omega^2,
  normalised so sum C = 1.627e6 J m^-3 K^-1; Lr_i = (C_i/tau_i) / sum(C/tau).
"""
from __future__ import annotations

import os
from dataclasses import dataclass, asdict

import numpy as np

HBAR = 1.054571817e-34
KB = 1.380649e-23
C_TOTAL = 1.627e6


# --------------------------------------------------------------------------- bands
def debye_bands(n_band: int, omega_max: float = 1e14, T: float = 300.0, C_total: float = C_TOTAL):
    d = omega_max / n_band
    w = (np.arange(1, n_band + 1) - 0.5) * d
    if n_band > 1:
        vg = 8000.0 - 6000.0 * (w - w[0]) / (w[-1] - w[0])
    else:
        vg = np.array([6400.0])
    tau = np.clip(1e-10 * (0.1 * w[-1] / w) ** 2, 1e-12, 1e-10)
    x = HBAR * w / (KB * T)
    dfdT = x / T * np.exp(x) / np.expm1(x) ** 2
    C = HBAR * w * dfdT * w ** 2 * d
    C = C * (C_total / C.sum())
    Lr = (C / tau) / np.sum(C / tau)
    return dict(vg=vg, tau=tau, C=C, Lr=Lr)


def write_band_file(path: str, bands: dict) -> None:
    with open(path, "w") as f:
        for i in range(len(bands["vg"])):
            f.write(" ".join(repr(float(bands[k][i])) for k in ("vg", "tau", "C", "Lr")) + "\n")


def write_bc_file(path: str, rows) -> None:
    """rows: iterable of (entity, type, temperature)."""
    rows = list(rows)
    with open(path, "w") as f:
        f.write(f"{len(rows)} #number of boundaries\n\n")
        f.write("#boundary indexs #boundary condition type #temperature\n")
        for e, t, T in rows:
            f.write(f"{int(e)} {int(t)} {float(T)!r}\n")


# --------------------------------------------------------------------------- 2D mesh
def _incircle(ax, ay, bx, by, cx, cy, dx, dy):
    """> 0 when d lies inside the circumcircle of the counter-clockwise triangle abc."""
    adx, ady, bdx, bdy, cdx, cdy = ax - dx, ay - dy, bx - dx, by - dy, cx - dx, cy - dy
    ad, bd, cd = adx * adx + ady * ady, bdx * bdx + bdy * bdy, cdx * cdx + cdy * cdy
    return adx * (bdy * cd - bd * cdy) - ady * (bdx * cd - bd * cdx) + ad * (bdx * cdy - bdy * cdx)


def _lawson_flip(P: np.ndarray, tris: np.ndarray) -> np.ndarray:
    """Flip interior edges until every edge is locally Delaunay (Lawson)."""
    tris = [list(t) for t in tris]
    edge_map = {}
    for ti, t in enumerate(tris):
        for k in range(3):
            a, b = t[k], t[(k + 1) % 3]
            edge_map.setdefault((min(a, b), max(a, b)), []).append(ti)
    stack = [e for e, ts in edge_map.items() if len(ts) == 2]
    guard = 0
    while stack:
        guard += 1
        if guard > 50 * len(tris) + 1000:
            raise RuntimeError("edge flipping did not terminate")
        e = stack.pop()
        ts = edge_map.get(e)
        if not ts or len(ts) != 2:
            continue
        t0, t1 = ts
        a, b = e
        c = [v for v in tris[t0] if v not in e][0]
        d = [v for v in tris[t1] if v not in e][0]
        # orient (a, b, c) counter-clockwise
        tri = [a, b, c]
        area = (P[b, 0] - P[a, 0]) * (P[c, 1] - P[a, 1]) - (P[b, 1] - P[a, 1]) * (P[c, 0] - P[a, 0])
        if area < 0:
            tri = [b, a, c]
        if _incircle(*P[tri[0]], *P[tri[1]], *P[tri[2]], *P[d]) <= 1e-30:
            continue
        # flip only a strictly convex quadrilateral (c and d on opposite sides of a-b,
        # a and b on opposite sides of c-d)
        def _o(u, v, w):
            return (P[v, 0] - P[u, 0]) * (P[w, 1] - P[u, 1]) - (P[v, 1] - P[u, 1]) * (P[w, 0] - P[u, 0])
        if _o(c, d, a) * _o(c, d, b) >= 0 or _o(a, b, c) * _o(a, b, d) >= 0:
            continue
        # flip a-b to c-d
        for tt in (t0, t1):
            for k in range(3):
                u, v = tris[tt][k], tris[tt][(k + 1) % 3]
                key = (min(u, v), max(u, v))
                edge_map[key] = [x for x in edge_map[key] if x != tt]
        tris[t0] = [c, d, a]
        tris[t1] = [d, c, b]
        del edge_map[e]
        for tt in (t0, t1):
            for k in range(3):
                u, v = tris[tt][k], tris[tt][(k + 1) % 3]
                key = (min(u, v), max(u, v))
                edge_map.setdefault(key, []).append(tt)
        for key in ((min(a, c), max(a, c)), (min(c, b), max(c, b)), (min(b, d), max(b, d)), (min(d, a), max(d, a))):
            if len(edge_map.get(key, [])) == 2:
                stack.append(key)
    return np.array(tris, dtype=np.int64)


def _morton_order(xy: np.ndarray, bits: int = 16) -> np.ndarray:
    lo, hi = xy.min(axis=0), xy.max(axis=0)
    q = ((xy - lo) / np.maximum(hi - lo, 1e-300) * ((1 << bits) - 1)).astype(np.int64)
    code = np.zeros(len(xy), dtype=np.int64)
    dim = xy.shape[1]
    for bit in range(bits):
        for k in range(dim):
            code |= ((q[:, k] >> bit) & 1) << (dim * bit + k)
    return np.argsort(code, kind="stable")


def square_mesh(n: int, jitter: float = 0.3, seed: int = 20261203, delaunay: bool = True, pores=()):
    """Jittered (n+1)^2 grid on [0,1]^2, Delaunay-triangulated (2 n^2 triangles).

    delaunay=False keeps the first valid diagonal of every quad instead (a valid
    triangulation whose upwind graphs may contain cycles).  pores: circles
    (cx, cy, r) in unit coordinates; triangles whose centroid lies inside one
    are removed and the edges they leave open form entity 4."""
    rng = np.random.default_rng(seed)
    h = 1.0 / n
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    ii, jj = ii.ravel(), jj.ravel()  # point p = i*(n+1)+j at (i h, j h)
    x, y = ii * h, jj * h
    dx = rng.uniform(-jitter, jitter, size=x.shape) * h
    dy = rng.uniform(-jitter, jitter, size=y.shape) * h
    dx[(ii == 0) | (ii == n)] = 0.0  # left/right edge points slide along y only
    dy[(jj == 0) | (jj == n)] = 0.0  # bottom/top edge points slide along x only
    P = np.stack([x + dx, y + dy], axis=1)
    pid = lambda i, j: i * (n + 1) + j
    def orient(u, v, w):
        return (P[v, 0] - P[u, 0]) * (P[w, 1] - P[u, 1]) - (P[v, 1] - P[u, 1]) * (P[w, 0] - P[u, 0])

    tris = []
    for i in range(n):
        for j in range(n):
            a, b, c, d = pid(i, j), pid(i + 1, j), pid(i + 1, j + 1), pid(i, j + 1)
            # a jittered quad can be non-convex: take the diagonal that keeps both triangles positive
            if orient(a, b, c) > 0 and orient(a, c, d) > 0:
                tris += [[a, b, c], [a, c, d]]
            else:
                tris += [[a, b, d], [b, c, d]]
    tris = _lawson_flip(P, np.array(tris)) if delaunay else np.array(tris)
    # canonical form: counter-clockwise, smallest vertex first, Morton order of centroids
    out = []
    for t in tris:
        a, b, c = t
        if (P[b, 0] - P[a, 0]) * (P[c, 1] - P[a, 1]) - (P[b, 1] - P[a, 1]) * (P[c, 0] - P[a, 0]) < 0:
            b, c = c, b
        r = [a, b, c]
        k = int(np.argmin(r))
        out.append(r[k:] + r[:k])
    tris = np.array(out, dtype=np.int64)
    if len(pores):
        cen = P[tris].mean(axis=1)
        keep = np.ones(len(tris), dtype=bool)
        for cx, cy, r in pores:
            keep &= (cen[:, 0] - cx) ** 2 + (cen[:, 1] - cy) ** 2 > r ** 2
        tris = tris[keep]
    tris = tris[_morton_order(P[tris].mean(axis=1))]
    segs, ents = [], []
    for j in range(n):  # left x=0
        segs.append([pid(0, j), pid(0, j + 1)]); ents.append(0)
    for i in range(n):  # bottom y=0
        segs.append([pid(i, 0), pid(i + 1, 0)]); ents.append(1)
    for j in range(n):  # right x=1
        segs.append([pid(n, j), pid(n, j + 1)]); ents.append(2)
    for i in range(n):  # top y=1
        segs.append([pid(i, n), pid(i + 1, n)]); ents.append(3)
    if len(pores):
        # pore walls: interior edges left with one triangle, in sorted order
        E = np.sort(np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]]), axis=1)
        uniq, cnt = np.unique(E, axis=0, return_counts=True)
        outer = {tuple(sorted(s_)) for s_ in segs}
        for e in uniq[cnt == 1]:
            if tuple(e) not in outer:
                segs.append([int(e[0]), int(e[1])]); ents.append(4)
        used = np.unique(tris.ravel())
        remap = -np.ones(len(P), dtype=np.int64)
        remap[used] = np.arange(len(used))
        segs = remap[np.array(segs)]
        return dict(dim=2, points=P[used], tri=remap[tris], seg=segs, seg_ent=np.array(ents))
    return dict(dim=2, points=P, tri=tris, seg=np.array(segs), seg_ent=np.array(ents))


# --------------------------------------------------------------------------- 3D mesh
_KUHN = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]


def _tet_signed_volume(P, T):
    a, b, c, d = P[T[:, 0]], P[T[:, 1]], P[T[:, 2]], P[T[:, 3]]
    return np.einsum("ij,ij->i", np.cross(b - a, c - a), d - a) / 6.0


def cube_mesh(n: int, jitter: float = 0.3, seed: int = 20261203, pore_radius: float = 0.0):
    """Jittered (n+1)^3 lattice on [0,1]^3 split into 6 n^3 Kuhn tetrahedra."""
    rng = np.random.default_rng(seed)
    h = 1.0 / n
    ii, jj, kk = np.meshgrid(np.arange(n + 1), np.arange(n + 1), np.arange(n + 1), indexing="ij")
    ii, jj, kk = ii.ravel(), jj.ravel(), kk.ravel()
    base = np.stack([ii, jj, kk], axis=1) * h
    J = rng.uniform(-jitter, jitter, size=base.shape) * h
    J[(ii == 0) | (ii == n), 0] = 0.0
    J[(jj == 0) | (jj == n), 1] = 0.0
    J[(kk == 0) | (kk == n), 2] = 0.0
    pid = lambda i, j, k: (i * (n + 1) + j) * (n + 1) + k
    ci, cj, ck = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    ci, cj, ck = ci.ravel(), cj.ravel(), ck.ravel()
    tets = []
    for perm in _KUHN:
        o = np.zeros((len(ci), 3), dtype=np.int64)
        verts = [pid(ci, cj, ck)]
        for ax in perm:
            o[:, ax] += 1
            verts.append(pid(ci + o[:, 0], cj + o[:, 1], ck + o[:, 2]))
        tets.append(np.stack(verts, axis=1))
    T = np.concatenate(tets, axis=0)
    # positive-volume guard: drop the jitter of the vertices of any tetrahedron
    # that got too thin, until every Kuhn tetrahedron keeps >= 20% of h^3/6
    for _ in range(50):
        P = base + J
        vol = _tet_signed_volume(P, T)
        bad = np.abs(vol) < 0.2 * h ** 3 / 6
        # all Kuhn tetrahedra of one permutation share orientation sign
        sgn = np.sign(_tet_signed_volume(base, T))
        bad |= np.sign(vol) != sgn
        if not bad.any():
            break
        J[np.unique(T[bad].ravel())] *= 0.5
    P = base + J
    keep = np.ones(len(T), dtype=bool)
    if pore_radius > 0:
        cen = P[T].mean(axis=1)
        keep = (cen[:, 0] - 0.5) ** 2 + (cen[:, 1] - 0.5) ** 2 > pore_radius ** 2
    T = T[keep]
    T = T[_morton_order(P[T].mean(axis=1))]
    # boundary faces: faces used by exactly one tetrahedron
    F = np.concatenate([T[:, [1, 2, 3]], T[:, [0, 2, 3]], T[:, [0, 1, 3]], T[:, [0, 1, 2]]])
    Fs = np.sort(F, axis=1)
    _, idx, cnt = np.unique(Fs, axis=0, return_index=True, return_counts=True)
    bf = F[idx[cnt == 1]]
    bf = bf[np.lexsort(np.sort(bf, axis=1).T[::-1])]
    IJK = np.stack([ii, jj, kk], axis=1)
    g = IJK[bf]  # (m, 3 vertices, 3 axes)
    ent = np.full(len(bf), 6, dtype=np.int64)
    for axis, (lo_e, hi_e) in enumerate(((0, 5), (1, 4), (2, 3))):
        ent[np.all(g[:, :, axis] == 0, axis=1)] = lo_e
        ent[np.all(g[:, :, axis] == n, axis=1)] = hi_e
    used = np.unique(T.ravel())
    remap = -np.ones(len(P), dtype=np.int64)
    remap[used] = np.arange(len(used))
    return dict(dim=3, points=P[used], tet=remap[T], tri=remap[bf], tri_ent=ent,
                seg=np.zeros((0, 2), dtype=np.int64), seg_ent=np.zeros(0, dtype=np.int64))


# --------------------------------------------------------------------------- writer
def _section(f, name, nodes, conn, ent):
    f.write(f"# Type #{name[1]}\n\n3 {name[0]} # type name\n\n\n")
    f.write(f"{nodes} # number of nodes per element\n{len(conn)} # number of elements\n# Elements\n")
    for row in conn:
        f.write(" ".join(str(int(v)) for v in row) + "\n")
    if ent is not None:
        f.write(f"\n{len(ent)} # number of geometric entity indices\n# Geometric entity indices\n")
        for v in ent:
            f.write(f"{int(v)}\n")
    f.write("\n")


def write_mphtxt(path: str, mesh: dict) -> None:
    dim, P = mesh["dim"], mesh["points"]
    types = [("edg", 1)] + ([("tri", 2)] if dim >= 2 else []) + ([("tet", 3)] if dim == 3 else [])
    with open(path, "w") as f:
        f.write("# Synthetic mesh written by staticbtesolver_gb300.synth\n\n\n")
        f.write("# Major & minor version\n0 1 \n1 # number of tags\n# Tags\n5 mesh1\n1 # number of types\n# Types\n3 obj\n\n")
        f.write("# --------- Object 0 ----------\n\n0 0 1\n4 Mesh # class\n4 # version\n")
        f.write(f"{dim} # sdim\n{len(P)} # number of mesh points\n0 # lowest mesh point index\n\n")
        f.write("# Mesh point coordinates\n")
        for p in P:
            f.write(" ".join(repr(float(v)) for v in p[:dim]) + "\n")
        f.write(f"\n{len(types)} # number of element types\n\n")
        _section(f, ("edg", 1), 2, mesh["seg"], mesh["seg_ent"])
        if dim >= 2:
            _section(f, ("tri", 2), 3, mesh["tri"], mesh.get("tri_ent") if dim == 3 else np.zeros(len(mesh["tri"]), int))
        if dim == 3:
            _section(f, ("tet", 3), 4, mesh["tet"], np.ones(len(mesh["tet"]), int))


# --------------------------------------------------------------------------- configs
@dataclass
class Problem:
    """Everything the reference's BTEcmd takes: -g -m -b -d -t -p -T -I -x -y -z."""

    name: str
    geo: str
    band_file: str
    bc_file: str
    DM: int
    num_theta: int
    num_phi: int
    T_ref: float = 300.0
    max_iter: int = 1000
    L_x: float = 0.0
    L_y: float = 0.0
    L_z: float = 0.0

    def args(self):
        return asdict(self)

    def btecmd_flags(self):
        """The BTEcmd command line of this problem (-m is the band file, -b the boundary file)."""
        return ["-g", self.geo, "-m", self.band_file, "-b", self.bc_file, "-d", str(self.DM), "-t",
                str(self.num_theta), "-p", str(self.num_phi), "-T", repr(self.T_ref), "-I", str(self.max_iter),
                "-x", repr(self.L_x), "-y", repr(self.L_y), "-z", repr(self.L_z)]


def make_problem(name: str, out_dir: str, seed: int = 20261203) -> Problem:
    """Write one named synthetic configuration into out_dir and describe it.

    Named configurations (sizes as in the reference's measurement configs):
      slab1d            100-cell 1D slab, 1e-8 m, DM=2, 8 polar directions, gray band,
                        isothermal 301 / 299 K ends.
      square20k         2D square 1e-7 m, 2 x 100^2 triangles, DM=2, 8x8 angles (32
                        directions), 40 bands, left 301 K / right 299 K isothermal,
                        top/bottom diffuse.
      cube200k          3D cube 1e-8 m, 6 x 32^3 tetrahedra, DM=3, 4x4 (128 directions),
                        40 bands, x faces isothermal, y faces mirror (32), z faces mirror (33).
      square100k        2D square 1e-4 m (diffusive), 2 x 224^2 triangles, 32 directions, 20 bands.
      cube1m            3D cube 1e-6 m, 6 x 55^3 tetrahedra minus a cylindrical pore of
                        radius 0.2 (diffuse wall), 128 directions, 40 bands.
      squarepores       2D square 1e-6 m, 2 x 48^2 triangles minus three circular pores
                        (diffuse walls, entity 4), 32 directions, 8 bands.
      square<N>_b<B>    2D square 1e-7 m with 2 N^2 triangles and B bands (small parity cases).
      cube<N>_b<B>      3D cube 1e-8 m with 6 N^3 tetrahedra and B bands.
      nondelaunay<N>_b<B>  as square<N>_b<B> without the Delaunay edge flips.
    """
    os.makedirs(out_dir, exist_ok=True)
    geo = os.path.join(out_dir, f"{name}.mphtxt")
    band_file = os.path.join(out_dir, f"{name}.band.dat")
    bc_file = os.path.join(out_dir, f"{name}.bc.dat")

    def square(n, n_band, side, bc_rows=None, delaunay=True, pores=()):
        write_mphtxt(geo, square_mesh(n, seed=seed, delaunay=delaunay, pores=pores))
        write_band_file(band_file, debye_bands(n_band))
        write_bc_file(bc_file, bc_rows or [(0, 1, 301.0), (1, 2, 300.0), (2, 1, 299.0), (3, 2, 300.0)])
        return Problem(name, geo, band_file, bc_file, 2, 8, 8, 300.0, 1000, side, side, 0.0)

    def cube(n, n_band, side, pore=0.0, nt=4, np_=4):
        write_mphtxt(geo, cube_mesh(n, seed=seed, pore_radius=pore))
        write_band_file(band_file, debye_bands(n_band))
        rows = [(0, 1, 301.0), (5, 1, 299.0), (1, 32, 300.0), (4, 32, 300.0), (2, 33, 300.0), (3, 33, 300.0)]
        if pore > 0:
            rows.append((6, 2, 300.0))
        write_bc_file(bc_file, rows)
        return Problem(name, geo, band_file, bc_file, 3, nt, np_, 300.0, 1000, side, side, side)

    if name == "slab1d":
        write_band_file(band_file, dict(vg=[6400.0], tau=[4e-11], C=[C_TOTAL], Lr=[1.0]))
        write_bc_file(bc_file, [(0, 1, 301.0), (1, 1, 299.0)])
        return Problem(name, "100", band_file, bc_file, 2, 8, 1, 300.0, 1000, 1e-8, 0.0, 0.0)
    if name == "square20k":
        return square(100, 40, 1e-7)
    if name == "cube200k":
        return cube(32, 40, 1e-8)
    if name == "square100k":
        p = square(224, 20, 1e-4)
        p.max_iter = 100000
        return p
    if name == "cube1m":
        return cube(55, 40, 1e-6, pore=0.2)
    if name == "squarepores":
        # three pores with diffuse walls in a 1e-6 m square (the moderately
        # diffusive regime), 2 x 48^2 triangles before the pores, 8 bands
        pores = ((0.3, 0.3, 0.12), (0.68, 0.42, 0.15), (0.4, 0.75, 0.1))
        return square(48, 8, 1e-6, pores=pores,
                      bc_rows=[(0, 1, 301.0), (1, 2, 300.0), (2, 1, 299.0), (3, 2, 300.0), (4, 2, 300.0)])
    if name.startswith("nondelaunay") and "_b" in name:
        n, b = name[len("nondelaunay"):].split("_b")
        return square(int(n), int(b), 1e-7, delaunay=False)
    if name.startswith("square") and "_b" in name:
        n, b = name[len("square"):].split("_b")
        return square(int(n), int(b), 1e-7)
    if name.startswith("cube") and "_b" in name:
        n, b = name[len("cube"):].split("_b")
        return cube(int(n), int(b), 1e-8)
    raise ValueError(f"unknown synthetic configuration {name!r}")


if __name__ == "__main__":
    # python -m staticbtesolver_gb300.synth NAME OUT_DIR: write the files, print the BTEcmd flags.
    import sys

    if len(sys.argv) != 3:
        sys.exit("usage: python -m staticbtesolver_gb300.synth NAME OUT_DIR")
    prob = make_problem(sys.argv[1], sys.argv[2])
    print(" ".join(prob.btecmd_flags()))
