"""Synthetic cavity cases in meso-lts's own file formats.

Writes Gambit neutral meshes (.neu), discrete-velocity files (.dvs) and case
files that both the reference solver and this library read unchanged:

  * quad_cavity      N x N uniform quads on the unit square, marks lid / wall
  * tri_cavity       seeded Delaunay triangulation of jittered points (about
                     2 (n-1)^2 triangles), corner triangles re-triangulated so
                     every cell has two non-collinear neighbours (the 2x2
                     least-squares matrix of src/mesh/geom.cpp:187-190 would be
                     singular otherwise)
  * gauss_hermite    `Gauss-Hermite` abscissae/weights (hermgauss)
  * half_range_gh    `half-range-Gauss-Hermite` set by the Golub-Welsch method on
                     the half-range Hermite recurrence (the construction of the
                     reference's files/scripts/hGH.py, eigenvalues taken real)
  * newton_cotes     `Newton-Cotes` parameter file
  * sparse_d2q9      `Sparse` 3x3 Gauss-Hermite set for the Shakhov solver

and the workloads the benchmark configurations name (`config1` ... `config4`).
Kn -> viscosity follows files/scripts/para_nodim.py:24-31.
"""
from __future__ import annotations

import math
import os

import numpy as np

# --------------------------------------------------------------------------- meshes


def _write_neu(path: str, nodes: np.ndarray, cells: list[list[int]], cell_type: int,
               bcs: dict[str, list[tuple[int, int, int]]], group: str = "fluid") -> None:
    """nodes [N,2] or [N,3]; cells 0-based node lists; bcs name -> [(cell0, elemtype, face1based)]."""
    n_nodes, n_cells = len(nodes), len(cells)
    ndim = int(np.asarray(nodes).shape[1])
    with open(path, "w") as f:
        f.write("        CONTROL INFO 2.4.6\n** GAMBIT NEUTRAL FILE\nmeso-gb300 synthetic cavity\n")
        f.write("PROGRAM:  meso-gb300 cases.py     VERSION:  1.0\n01 Jan 2026 00:00:00\n")
        f.write("     NUMNP     NELEM     NGRPS    NBSETS     NDFCD     NDFVL\n")
        f.write(f"{n_nodes:10d}{n_cells:10d}{1:10d}{len(bcs):10d}{ndim:10d}{ndim:10d}\nENDOFSECTION\n")
        f.write("   NODAL COORDINATES 2.4.6\n")
        for i, xyz in enumerate(nodes):
            f.write(f"{i + 1:10d}" + "".join(f"{v:20.11E}" for v in xyz) + "\n")
        f.write("ENDOFSECTION\n      ELEMENTS/CELLS 2.4.6\n")
        for i, c in enumerate(cells):
            f.write(f"{i + 1:8d} {cell_type:2d} {len(c):2d} " + " ".join(f"{v + 1:8d}" for v in c) + "\n")
        f.write("ENDOFSECTION\n       ELEMENT GROUP 2.4.6\n")
        f.write(f"GROUP:          1 ELEMENTS:{n_cells:11d} MATERIAL:          2 NFLAGS:          1\n")
        f.write(f"{group:>32s}\n       0\n")
        for i in range(0, n_cells, 10):
            f.write("".join(f"{k + 1:8d}" for k in range(i, min(i + 10, n_cells))) + "\n")
        f.write("ENDOFSECTION\n")
        for name, ents in bcs.items():
            f.write(" BOUNDARY CONDITIONS 2.4.6\n")
            f.write(f"{name:>32s}{1:8d}{len(ents):8d}{0:8d}{6:8d}\n")
            for c, t, fc in ents:
                f.write(f"{c + 1:10d}{t:5d}{fc:5d}\n")
            f.write("ENDOFSECTION\n")


def quad_cavity(path: str, n: int, length: float = 1.0) -> dict:
    """n x n quads; local faces 1..4 = bottom, right, top, left (object.cpp:23)."""
    h = length / n
    xs = np.arange(n + 1) * h
    xs[-1] = length
    X, Y = np.meshgrid(xs, xs)
    nodes = np.stack([X.ravel(), Y.ravel()], 1)
    nid = lambda i, j: j * (n + 1) + i
    cells, lid, wall = [], [], []
    for j in range(n):
        for i in range(n):
            c = len(cells)
            cells.append([nid(i, j), nid(i + 1, j), nid(i + 1, j + 1), nid(i, j + 1)])
            if j == n - 1:
                lid.append((c, 2, 3))
            if j == 0:
                wall.append((c, 2, 1))
            if i == n - 1:
                wall.append((c, 2, 2))
            if i == 0:
                wall.append((c, 2, 4))
    _write_neu(path, nodes, cells, 2, {"lid": lid, "wall": wall})
    return dict(ncell=n * n, min_cell_size=2.0 * math.sqrt(h * h / math.pi))


def quad_channel(path: str, nx: int, ny: int, lx: float = 2.0, ly: float = 1.0) -> dict:
    """nx x ny quads on [0,lx]x[0,ly]; marks inlet (x=0), outlet (x=lx), bottom (y=0), top (y=ly)."""
    hx, hy = lx / nx, ly / ny
    xs = np.arange(nx + 1) * hx
    ys = np.arange(ny + 1) * hy
    xs[-1], ys[-1] = lx, ly
    X, Y = np.meshgrid(xs, ys)
    nodes = np.stack([X.ravel(), Y.ravel()], 1)
    nid = lambda i, j: j * (nx + 1) + i
    cells = []
    bc = {"inlet": [], "outlet": [], "bottom": [], "top": []}
    for j in range(ny):
        for i in range(nx):
            c = len(cells)
            cells.append([nid(i, j), nid(i + 1, j), nid(i + 1, j + 1), nid(i, j + 1)])
            if j == ny - 1:
                bc["top"].append((c, 2, 3))
            if j == 0:
                bc["bottom"].append((c, 2, 1))
            if i == nx - 1:
                bc["outlet"].append((c, 2, 2))
            if i == 0:
                bc["inlet"].append((c, 2, 4))
    _write_neu(path, nodes, cells, 2, bc)
    return dict(ncell=nx * ny, min_cell_size=2.0 * math.sqrt(hx * hy / math.pi))


def jquad_cavity(path: str, n: int, seed: int = 0, jitter: float = 0.25) -> dict:
    """n x n unstructured quadrilaterals: lattice nodes moved by up to `jitter` h (wall nodes slide along
    their wall, corners fixed), seeded; every cell is a convex quad with an over-determined gradient."""
    rng = np.random.default_rng(seed)
    h = 1.0 / n
    P = np.zeros((n + 1, n + 1, 2))
    for j in range(n + 1):
        for i in range(n + 1):
            x, y = i * h, j * h
            if 0 < i < n:
                x += rng.uniform(-jitter, jitter) * h
            if 0 < j < n:
                y += rng.uniform(-jitter, jitter) * h
            P[j, i] = (x if i < n else 1.0, y if j < n else 1.0)
    nodes = P.reshape(-1, 2)
    nid = lambda i, j: j * (n + 1) + i
    cells, lid, wall = [], [], []
    amin = 1e300
    for j in range(n):
        for i in range(n):
            c = len(cells)
            q = [nid(i, j), nid(i + 1, j), nid(i + 1, j + 1), nid(i, j + 1)]
            cells.append(q)
            a1, a2 = _tri_area(nodes, [q[0], q[1], q[2]]), _tri_area(nodes, [q[0], q[2], q[3]])
            b1, b2 = _tri_area(nodes, [q[0], q[1], q[3]]), _tri_area(nodes, [q[1], q[2], q[3]])
            assert min(a1, a2, b1, b2) > 0, "non-convex quad"
            amin = min(amin, a1 + a2)
            if j == n - 1:
                lid.append((c, 2, 3))
            if j == 0:
                wall.append((c, 2, 1))
            if i == n - 1:
                wall.append((c, 2, 2))
            if i == 0:
                wall.append((c, 2, 4))
    _write_neu(path, nodes, cells, 2, {"lid": lid, "wall": wall})
    return dict(ncell=n * n, min_cell_size=2.0 * math.sqrt(amin / math.pi))


def brick_cavity(path: str, n: int, length: float = 1.0) -> dict:
    """n^3 bricks on the unit cube (gambit element type 4, nodes in gambit order: x fastest, then y,
    then z).  Local faces 1..6 = y-, x+, y+, x-, z-, z+ (object.cpp:32).  Marks: lid (y = 1, the moving
    wall) and wall (the other five sides)."""
    h = length / n
    xs = np.arange(n + 1) * h
    xs[-1] = length
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    nodes = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    nid = lambda i, j, k: (k * (n + 1) + j) * (n + 1) + i
    cells, lid, wall = [], [], []
    for k in range(n):
        for j in range(n):
            for i in range(n):
                c = len(cells)
                cells.append([nid(i, j, k), nid(i + 1, j, k), nid(i, j + 1, k), nid(i + 1, j + 1, k),
                              nid(i, j, k + 1), nid(i + 1, j, k + 1), nid(i, j + 1, k + 1), nid(i + 1, j + 1, k + 1)])
                if j == n - 1:
                    lid.append((c, 4, 3))
                if j == 0:
                    wall.append((c, 4, 1))
                if i == n - 1:
                    wall.append((c, 4, 2))
                if i == 0:
                    wall.append((c, 4, 4))
                if k == 0:
                    wall.append((c, 4, 5))
                if k == n - 1:
                    wall.append((c, 4, 6))
    _write_neu(path, nodes, cells, 4, {"lid": lid, "wall": wall})
    return dict(ncell=n ** 3, min_cell_size=2.0 * (3.0 * h ** 3 / (4.0 * math.pi)) ** (1.0 / 3.0))


def tetra_cavity(path: str, n: int, length: float = 1.0) -> dict:
    """n^3 cubes on the unit cube, each cut into six tetrahedra around its main diagonal (gambit element
    type 6).  Local faces of a tetrahedron {1,0,2}, {0,1,3}, {1,2,3}, {2,0,3} (object.cpp:34).  Tetrahedra
    with two faces on the boundary have two neighbours only (a singular 3x3 least-squares matrix,
    geom.cpp:193-210), so cases on this mesh turn the gradient off.  Marks: lid (y = 1) and wall."""
    h = length / n
    xs = np.arange(n + 1) * h
    xs[-1] = length
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    nodes = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    nid = lambda i, j, k: (k * (n + 1) + j) * (n + 1) + i
    faces_local = ((1, 0, 2), (0, 1, 3), (1, 2, 3), (2, 0, 3))
    cells = []
    for k in range(n):
        for j in range(n):
            for i in range(n):
                v = lambda a, b, c: nid(i + a, j + b, k + c)
                d0, d1 = v(0, 0, 0), v(1, 1, 1)
                for path3 in ((v(1, 0, 0), v(1, 1, 0)), (v(1, 0, 0), v(1, 0, 1)), (v(0, 1, 0), v(1, 1, 0)),
                              (v(0, 1, 0), v(0, 1, 1)), (v(0, 0, 1), v(1, 0, 1)), (v(0, 0, 1), v(0, 1, 1))):
                    t = [d0, path3[0], path3[1], d1]
                    a, b, c, d = (nodes[x] for x in t)
                    if np.dot(np.cross(b - a, c - a), d - a) < 0.0:
                        t = [t[0], t[2], t[1], t[3]]
                    cells.append(t)
    fmap = {}
    for ci, t in enumerate(cells):
        for fi, loc in enumerate(faces_local):
            fmap.setdefault(tuple(sorted(t[x] for x in loc)), []).append((ci, fi))
    lid, wall = [], []
    for key, ents in fmap.items():
        if len(ents) != 1:
            continue
        ci, fi = ents[0]
        pts = nodes[list(key)]
        (lid if np.all(pts[:, 1] == length) else wall).append((ci, 6, fi + 1))
    _write_neu(path, nodes, cells, 6, {"lid": lid, "wall": wall})
    vol = h ** 3 / 6.0
    return dict(ncell=len(cells), min_cell_size=2.0 * (3.0 * vol / (4.0 * math.pi)) ** (1.0 / 3.0))


def _tri_area(p, t):
    a, b, c = p[t[0]], p[t[1]], p[t[2]]
    return 0.5 * ((b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0]))


def tri_cavity(path: str, n: int = 64, seed: int = 0, jitter: float = 0.3) -> dict:
    """Delaunay triangles of an n x n jittered point grid on the unit square."""
    from scipy.spatial import Delaunay

    rng = np.random.default_rng(seed)
    h = 1.0 / (n - 1)
    pts = []
    for j in range(n):
        for i in range(n):
            x, y = i * h, j * h
            on_x = i in (0, n - 1)
            on_y = j in (0, n - 1)
            if not on_x:
                x += rng.uniform(-jitter, jitter) * h
            if not on_y:
                y += rng.uniform(-jitter, jitter) * h
            pts.append((min(max(x, 0.0), 1.0), min(max(y, 0.0), 1.0)))
    p = np.array(pts)
    tri = [list(t) for t in Delaunay(p).simplices]
    on_bnd = lambda k: p[k, 0] in (0.0, 1.0) or p[k, 1] in (0.0, 1.0)

    def edge_map(tris):
        em = {}
        for ti, t in enumerate(tris):
            for a, b in ((t[0], t[1]), (t[1], t[2]), (t[2], t[0])):
                em.setdefault((min(a, b), max(a, b)), []).append(ti)
        return em

    def is_bnd_edge(a, b):
        return (p[a, 0] == p[b, 0] and p[a, 0] in (0.0, 1.0)) or (p[a, 1] == p[b, 1] and p[a, 1] in (0.0, 1.0))

    # flip the interior edge of every triangle with two boundary edges
    for _ in range(4):
        em = edge_map(tri)
        changed = False
        for ti in range(len(tri)):
            t = tri[ti]
            edges = [(t[k], t[(k + 1) % 3]) for k in range(3)]
            bnd = [e for e in edges if len(em[(min(e), max(e))]) == 1]
            if len(bnd) < 2:
                continue
            inner = [e for e in edges if len(em[(min(e), max(e))]) == 2][0]
            a, b = inner
            corner = [v for v in t if v not in inner][0]
            tj = [x for x in em[(min(a, b), max(a, b))] if x != ti][0]
            d = [v for v in tri[tj] if v not in inner][0]
            tri[ti] = [corner, a, d]
            tri[tj] = [corner, d, b]
            changed = True
            em = edge_map(tri)
        if not changed:
            break
    # counter-clockwise orientation
    tri = [t if _tri_area(p, t) > 0 else [t[0], t[2], t[1]] for t in tri]
    em = edge_map(tri)
    for ti, t in enumerate(tri):
        nb = [x for k in range(3) for x in em[(min(t[k], t[(k + 1) % 3]), max(t[k], t[(k + 1) % 3]))] if x != ti]
        assert len(nb) >= 2, f"triangle {ti} has {len(nb)} neighbours"
        c0 = p[t].mean(0)
        d = np.array([p[tri[x]].mean(0) - c0 for x in nb])
        assert abs(np.linalg.det(d.T @ d)) > 1e-14, f"triangle {ti} has collinear neighbours"
        assert _tri_area(p, t) > 0
    lid, wall = [], []
    for ti, t in enumerate(tri):
        for k in range(3):
            a, b = t[k], t[(k + 1) % 3]
            if len(em[(min(a, b), max(a, b))]) == 1:
                assert is_bnd_edge(a, b)
                ent = (ti, 3, k + 1)  # local faces of a triangle: {0,1},{1,2},{2,0}
                (lid if p[a, 1] == 1.0 and p[b, 1] == 1.0 else wall).append(ent)
    _write_neu(path, p, tri, 3, {"lid": lid, "wall": wall})
    amin = min(_tri_area(p, t) for t in tri)
    return dict(ncell=len(tri), min_cell_size=2.0 * math.sqrt(amin / math.pi))


def mixed_cavity(path: str, n: int = 64, seed: int = 0, jitter: float = 0.3) -> dict:
    """Unstructured cavity: a one-cell quad layer along the walls, seeded Delaunay triangles inside.

    Nodes sit on an n x n lattice of spacing h = 1/(n-1); lattice nodes at
    least two rows from the walls are jittered by up to `jitter` h.  Cells
    touching a wall are h x h quads (three face neighbours, as in the shipped
    cavity.neu), the inner square [h, 1-h]^2 is the Delaunay triangulation of
    its nodes, so every triangle has three neighbours.  (On an all-triangle
    wall row the reference scheme grows an unstable mode: a boundary triangle
    has two neighbours and its least-squares gradient is exactly determined.)
    """
    from scipy.spatial import Delaunay

    rng = np.random.default_rng(seed)
    h = 1.0 / (n - 1)
    idx = {}
    pts = []
    for j in range(n):
        for i in range(n):
            layer = min(i, j, n - 1 - i, n - 1 - j)
            x, y = i * h, j * h
            if i == n - 1:
                x = 1.0
            if j == n - 1:
                y = 1.0
            if layer >= 2:
                x += rng.uniform(-jitter, jitter) * h
                y += rng.uniform(-jitter, jitter) * h
            idx[(i, j)] = len(pts)
            pts.append((x, y))
    p = np.array(pts)
    cells, types, lid, wall = [], [], [], []
    for j in range(n - 1):
        for i in range(n - 1):
            if not (i == 0 or j == 0 or i == n - 2 or j == n - 2):
                continue
            c = len(cells)
            cells.append([idx[(i, j)], idx[(i + 1, j)], idx[(i + 1, j + 1)], idx[(i, j + 1)]])
            types.append(2)
            if j == n - 2:
                lid.append((c, 2, 3))
            if j == 0:
                wall.append((c, 2, 1))
            if i == n - 2:
                wall.append((c, 2, 2))
            if i == 0:
                wall.append((c, 2, 4))
    inner = [idx[(i, j)] for j in range(1, n - 1) for i in range(1, n - 1)]
    tri = Delaunay(p[inner])
    assert len(np.unique(tri.simplices)) == len(inner), "Delaunay dropped a node"
    for t in tri.simplices:
        t = [inner[k] for k in t]
        if _tri_area(p, t) < 0:
            t = [t[0], t[2], t[1]]
        assert _tri_area(p, t) > 1e-14
        cells.append(t)
        types.append(3)
    # conformity: every edge is shared by two cells, except the outer walls
    em = {}
    for ci, c in enumerate(cells):
        for k in range(len(c)):
            a, b = c[k], c[(k + 1) % len(c)]
            em.setdefault((min(a, b), max(a, b)), []).append(ci)
    for (a, b), cs in em.items():
        on_wall = (p[a, 0] == p[b, 0] and p[a, 0] in (0.0, 1.0)) or (p[a, 1] == p[b, 1] and p[a, 1] in (0.0, 1.0))
        assert len(cs) == (1 if on_wall else 2), f"non-conforming edge {(a, b)}"
    _write_neu_mixed(path, p, cells, types, {"lid": lid, "wall": wall})
    amin = min(abs(_tri_area(p, c)) if len(c) == 3 else h * h for c in cells)
    return dict(ncell=len(cells), min_cell_size=2.0 * math.sqrt(amin / math.pi))


def _write_neu_mixed(path, nodes, cells, types, bcs):
    """_write_neu for meshes whose cells have different shapes (type per element)."""
    tmp = path + ".tmp"
    _write_neu(tmp, nodes, cells, 0, bcs)
    with open(tmp) as f:
        lines = f.read().split("\n")
    out, in_cells, k = [], False, 0
    for line in lines:
        if line.strip().startswith("ELEMENTS/CELLS"):
            in_cells = True
        elif line.strip() == "ENDOFSECTION":
            in_cells = False
        elif in_cells:
            parts = line.split()
            line = f"{int(parts[0]):8d} {types[k]:2d} {len(parts) - 3:2d} " + " ".join(f"{int(v):8d}" for v in parts[3:])
            k += 1
        out.append(line)
    with open(path, "w") as f:
        f.write("\n".join(out))
    os.remove(tmp)


# --------------------------------------------------------------------------- velocity sets


def gauss_hermite(path: str, n: int) -> np.ndarray:
    x, w = np.polynomial.hermite.hermgauss(n)
    with open(path, "w") as f:
        f.write("Gauss-Hermite\n")
        for a, b in zip(x, w):
            f.write(f"{a:.18f} {b:.18f}\n")
    return x


def _half_range_nodes(m: int):
    """Nodes/weights on [0, inf) for weight exp(-x^2) (m nodes): recurrence + Golub-Welsch."""
    a = np.zeros(m)
    b = np.zeros(m)
    a[0] = 1.0 / math.sqrt(math.pi)
    if m > 1:
        a[1] = 2.0 / math.sqrt(math.pi) / (math.pi - 2.0)
        b[1] = a[0] / (a[0] + a[1]) / 2.0
    for i in range(2, m):
        b[i] = (i - 1) + 0.5 - b[i - 1] - a[i - 1] ** 2
        a[i] = (i * i / 4.0 / b[i] - b[i - 1] - 0.5) / a[i - 1] - a[i - 1]
    J = np.diag(a) + np.diag(np.sqrt(b[1:]), 1) + np.diag(np.sqrt(b[1:]), -1)
    v, V = np.linalg.eigh(J)
    w = V[0, :] ** 2 * math.sqrt(math.pi) / 2.0
    order = np.argsort(v)
    return v[order], w[order]


def half_range_gh(path: str, n2: int) -> np.ndarray:
    """n2 (even) nodes on the real line: mirrored half-range sets, weights times exp(x^2)."""
    v, w = _half_range_nodes(n2 // 2)
    xs = np.concatenate([-v[::-1], v])
    ws = np.concatenate([w[::-1], w]) * np.exp(xs ** 2)
    with open(path, "w") as f:
        f.write("half-range-Gauss-Hermite\n")
        for a, b in zip(xs, ws):
            f.write(f"{a:18.15e} {b:18.15e}\n")
    return xs


def newton_cotes(path: str, order: int = 1, mount: int = 100, scale: float = 5.0) -> None:
    with open(path, "w") as f:
        f.write(f"Newton-Cotes\n{order} {mount} {scale!r}\n")


def sparse_d2q9(path: str, RT: float = 0.5) -> None:
    """3x3 Gauss-Hermite velocities with weights 2RT w_i w_j exp(x_i^2 + x_j^2)."""
    x, w = np.polynomial.hermite.hermgauss(3)
    s = math.sqrt(2.0 * RT)
    with open(path, "w") as f:
        f.write("Sparse\n")
        for j in range(3):
            for i in range(3):
                W = 2.0 * RT * w[i] * w[j] * math.exp(x[i] ** 2 + x[j] ** 2)
                f.write(f"{float(s * x[i])!r} {float(s * x[j])!r} 0.0 {float(W)!r}\n")


# --------------------------------------------------------------------------- case files


def viscosity_from_kn(kn: float, rho: float = 1.0, R: float = 0.5, T: float = 1.0, omega: float = 0.5,
                      L: float = 1.0) -> float:
    mfp = L * kn
    return (15.0 * rho * mfp) / (2.0 * (5.0 - 2.0 * omega) * (7.0 - 2.0 * omega)) * math.sqrt(2.0 * math.pi * R * T)


def write_case(path: str, settings: dict, groups: list[dict], marks: list[dict]) -> str:
    def fmt(v):
        if isinstance(v, bool):
            return "True" if v else "False"
        if isinstance(v, float):
            return repr(v)
        return str(v)

    with open(path, "w") as f:
        f.write("[settings]\n")
        for k, v in settings.items():
            f.write(f"{k:<20s}{fmt(v)}\n")
        for g in groups:
            f.write("\n[group]\n")
            for k, v in g.items():
                f.write(f"{k:<16s}{v}\n")
        for m in marks:
            f.write("\n[mark]\n")
            for k, v in m.items():
                f.write(f"{k:<16s}{v}\n")
    return path


def _vec(u, v=0.0, w=0.0):
    return f"fixedValue  vector  {u!r} {v!r} {w!r}"


def _sc(x):
    return f"fixedValue  scalar  {float(x)!r}"


def bgk_cavity(d: str, n: int = 64, steps: int = 2000, lid: float = 0.1, solver: str = "cdugks@incompressible",
               name: str = "bgk", gradient: bool = True, dt: float = 2.5e-3) -> str:
    """Config 1 shape: incompressible BGK cavity on n x n quads with D2Q9 (gh-3)."""
    os.makedirs(d, exist_ok=True)
    quad_cavity(os.path.join(d, "mesh.neu"), n)
    gauss_hermite(os.path.join(d, "gh-3.dvs"), 3)
    settings = {"solver": solver, "case-name": name, "mesh-file": "mesh.neu", "dvs-file": "gh-3.dvs",
                "dvs-type": "Gauss-Hermite", "write-interval": 1000, "max-step": steps, "Re": 400.0,
                "Ma": 0.1414213562373095, "gradient-switch": gradient, "timeStep": dt, "gas-constant": 0.5,
                "ref-density": 1.0, "ref-length": 1.0, "ref-temperature": 1.0, "CFL": 0.8}
    return write_case(os.path.join(d, "case.txt"), settings, [{"name": "fluid", "density": _sc(1.0)}],
                      [{"name": "lid", "type": "wall", "velocity": _vec(lid)}, {"name": "wall", "type": "wall"}])


def shakhov_cavity(d: str, mesh: str = "quad", n: int = 61, dvs: str = "hgh", nv1d: int = 28, kn: float = 0.075,
                   lid: float = 0.15, steps: int = 500, seed: int = 0, name: str = "shakhov",
                   cfl: float = 0.8, precision: str = "fp64", extra_marks: list | None = None,
                   gradient: bool = True, limiter: bool = False) -> str:
    """Shakhov CDUGKS cavity (configs 2-4): quad or Delaunay mesh; hGH, NC or D2Q9 velocities."""
    os.makedirs(d, exist_ok=True)
    meshf = os.path.join(d, "mesh.neu")
    if mesh == "quad":
        info = quad_cavity(meshf, n)
    elif mesh == "jquad":
        info = jquad_cavity(meshf, n, seed)
    elif mesh == "mixed":
        info = mixed_cavity(meshf, n, seed)
    else:
        info = tri_cavity(meshf, n, seed)
    RT = 0.5
    if dvs == "hgh":
        xs = half_range_gh(os.path.join(d, "v.dvs"), nv1d)
        vmax = math.sqrt(2.0) * math.sqrt(2 * RT) * float(np.max(np.abs(xs)))
        dvs_type = "half-range-Gauss-Hermite"
    elif dvs == "nc":
        newton_cotes(os.path.join(d, "v.dvs"), 1, nv1d - 1, 5.0)
        vmax = 5.0 * math.sqrt(2.0)
        dvs_type = "Newton-Cotes"
    elif dvs == "d2q9":
        sparse_d2q9(os.path.join(d, "v.dvs"), RT)
        vmax = math.sqrt(2.0) * math.sqrt(2 * RT) * math.sqrt(1.5)
        dvs_type = "Sparse"
    else:
        raise ValueError(dvs)
    dt = cfl * info["min_cell_size"] / vmax
    mu = viscosity_from_kn(kn)
    settings = {"solver": "cdugks@shakhov", "case-name": name, "mesh-file": "mesh.neu", "dvs-file": "v.dvs",
                "dvs-type": dvs_type, "write-interval": 1000, "max-step": steps, "Pr": 0.6666666666666667,
                "gradient-switch": gradient, "limiter-switch": limiter, "output-np": False, "timeStep": dt,
                "gas-constant": 0.5, "gas-k": 0, "ref-density": 1.0, "ref-length": 1.0, "ref-temperature": 1.0,
                "ref-viscosity": mu, "vhs-index": 0.5, "gpu-precision": precision}
    marks = [{"name": "lid", "type": "wall", "velocity": _vec(lid), "temperature": _sc(1.0)},
             {"name": "wall", "type": "wall", "velocity": _vec(0.0), "temperature": _sc(1.0)}]
    if extra_marks:
        names = {m["name"] for m in extra_marks}
        marks = [m for m in marks if m["name"] not in names] + extra_marks
    return write_case(os.path.join(d, "case.txt"), settings,
                      [{"name": "fluid", "density": _sc(1.0), "temperature": _sc(1.0)}], marks)


# The four benchmark workloads (sizes from the configuration list they serve).
def config1(d: str, steps: int = 2000) -> str:
    """Incompressible BGK cavity, 64x64 quads, D2Q9, Re 400, lid 0.1, dt 2.5e-3."""
    return bgk_cavity(d, 64, steps)


def config2(d: str, steps: int = 500, precision: str = "fp32", n: int = 88, nv1d: int = 101) -> str:
    """Rarefied Shakhov cavity: 7744 unstructured (jittered) quadrilaterals, Newton-Cotes 101x101 on [-5,5]^2,
    Kn 1, lid 0.15.  (On Delaunay-triangle meshes of this size the reference scheme, whose least-squares
    reconstruction is unlimited, grows an unstable mode before 500 steps; jittered quads keep the
    unstructured geometry with over-determined gradients.)"""
    return shakhov_cavity(d, "jquad", n, "nc", nv1d, 1.0, 0.15, steps, seed=0, name="config2", precision=precision)


def config3(d: str, steps: int = 5000, precision: str = "fp32") -> str:
    """Transitional Shakhov cavity: 61x61 quads, half-range GH 28x28, Kn 0.075, lid 0.15, CFL 0.5 (at CFL
    0.8 the reference scheme blows up at step 140 on this cavity; its own Kn 0.075 case runs at 0.66)."""
    return shakhov_cavity(d, "quad", 61, "hgh", 28, 0.075, 0.15, steps, name="config3", precision=precision,
                          cfl=0.5)


def config4_instances(seed: int = 1, count: int = 64) -> list[dict]:
    """Batch draws: side in {32,48,64,96,128}, log10 Kn ~ U(-2,0), DVS in {D2Q9, hGH 28^2, NC 101^2}, lid ~ U(.05,.15)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        side = int(rng.choice([32, 48, 64, 96, 128]))
        kn = float(10.0 ** rng.uniform(-2.0, 0.0))
        dvs = ["d2q9", "hgh", "nc"][int(rng.integers(0, 3))]
        lid = float(rng.uniform(0.05, 0.15))
        out.append(dict(index=i, side=side, kn=kn, dvs=dvs, lid=lid))
    return out


def config4_case(d: str, inst: dict, steps: int = 500, precision: str = "fp32") -> str:
    nv1d = {"d2q9": 3, "hgh": 28, "nc": 101}[inst["dvs"]]
    # CFL 0.5 (the reference's shipped Kn 0.075 case runs at 0.66): at 0.8 the scheme is unstable on
    # some of these cavities over a few hundred steps
    return shakhov_cavity(d, "quad", inst["side"], inst["dvs"], nv1d, inst["kn"], inst["lid"], steps,
                          name=f"inst{inst['index']}", precision=precision, cfl=0.5)


def config5_requests(seed: int = 2, count: int = 200, rate: float = 20.0,
                     sides=(16, 24, 32), dvs_kinds=("hgh", "nc")) -> list[dict]:
    """Served stream: Poisson arrivals (mean `rate` per second) of cavity solves drawn like config 4
    (log10 Kn ~ U(-2,0), lid ~ U(.05,.15), DVS kind uniform) on the given mesh sides.  The velocity
    sets are hGH 28x28 and NC 21x21: the reference scheme is unstable on the coarser hGH and D2Q9
    sets above Kn ~ 0.1, and a request that blows up never converges."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(count):
        t += float(rng.exponential(1.0 / rate))
        side = int(rng.choice(list(sides)))
        kn = float(10.0 ** rng.uniform(-2.0, 0.0))
        dvs = dvs_kinds[int(rng.integers(0, len(dvs_kinds)))]
        lid = float(rng.uniform(0.05, 0.15))
        out.append(dict(index=i, arrival=t, side=side, kn=kn, dvs=dvs, lid=lid))
    return out


def config5_case(d: str, req: dict, max_step: int = 4000, nc_points: int = 21) -> str:
    """One served request's case: NC nc_points^2 (21 in the scaled stream, 101 in the stream drawn from
    the batch workload's distribution), hGH 28^2 or D2Q9; CFL 0.5."""
    nv1d = {"d2q9": 3, "hgh": 28, "nc": nc_points}[req["dvs"]]
    return shakhov_cavity(d, "quad", req["side"], req["dvs"], nv1d, req["kn"], req["lid"], max_step,
                          name=f"req{req['index']}", precision="fp32", cfl=0.5)


def shakhov_cavity3d(d: str, mesh: str = "brick", n: int = 4, nv1d: int = 9, kn: float = 0.5, lid: float = 0.15,
                     steps: int = 20, cfl: float = 0.8, name: str = "cav3d", gradient: bool = True) -> str:
    """3-D Shakhov cavity (brick or tetra mesh of n^3 cubes), Newton-Cotes nv1d^3 velocities on [-4, 4]^3
    (the reference's 3-D Gauss-Hermite weights are wrong, dvs_generator.cpp:59,133; its Newton-Cotes set is
    not), diffuse walls, lid moving along x."""
    os.makedirs(d, exist_ok=True)
    meshf = os.path.join(d, "mesh.neu")
    info = brick_cavity(meshf, n) if mesh == "brick" else tetra_cavity(meshf, n)
    newton_cotes(os.path.join(d, "v.dvs"), 1, nv1d - 1, 4.0)
    dt = cfl * info["min_cell_size"] / (4.0 * math.sqrt(3.0))
    settings = {"solver": "cdugks@shakhov", "case-name": name, "mesh-file": "mesh.neu", "dvs-file": "v.dvs",
                "dvs-type": "Newton-Cotes", "write-interval": 1000, "max-step": steps, "Pr": 0.6666666666666667,
                "gradient-switch": gradient, "limiter-switch": False, "output-np": False, "timeStep": dt,
                "gas-constant": 0.5, "gas-k": 0, "ref-density": 1.0, "ref-length": 1.0, "ref-temperature": 1.0,
                "ref-viscosity": viscosity_from_kn(kn), "vhs-index": 0.5}
    marks = [{"name": "lid", "type": "wall", "velocity": _vec(lid), "temperature": _sc(1.0)},
             {"name": "wall", "type": "wall", "velocity": _vec(0.0), "temperature": _sc(1.0)}]
    return write_case(os.path.join(d, "case.txt"), settings,
                      [{"name": "fluid", "density": _sc(1.0), "temperature": _sc(1.0)}], marks)


def bgk_cavity3d(d: str, n: int = 4, steps: int = 40, lid: float = 0.1, name: str = "bgk3d") -> str:
    """3-D incompressible BGK cavity on n^3 bricks with the 27-velocity Gauss-Hermite set (gh-3)."""
    os.makedirs(d, exist_ok=True)
    brick_cavity(os.path.join(d, "mesh.neu"), n)
    gauss_hermite(os.path.join(d, "gh-3.dvs"), 3)
    settings = {"solver": "cdugks@incompressible", "case-name": name, "mesh-file": "mesh.neu", "dvs-file": "gh-3.dvs",
                "dvs-type": "Gauss-Hermite", "write-interval": 1000, "max-step": steps, "Re": 100.0,
                "Ma": 0.1414213562373095, "gradient-switch": True, "timeStep": 2.5e-3, "gas-constant": 0.5,
                "ref-density": 1.0, "ref-length": 1.0, "ref-temperature": 1.0}
    return write_case(os.path.join(d, "case.txt"), settings, [{"name": "fluid", "density": _sc(1.0)}],
                      [{"name": "lid", "type": "wall", "velocity": _vec(lid)}, {"name": "wall", "type": "wall"}])


def shakhov_channel(d: str, kind: str = "pressure", nx: int = 10, ny: int = 6, dvs: str = "hgh", nv1d: int = 8,
                    kn: float = 0.1, steps: int = 50, name: str = "channel", cfl: float = 0.5,
                    precision: str = "fp64") -> str:
    """Shakhov channel exercising the open and mirror boundaries of cdugks_shakhov.cpp:364-607.

    kind = "pressure":  pressure-inlet / pressure-outlet, symmetry bottom, slip-wall top
    kind = "farfield":  farfield-inlet / farfield-outlet, walls (zeroGradient balance T)
    kind = "freestream": freestream-inlet / farfield-outlet, symmetry bottom and top
    """
    os.makedirs(d, exist_ok=True)
    info = quad_channel(os.path.join(d, "mesh.neu"), nx, ny)
    RT = 0.5
    if dvs == "hgh":
        xs = half_range_gh(os.path.join(d, "v.dvs"), nv1d)
        vmax = math.sqrt(2.0) * math.sqrt(2 * RT) * float(np.max(np.abs(xs)))
        dvs_type = "half-range-Gauss-Hermite"
    else:
        newton_cotes(os.path.join(d, "v.dvs"), 1, nv1d - 1, 5.0)
        vmax = 5.0 * math.sqrt(2.0)
        dvs_type = "Newton-Cotes"
    dt = cfl * info["min_cell_size"] / vmax
    settings = {"solver": "cdugks@shakhov", "case-name": name, "mesh-file": "mesh.neu", "dvs-file": "v.dvs",
                "dvs-type": dvs_type, "max-step": steps, "Pr": 0.6666666666666667, "gradient-switch": True,
                "limiter-switch": False, "timeStep": dt, "gas-constant": 0.5, "gas-k": 0, "ref-density": 1.0,
                "ref-length": 1.0, "ref-temperature": 1.0, "ref-viscosity": viscosity_from_kn(kn),
                "vhs-index": 0.5, "gpu-precision": precision}
    if kind == "pressure":
        marks = [{"name": "inlet", "type": "pressure-inlet", "pressure": _sc(0.52), "temperature": _sc(1.0)},
                 {"name": "outlet", "type": "pressure-outlet", "pressure": _sc(0.48), "temperature": _sc(1.0)},
                 {"name": "bottom", "type": "symmetry", "direction": "fixedValue  objectType  1"},
                 {"name": "top", "type": "slip-wall", "direction": "fixedValue  objectType  1",
                  "velocity": _vec(0.0), "temperature": _sc(1.0), "slip-wall-alpha-u": _sc(0.7),
                  "slip-wall-alpha-T": _sc(0.4)}]
    elif kind == "farfield":
        marks = [{"name": "inlet", "type": "farfield-inlet", "density": _sc(1.02), "velocity": _vec(0.08),
                  "temperature": _sc(1.0)},
                 {"name": "outlet", "type": "farfield-outlet"},
                 # value line first, then zeroGradient: the balance reads T_cell (cdugks_shakhov.cpp:475-476)
                 # while the wall set reads the scalar (:533), as in a Patch given both lines
                 {"name": "bottom", "type": "wall", "velocity": _vec(0.0), "temperature": _sc(1.0),
                  "temperature ": "zeroGradient"},
                 {"name": "top", "type": "wall", "velocity": _vec(0.0), "temperature": _sc(1.0)}]
    elif kind == "freestream":
        marks = [{"name": "inlet", "type": "freestream-inlet", "pressure": _sc(0.51), "velocity": _vec(0.05),
                  "temperature": _sc(1.0)},
                 {"name": "outlet", "type": "farfield-outlet"},
                 {"name": "bottom", "type": "symmetry", "direction": "fixedValue  objectType  1"},
                 {"name": "top", "type": "symmetry", "direction": "fixedValue  objectType  1"}]
    else:
        raise ValueError(kind)
    return write_case(os.path.join(d, "case.txt"), settings,
                      [{"name": "fluid", "density": _sc(1.0), "temperature": _sc(1.0),
                        "velocity": _vec(0.0)}], marks)
