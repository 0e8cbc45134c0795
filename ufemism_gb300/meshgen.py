"""Seeded synthetic Delaunay meshes in UFEMISM's mesh conventions.

The reference builds its meshes by Ruppert refinement (mesh_creation_module.f90:354-485);
that machinery is set-up work, not part of the ice-velocity solve, so meshes here come
from seeded jittered points triangulated by Qhull (scipy.spatial.Delaunay). What the
solve relies on are the conventions of the reference's ``type_mesh``
(data_types_module.f90:216-345), which this module reproduces:

* the square domain's four corners are vertices 1..4, in the order SW, SE, NE, NW, with
  edge_index 6, 4, 2, 8 (mesh_creation_module.f90:1962-1963); apply_Neumann_boundary_AaAc
  treats vertices 1..4 as the corners (mesh_ArakawaC_module.f90:675, 706-721);
* edge_index codes 1..8 = N, NE, E, SE, S, SW, W, NW; 0 = free vertex;
* ``C(vi,:)`` lists the neighbours counter-clockwise, running from edge to edge for
  boundary vertices (data_types_module.f90: comment on ``C``);
* ``iTri(vi,k)`` is the triangle between ``C(vi,k)`` and ``C(vi,k+1)``, counter-clockwise;
  ``Tri(ti,:)`` is counter-clockwise.

All index arrays are returned 1-based and all 2-D arrays column-major (Fortran order), the
layout the reference's Fortran model hands to the C-ABI.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

NC_MEM = 16  # nconmax, configuration_module.f90:78

# edge_index codes (mesh_creation_module.f90:1898-1920)
EDGE_N, EDGE_NE, EDGE_E, EDGE_SE, EDGE_S, EDGE_SW, EDGE_W, EDGE_NW = 1, 2, 3, 4, 5, 6, 7, 8


@dataclass
class BaseMesh:
    """A triangulated square in UFEMISM conventions (1-based indices, Fortran order)."""

    xmin: float
    xmax: float
    ymin: float
    ymax: float
    V: np.ndarray          # (nV,2) float64, Fortran order
    nC: np.ndarray         # (nV,) int32
    C: np.ndarray          # (nV,NC_MEM) int32, 1-based, 0 = unused
    niTri: np.ndarray      # (nV,) int32
    iTri: np.ndarray       # (nV,NC_MEM) int32, 1-based
    Tri: np.ndarray        # (nTri,3) int32, 1-based, CCW
    edge_index: np.ndarray  # (nV,) int32

    @property
    def nV(self) -> int:
        return int(self.V.shape[0])

    @property
    def nTri(self) -> int:
        return int(self.Tri.shape[0])


def _quadtree_points(xmin, xmax, ymin, ymax, spacing_fn, rng):
    """Leaf cells of a quadtree refined until each cell is no larger than the target
    spacing anywhere inside it; one jittered point per leaf (jitter <= 0.25 * cell size).
    Returns (interior points, boundary points without the corners)."""
    L = xmax - xmin
    cx = np.array([0.5 * (xmin + xmax)])
    cy = np.array([0.5 * (ymin + ymax)])
    size = np.array([L])
    leaves_x, leaves_y, leaves_s = [], [], []
    for _ in range(40):
        if cx.size == 0:
            break
        hmin = spacing_fn(cx, cy, size)
        refine = size > hmin
        leaves_x.append(cx[~refine])
        leaves_y.append(cy[~refine])
        leaves_s.append(size[~refine])
        cx, cy, size = cx[refine], cy[refine], size[refine]
        q = 0.25 * size
        cx = np.concatenate([cx - q, cx + q, cx - q, cx + q])
        cy = np.concatenate([cy - q, cy - q, cy + q, cy + q])
        size = np.concatenate([size, size, size, size]) * 0.5
    lx = np.concatenate(leaves_x)
    ly = np.concatenate(leaves_y)
    ls = np.concatenate(leaves_s)
    # Deterministic leaf order before the random draw.
    order = np.lexsort((lx, ly, ls))
    lx, ly, ls = lx[order], ly[order], ls[order]
    jx = (rng.random(lx.size) - 0.5) * 0.5 * ls
    jy = (rng.random(lx.size) - 0.5) * 0.5 * ls
    interior = np.stack([lx + jx, ly + jy], axis=1)

    # Boundary points at the leaf-cell corners that lie on the domain edges.
    tol = 1e-9 * L
    half = 0.5 * ls
    on_s = np.abs(ly - half - ymin) < tol
    on_n = np.abs(ly + half - ymax) < tol
    on_w = np.abs(lx - half - xmin) < tol
    on_e = np.abs(lx + half - xmax) < tol
    xs = np.concatenate([lx[on_s] - half[on_s], lx[on_s] + half[on_s],
                         lx[on_n] - half[on_n], lx[on_n] + half[on_n]])
    ys = np.concatenate([np.full(2 * on_s.sum(), ymin), np.full(2 * on_n.sum(), ymax)])
    yw = np.concatenate([ly[on_w] - half[on_w], ly[on_w] + half[on_w],
                         ly[on_e] - half[on_e], ly[on_e] + half[on_e]])
    xw = np.concatenate([np.full(2 * on_w.sum(), xmin), np.full(2 * on_e.sum(), xmax)])
    bx = np.concatenate([xs, xw])
    by = np.concatenate([ys, yw])
    # Snap to the exact edge coordinates and drop the corners and duplicates.
    key = np.round(np.stack([bx, by], axis=1) / tol).astype(np.int64)
    _, uniq = np.unique(key, axis=0, return_index=True)
    bx, by = bx[np.sort(uniq)], by[np.sort(uniq)]
    is_corner = ((np.abs(bx - xmin) < tol) | (np.abs(bx - xmax) < tol)) & \
                ((np.abs(by - ymin) < tol) | (np.abs(by - ymax) < tol))
    bx, by = bx[~is_corner], by[~is_corner]
    return interior, np.stack([bx, by], axis=1)


def _morton_key(x, y, xmin, ymin, L, bits=16):
    xi = np.clip(((x - xmin) / L * (1 << bits)).astype(np.int64), 0, (1 << bits) - 1)
    yi = np.clip(((y - ymin) / L * (1 << bits)).astype(np.int64), 0, (1 << bits) - 1)
    key = np.zeros_like(xi)
    for b in range(bits):
        key |= ((xi >> b) & 1) << (2 * b)
        key |= ((yi >> b) & 1) << (2 * b + 1)
    return key


def triangulate_square(points_inner, points_boundary, xmin, xmax, ymin, ymax) -> BaseMesh:
    """Delaunay-triangulate corners + boundary + interior points and return the mesh in
    UFEMISM conventions."""
    from scipy.spatial import Delaunay

    L = max(xmax - xmin, ymax - ymin)
    corners = np.array([[xmin, ymin], [xmax, ymin], [xmax, ymax], [xmin, ymax]], dtype=np.float64)
    rest = np.concatenate([points_boundary, points_inner], axis=0)
    # Spatially coherent order for everything after the four corners.
    order = np.argsort(_morton_key(rest[:, 0], rest[:, 1], xmin, ymin, L), kind="stable")
    pts = np.concatenate([corners, rest[order]], axis=0)
    nV = pts.shape[0]

    tol = 1e-9 * L
    edge = np.zeros(nV, dtype=np.int32)
    on_n = np.abs(pts[:, 1] - ymax) < tol
    on_s = np.abs(pts[:, 1] - ymin) < tol
    on_e = np.abs(pts[:, 0] - xmax) < tol
    on_w = np.abs(pts[:, 0] - xmin) < tol
    edge[on_n] = EDGE_N
    edge[on_s] = EDGE_S
    edge[on_e] = EDGE_E
    edge[on_w] = EDGE_W
    edge[on_n & on_e] = EDGE_NE
    edge[on_s & on_e] = EDGE_SE
    edge[on_s & on_w] = EDGE_SW
    edge[on_n & on_w] = EDGE_NW
    # Exact coordinates on the edges.
    pts[on_n, 1] = ymax
    pts[on_s, 1] = ymin
    pts[on_e, 0] = xmax
    pts[on_w, 0] = xmin

    tri = Delaunay(pts, qhull_options="Qbb Qc Qz Q12 Qt")
    if getattr(tri, "coplanar", np.zeros((0, 3))).shape[0] != 0:
        raise RuntimeError("triangulation dropped points")
    T = tri.simplices.astype(np.int64)
    # Orient counter-clockwise and drop zero-area triangles along the hull.
    p0, p1, p2 = pts[T[:, 0]], pts[T[:, 1]], pts[T[:, 2]]
    cross = (p1[:, 0] - p0[:, 0]) * (p2[:, 1] - p0[:, 1]) - (p1[:, 1] - p0[:, 1]) * (p2[:, 0] - p0[:, 0])
    keep = np.abs(cross) > 1e-12 * L * L
    T, cross = T[keep], cross[keep]
    flip = cross < 0
    T[flip, 1], T[flip, 2] = T[flip, 2].copy(), T[flip, 1].copy()
    # Deterministic triangle order.
    T = T[np.lexsort((T[:, 2], T[:, 1], T[:, 0]))]
    used = np.zeros(nV, dtype=bool)
    used[T.ravel()] = True
    if not used.all():
        raise RuntimeError("triangulation lost %d vertices" % (~used).sum())
    nTri = T.shape[0]

    # Directed edges a->b of every CCW triangle, with the triangle on their left.
    a = np.concatenate([T[:, 0], T[:, 1], T[:, 2]])
    b = np.concatenate([T[:, 1], T[:, 2], T[:, 0]])
    tid = np.concatenate([np.arange(nTri)] * 3)
    # Neighbour sets (undirected).
    ua = np.concatenate([a, b])
    ub = np.concatenate([b, a])
    key = ua * nV + ub
    key = np.unique(key)
    na = key // nV
    nb = key % nV
    deg = np.bincount(na, minlength=nV)
    if deg.max() > NC_MEM:
        raise RuntimeError("vertex degree %d exceeds nC_mem=%d" % (deg.max(), NC_MEM))

    # Start angle per vertex: east for free vertices; for boundary vertices the direction
    # of the boundary neighbour that opens the counter-clockwise sweep.
    start = np.zeros(nV)
    start[edge == EDGE_S] = 0.0
    start[edge == EDGE_SW] = 0.0
    start[edge == EDGE_E] = 0.5 * math.pi
    start[edge == EDGE_SE] = 0.5 * math.pi
    start[edge == EDGE_N] = math.pi
    start[edge == EDGE_NE] = math.pi
    start[edge == EDGE_W] = 1.5 * math.pi
    start[edge == EDGE_NW] = 1.5 * math.pi
    dx = pts[nb, 0] - pts[na, 0]
    dy = pts[nb, 1] - pts[na, 1]
    ang = np.arctan2(dy, dx)
    rel = np.mod(ang - start[na], 2 * math.pi)
    # Boundary vertices: the opening boundary neighbour sits at rel == 0 exactly (or at
    # 2*pi - eps through rounding); force it first.
    bnd = edge[na] > 0
    rel = np.where(bnd & (rel > 2 * math.pi - 1e-9), 0.0, rel)
    order = np.lexsort((rel, na))
    na, nb = na[order], nb[order]
    rowstart = np.concatenate([[0], np.cumsum(deg)])
    pos = np.arange(na.size) - rowstart[na]
    C = np.zeros((nV, NC_MEM), dtype=np.int32)
    C[na, pos] = nb + 1
    nC = deg.astype(np.int32)

    # iTri(vi,k): triangle left of the directed edge vi -> C(vi,k), i.e. between C(k) and C(k+1).
    dir_key = a * nV + b
    sort_d = np.argsort(dir_key)
    dir_sorted = dir_key[sort_d]
    q = na * nV + nb
    loc = np.searchsorted(dir_sorted, q)
    found = (loc < dir_sorted.size) & (dir_sorted[np.minimum(loc, dir_sorted.size - 1)] == q)
    iTri = np.zeros((nV, NC_MEM), dtype=np.int32)
    ti_of = np.where(found, tid[sort_d[np.minimum(loc, dir_sorted.size - 1)]] + 1, 0)
    iTri[na, pos] = ti_of
    niTri = np.where(edge > 0, nC - 1, nC).astype(np.int32)
    # Consistency: free vertices have a triangle after every neighbour, boundary vertices
    # after all but the last.
    for vi_check in (np.flatnonzero(edge == 0)[:1000], np.flatnonzero(edge > 0)):
        for vi in vi_check:
            k = niTri[vi]
            if np.any(iTri[vi, :k] == 0):
                raise RuntimeError("vertex %d: missing triangle in CCW fan" % (vi + 1))
    # Boundary vertices: the last neighbour must close the fan (no triangle after it).
    bv = np.flatnonzero(edge > 0)
    if np.any(iTri[bv, nC[bv] - 1] != 0):
        raise RuntimeError("boundary vertex fan does not run edge to edge")

    return BaseMesh(
        xmin=float(xmin), xmax=float(xmax), ymin=float(ymin), ymax=float(ymax),
        V=np.asfortranarray(pts),
        nC=nC,
        C=np.asfortranarray(C),
        niTri=niTri,
        iTri=np.asfortranarray(iTri),
        Tri=np.asfortranarray((T + 1).astype(np.int32)),
        edge_index=edge,
    )


def graded_spacing(h_min, h_max, grading, R):
    """Target spacing that is h_min on the circle r = R and grows linearly with the
    distance from it, capped at h_max. Evaluated at the point of each cell nearest to the
    circle so that a cell straddling the band is refined."""

    def fn(cx, cy, size):
        r = np.hypot(cx, cy)
        d = np.maximum(0.0, np.abs(r - R) - size * (0.5 * math.sqrt(2.0)))
        return np.minimum(h_max, h_min + grading * d)

    return fn


def dome_mesh(n_target: str = "4k", seed: int = 20261204, L: float = 750e3) -> BaseMesh:
    """Square [-L, L]^2 refined towards the dome margin r = L.

    Presets (vertex counts are approximate):
    ``"4k"``   about 4,000 vertices, 30 km at the margin grading to 100 km;
    ``"100k"`` about 100,000 vertices, 2 km grading to 20 km;
    ``"200k"`` about 200,000 vertices, 2 km grading to 20 km;
    ``"300k"`` about 300,000 vertices, 2 km grading to 20 km;
    plus small ``"tiny"``, ``"1k"``, ``"16k"`` cases for tests.
    """
    rng = np.random.default_rng(seed)
    presets = {
        "tiny": (150e3, 300e3, 0.5),
        "1k": (50e3, 150e3, 0.5),
        "4k": (30e3, 100e3, 0.04),
        "16k": (10e3, 60e3, 0.1),
        "50k": (4e3, 40e3, 0.1),
        "100k": (2e3, 20e3, 0.095),
        "200k": (2e3, 20e3, 0.036),
        "300k": (2e3, 20e3, 0.021),
    }
    h_min, h_max, g = presets[n_target]
    fn = graded_spacing(h_min, h_max, g, L)
    inner, bnd = _quadtree_points(-L, L, -L, L, fn, rng)
    return triangulate_square(inner, bnd, -L, L, -L, L)


def sized_mesh(n_vertices: int, seed: int, L: float = 750e3) -> BaseMesh:
    """Mesh of roughly ``n_vertices`` vertices (for ensembles of uneven meshes): spacing s
    at the margin grading to 10 s, with s chosen by bisection on the leaf count."""
    def count(s):
        inner, bnd = _quadtree_points(-L, L, -L, L, graded_spacing(s, 10 * s, 0.1, L),
                                      np.random.default_rng(0))
        return inner.shape[0] + bnd.shape[0] + 4

    lo, hi = 0.5e3, 400e3
    for _ in range(30):
        mid = math.sqrt(lo * hi)
        if count(mid) > n_vertices:
            lo = mid
        else:
            hi = mid
        if hi / lo < 1.01:
            break
    rng = np.random.default_rng(seed)
    inner, bnd = _quadtree_points(-L, L, -L, L, graded_spacing(hi, 10 * hi, 0.1, L), rng)
    return triangulate_square(inner, bnd, -L, L, -L, L)
