"""Equiangular gnomonic cubed-sphere geometry, tile topology and hybrid levels.

This module generates the grid metrics that FV3's ``fv_grid_type`` carries into
the tracer path (dx, dy, dxa, dya, area, rarea, sin_sg, the damping metrics
del6_u/del6_v and da_min, corner flags; upstream
``fv_grid_tools`` / ``fv_grid_utils``, absent from the reference tree, whose only
in-tree users are ``atmos_model.F90:578-614``) and the six-tile connectivity that
the on-device halo gather and the tile-edge flux reconciliation use.

Arrays are numpy float64 with shape ``(nj, ni)`` in C order, so memory is
i-fastest exactly like a Fortran ``(i, j)`` array.  ``tile_geometry`` gives one
face on its extended gnomonic grid (halo included), which requires ``n >= 12``
with a 3-cell halo.  ``cube_geometry`` then replaces the halo metrics of the six
faces by those of the cells they stand for, as FV3's halo updates of the grid
do: an edge-strip cell takes the neighbouring tile's metrics (rotated into the
tile's directions), a cube-corner cell those of the cell that the copy_corners
rotation of the sweep direction puts there (x metrics by the x-sweep rotation,
y metrics by the y-sweep one).  Both tiles beside a cube edge then see the
same cells on either side of it, so they compute the same face fluxes.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

RADIUS = 6.371e6  # m

# Face definitions: (centre, i axis, j axis).  e_i x e_j = centre on every face.
FACES = (
    ((1, 0, 0), (0, 1, 0), (0, 0, 1)),
    ((0, 1, 0), (-1, 0, 0), (0, 0, 1)),
    ((-1, 0, 0), (0, -1, 0), (0, 0, 1)),
    ((0, -1, 0), (1, 0, 0), (0, 0, 1)),
    ((0, 0, 1), (0, 1, 0), (-1, 0, 0)),
    ((0, 0, -1), (0, 1, 0), (1, 0, 0)),
)
W, E, S, N = 0, 1, 2, 3
# endpoints of each edge in face coordinates (sx, sy); "along" runs first -> second
_EDGE_ENDS = {W: ((-1, -1), (-1, 1)), E: ((1, -1), (1, 1)), S: ((-1, -1), (1, -1)), N: ((-1, 1), (1, 1))}


def _cube_point(face: int, sx: int, sy: int) -> tuple:
    c, e1, e2 = (np.array(v) for v in FACES[face])
    return tuple(int(v) for v in (c + sx * e1 + sy * e2))


def cube_topology() -> np.ndarray:
    """(6, 4, 3) int32: neighbour tile, neighbour edge, reversed-along flag."""
    topo = np.zeros((6, 4, 3), dtype=np.int32)
    for t in range(6):
        for e in range(4):
            p0 = _cube_point(t, *_EDGE_ENDS[e][0])
            p1 = _cube_point(t, *_EDGE_ENDS[e][1])
            found = None
            for u in range(6):
                if u == t:
                    continue
                for f in range(4):
                    q0 = _cube_point(u, *_EDGE_ENDS[f][0])
                    q1 = _cube_point(u, *_EDGE_ENDS[f][1])
                    if {q0, q1} == {p0, p1}:
                        found = (u, f, 0 if q0 == p0 else 1)
            assert found is not None
            topo[t, e] = found
    return topo


def halo_source(topo: np.ndarray, n: int, t: int, i: int, j: int) -> tuple:
    """Tile-local 1-based halo cell (i, j) of tile t -> (tile, i, j) interior cell."""
    if i < 1:
        e, d, s = W, 1 - i, j - 1
    elif i > n:
        e, d, s = E, i - n, j - 1
    elif j < 1:
        e, d, s = S, 1 - j, i - 1
    else:
        e, d, s = N, j - n, i - 1
    nt, ne, rev = (int(v) for v in topo[t, e])
    sb = n - 1 - s if rev else s
    if ne == W:
        return nt, d, sb + 1
    if ne == E:
        return nt, n + 1 - d, sb + 1
    if ne == S:
        return nt, sb + 1, d
    return nt, sb + 1, n + 1 - d


def _gnomonic(face: int, a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Unit vectors of equiangular face coordinates (a, b) in radians."""
    c, e1, e2 = (np.array(v, dtype=np.float64) for v in FACES[face])
    x, y = np.tan(a), np.tan(b)
    p = c[None, None, :] + x[..., None] * e1 + y[..., None] * e2
    return p / np.linalg.norm(p, axis=-1, keepdims=True)


def _arc(p: np.ndarray, q: np.ndarray) -> np.ndarray:
    """Great-circle angle between unit vectors (numerically robust form)."""
    return 2.0 * np.arcsin(np.clip(0.5 * np.linalg.norm(p - q, axis=-1), 0.0, 1.0))


def _tri_area(a: np.ndarray, b: np.ndarray, c: np.ndarray) -> np.ndarray:
    """Solid angle of spherical triangles (Van Oosterom & Strackee 1983)."""
    num = np.abs(np.einsum("...k,...k->...", a, np.cross(b, c)))
    den = 1.0 + np.einsum("...k,...k->...", a, b) + np.einsum("...k,...k->...", b, c) + np.einsum(
        "...k,...k->...", c, a)
    return 2.0 * np.arctan2(num, den)


def _sin_angle(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Sine of the angle between the equiangular coordinate lines at (a, b)."""
    x, y = np.tan(a), np.tan(b)
    cos = -x * y / np.sqrt((1.0 + x * x) * (1.0 + y * y))
    return np.sqrt(1.0 - cos * cos)


@dataclasses.dataclass
class TileGeom:
    """Metrics of one tile on the data domain (isd:ied, jsd:jed), shape (nj, ni)."""

    n: int
    ng: int
    tile: int
    dx: np.ndarray      # (n+2ng+1, n+2ng)   south-edge length, rows jsd..jed+1
    dy: np.ndarray      # (n+2ng, n+2ng+1)   west-edge length, cols isd..ied+1
    dxa: np.ndarray
    dya: np.ndarray
    area: np.ndarray
    rarea: np.ndarray
    sin_sg: np.ndarray  # (9, n+2ng, n+2ng); slots 0..3 = W, S, E, N edges
    corners: np.ndarray  # (n+2ng+1, n+2ng+1, 3) unit vectors of cell corners
    centers: np.ndarray  # (n+2ng, n+2ng, 3)
    del6_u: np.ndarray   # (n+2ng+1, n+2ng)   y faces: sina_v dx / dyc
    del6_v: np.ndarray   # (n+2ng, n+2ng+1)   x faces: sina_u dy / dxc
    sw_corner: int = 1
    se_corner: int = 1
    nw_corner: int = 1
    ne_corner: int = 1


def tile_geometry(n: int, tile: int, ng: int = 3, radius: float = RADIUS) -> TileGeom:
    if n < 12:
        raise ValueError("tile size n must be >= 12 for a 3-cell extended-gnomonic halo")
    h = 0.5 * math.pi / n
    ic = np.arange(1 - ng, n + 2 + ng)           # corner indices I = isd..ied+1
    ac = -0.25 * math.pi + (ic - 1) * h           # corner angles
    am = ac[:-1] + 0.5 * h                        # cell-centre angles
    B, A = np.meshgrid(ac, ac, indexing="ij")     # [J, I]
    corners = _gnomonic(tile, A, B)
    Bm, Am = np.meshgrid(am, am, indexing="ij")
    centers = _gnomonic(tile, Am, Bm)
    # edge midpoints (equiangular midpoints)
    Bw, Aw = np.meshgrid(am, ac, indexing="ij")   # x-faces: (J cell, I face)
    xmid = _gnomonic(tile, Aw, Bw)                # (nd, nd+1)
    Bs, As = np.meshgrid(ac, am, indexing="ij")   # y-faces: (J face, I cell)
    ymid = _gnomonic(tile, As, Bs)                # (nd+1, nd)
    dx = radius * _arc(corners[:, :-1], corners[:, 1:])     # (nd+1, nd)
    dy = radius * _arc(corners[:-1, :], corners[1:, :])     # (nd, nd+1)
    dxa = radius * _arc(xmid[:, :-1], xmid[:, 1:])          # (nd, nd)
    dya = radius * _arc(ymid[:-1, :], ymid[1:, :])          # (nd, nd)
    c00, c10, c01, c11 = corners[:-1, :-1], corners[:-1, 1:], corners[1:, :-1], corners[1:, 1:]
    area = radius * radius * (_tri_area(c00, c10, c11) + _tri_area(c00, c11, c01))
    nd = n + 2 * ng
    sin_sg = np.empty((9, nd, nd))
    sin_sg[0] = _sin_angle(Aw[:, :-1], Bw[:, :-1])   # west edge
    sin_sg[1] = _sin_angle(As[:-1, :], Bs[:-1, :])   # south edge
    sin_sg[2] = _sin_angle(Aw[:, 1:], Bw[:, 1:])     # east edge
    sin_sg[3] = _sin_angle(As[1:, :], Bs[1:, :])     # north edge
    sin_sg[4:] = _sin_angle(Am, Bm)[None]
    # Damping metrics of the del-n tracer diffusion: face length times the sine
    # of the grid angle at the face over the distance between the two cell
    # centres across it (dxc, dyc), on the extended grid of the face.
    ae = np.concatenate([[ac[0] - 0.5 * h], am, [ac[-1] + 0.5 * h]])  # centres, one extra each side
    Bx, Ax = np.meshgrid(am, ae, indexing="ij")                          # (nd, nd+2)
    cx_ext = _gnomonic(tile, Ax, Bx)
    dxc = radius * _arc(cx_ext[:, :-1], cx_ext[:, 1:])                   # (nd, nd+1) x faces
    By, Ay = np.meshgrid(ae, am, indexing="ij")                          # (nd+2, nd)
    cy_ext = _gnomonic(tile, Ay, By)
    dyc = radius * _arc(cy_ext[:-1, :], cy_ext[1:, :])                   # (nd+1, nd) y faces
    del6_v = _sin_angle(Aw, Bw) * dy / dxc
    del6_u = _sin_angle(As, Bs) * dx / dyc
    return TileGeom(n=n, ng=ng, tile=tile, dx=dx, dy=dy, dxa=dxa, dya=dya, area=area, rarea=1.0 / area,
                    sin_sg=sin_sg, corners=corners, centers=centers, del6_u=del6_u, del6_v=del6_v)


def da_min(geoms) -> float:
    """Smallest interior cell area over the tiles given (gridstruct%da_min)."""
    return float(min(g.area[g.ng:g.ng + g.n, g.ng:g.ng + g.n].min() for g in geoms))


def edge_matrix(topo: np.ndarray, n: int, t: int, e: int) -> np.ndarray:
    """2x2 integer matrix taking a displacement (di, dj) in tile t's edge-e halo strip to the neighbour tile's
    (di, dj) at the cells the strip stands for."""
    # a strip cell at depth 2, position 2: its four neighbours stay in the strip
    if e == W:
        c = (-1, 2)
    elif e == E:
        c = (n + 2, 2)
    elif e == S:
        c = (2, -1)
    else:
        c = (2, n + 2)
    _, i0, j0 = halo_source(topo, n, t, *c)
    _, i1, j1 = halo_source(topo, n, t, c[0] + 1, c[1])
    _, i2, j2 = halo_source(topo, n, t, c[0], c[1] + 1)
    return np.array([[i1 - i0, i2 - i0], [j1 - j0, j2 - j0]], dtype=np.int64)


def corner_source(n: int, i: int, j: int, direction: int) -> tuple:
    """The edge-strip cell of the same tile that copy_corners puts at cube-corner halo cell (i, j) for a sweep
    in `direction` (1 = x, 2 = y), and the matrix taking displacements at (i, j) to displacements there
    (a quarter turn about the corner point)."""
    su = -1 if i < 1 else 1
    sv = -1 if j < 1 else 1
    cx2 = 1 if su < 0 else 2 * n + 1  # doubled corner coordinates
    cy2 = 1 if sv < 0 else 2 * n + 1
    u, v = 2 * i - cx2, 2 * j - cy2
    plus = (su == -sv) if direction == 1 else (su == sv)
    if plus:
        u2, v2, R = -v, u, np.array([[0, -1], [1, 0]], dtype=np.int64)
    else:
        u2, v2, R = v, -u, np.array([[0, 1], [-1, 0]], dtype=np.int64)
    return (u2 + cx2) // 2, (v2 + cy2) // 2, R


def resolve_cell(topo: np.ndarray, n: int, t: int, i: int, j: int, direction: int) -> tuple:
    """(tile, i, j, M) of the interior cell that data-domain cell (i, j) of tile t stands for, and the matrix
    taking displacements at (i, j) to displacements there; cube-corner cells use the copy_corners rotation of
    `direction`."""
    oi, oj = i < 1 or i > n, j < 1 or j > n
    if not oi and not oj:
        return t, i, j, np.eye(2, dtype=np.int64)
    if oi and oj:
        i2, j2, R = corner_source(n, i, j, direction)
        tt, i3, j3, M = resolve_cell(topo, n, t, i2, j2, direction)
        return tt, i3, j3, M @ R
    e = (W if i < 1 else E) if oi else (S if j < 1 else N)
    tt, i2, j2 = halo_source(topo, n, t, i, j)
    return tt, i2, j2, edge_matrix(topo, n, t, e)


# sin_sg slots of the four cell edges by outward direction
_SIN_SLOT = {(-1, 0): 0, (0, -1): 1, (1, 0): 2, (0, 1): 3}


def _face_of(tt: int, i: int, j: int, d: tuple) -> tuple:
    """('x' or 'y', i, j) of the face of cell (i, j) in direction d: x faces are west faces, y faces south."""
    if d == (-1, 0):
        return "x", i, j
    if d == (1, 0):
        return "x", i + 1, j
    if d == (0, -1):
        return "y", i, j
    return "y", i, j + 1


def face_source(topo: np.ndarray, n: int, t: int, kind: str, i: int, j: int) -> tuple:
    """The face of an interior cell that halo face (kind, i, j) of tile t stands for: (tile, kind, i, j, sign),
    sign = -1 where the neighbour's positive direction across the face is the opposite one.  x face (i, j)
    separates cells (i-1, j) and (i, j); y face (i, j) cells (i, j-1) and (i, j).  Returns None for a face of
    the tile itself (both cells interior, or one interior: a tile-edge face)."""
    cells = [(i - 1, j), (i, j)] if kind == "x" else [(i, j - 1), (i, j)]
    inside = [1 <= a <= n and 1 <= b <= n for a, b in cells]
    if any(inside):
        return None
    strip = [not ((a < 1 or a > n) and (b < 1 or b > n)) for a, b in cells]
    k = 1 if strip[1] else (0 if strip[0] else 1)
    c = cells[k]
    d = (-1, 0) if kind == "x" else (0, -1)
    if k == 0:
        d = (-d[0], -d[1])
    direction = 1 if kind == "x" else 2
    tt, ci, cj, M = resolve_cell(topo, n, t, c[0], c[1], direction)
    md = tuple(int(v) for v in M @ np.array(d))
    fk, fi, fj = _face_of(tt, ci, cj, md)
    # the tile's positive direction across the face, +i (x) or +j (y), in the neighbour's frame
    pos = M @ (np.array([1, 0]) if kind == "x" else np.array([0, 1]))
    sign = int(pos[0] + pos[1])
    return tt, fk, fi, fj, sign


def fill_halo_metrics(geoms: list, topo: np.ndarray) -> None:
    """Replace the halo metrics of six faces in place by those of the cells they stand for (module docstring)."""
    g0 = geoms[0]
    n, ng = g0.n, g0.ng
    src = [dict(dxa=g.dxa.copy(), dya=g.dya.copy(), area=g.area.copy(), sin_sg=g.sin_sg.copy(), dx=g.dx.copy(),
                dy=g.dy.copy(), del6_u=g.del6_u.copy(), del6_v=g.del6_v.copy()) for g in geoms]
    o = ng - 1  # array index of tile index i is i + o
    rng_ = range(1 - ng, n + ng + 1)
    for t, g in enumerate(geoms):
        for j in rng_:
            for i in rng_:
                if 1 <= i <= n and 1 <= j <= n:
                    continue
                for direction in (1, 2):
                    tt, ci, cj, M = resolve_cell(topo, n, t, i, j, direction)
                    s = src[tt]
                    along_i = M[0, 0] != 0 if direction == 1 else M[0, 1] != 0
                    if direction == 1:
                        g.dxa[j + o, i + o] = s["dxa" if along_i else "dya"][cj + o, ci + o]
                        g.area[j + o, i + o] = s["area"][cj + o, ci + o]
                    else:
                        g.dya[j + o, i + o] = s["dxa" if along_i else "dya"][cj + o, ci + o]
                    for d in (((-1, 0), (1, 0)) if direction == 1 else ((0, -1), (0, 1))):
                        md = tuple(int(v) for v in M @ np.array(d))
                        g.sin_sg[_SIN_SLOT[d], j + o, i + o] = s["sin_sg"][_SIN_SLOT[md], cj + o, ci + o]
                    for slot in range(4, 9):
                        g.sin_sg[slot, j + o, i + o] = s["sin_sg"][slot, cj + o, ci + o]
        # faces: dx, del6_u on y faces (rows jsd..jed+1), dy, del6_v on x faces (cols isd..ied+1)
        for kind in ("x", "y"):
            fi_rng = range(1 - ng, n + ng + 2) if kind == "x" else rng_
            fj_rng = rng_ if kind == "x" else range(1 - ng, n + ng + 2)
            for j in fj_rng:
                for i in fi_rng:
                    r = face_source(topo, n, t, kind, i, j)
                    if r is None:
                        continue
                    tt, fk, fi, fj, _ = r
                    s = src[tt]
                    names = ("dy", "del6_v") if kind == "x" else ("dx", "del6_u")
                    snames = ("dy", "del6_v") if fk == "x" else ("dx", "del6_u")
                    for a_, b_ in zip(names, snames):
                        getattr(g, a_)[j + o, i + o] = s[b_][fj + o, fi + o]
        g.rarea[...] = 1.0 / g.area
    # tile-edge faces: one value, the lower-numbered tile's
    for t, g in enumerate(geoms):
        for e in range(4):
            nt, ne, rev = (int(v) for v in topo[t, e])
            if nt > t:
                continue
            for sidx in range(n):
                own = _edge_face_slots(n, ng, e, sidx)
                other = _edge_face_slots(n, ng, ne, n - 1 - sidx if rev else sidx)
                for key, (name, idx) in own.items():
                    oname, oidx = other[key]
                    getattr(g, name)[idx] = getattr(geoms[nt], oname)[oidx]


def _edge_face_slots(n: int, ng: int, e: int, s: int) -> dict:
    """Array name and index of the length and damping metric of face s (0-based) along tile edge e."""
    o = ng - 1
    if e in (W, E):
        idx = (s + 1 + o, (1 if e == W else n + 1) + o)
        return {"len": ("dy", idx), "del6": ("del6_v", idx)}
    idx = ((1 if e == S else n + 1) + o, s + 1 + o)
    return {"len": ("dx", idx), "del6": ("del6_u", idx)}


def cube_geometry(n: int, ng: int = 3, radius: float = RADIUS) -> list:
    """The six faces with the halo metrics of the cells they stand for (module docstring)."""
    geoms = [tile_geometry(n, t, ng, radius) for t in range(6)]
    fill_halo_metrics(geoms, cube_topology())
    return geoms


def hybrid_levels(km: int, ptop: float = 100.0, p0: float = 1.0e5, eta_c: float = 0.2) -> tuple:
    """Synthetic monotone hybrid sigma-pressure coefficients (ak, bk), km+1 each.

    The operational GFS L63/L127 tables live in the absent ``fv_eta.F90``; this
    coordinate is pure pressure above eta_c and blends quadratically to sigma
    at the surface.  Interfaces stay monotone for ps in [900, 1100] hPa.
    """
    eta = np.arange(km + 1, dtype=np.float64) / km
    pref = ptop + (p0 - ptop) * eta ** 1.5
    bk = np.where(eta > eta_c, ((eta - eta_c) / (1.0 - eta_c)) ** 2, 0.0)
    ak = pref - bk * p0
    ak[-1] = 0.0
    bk[-1] = 1.0
    return ak, bk
