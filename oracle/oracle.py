"""ctypes bindings of the FP64 CPU oracle (oracle/fv3_oracle.cpp).

TEST INFRASTRUCTURE ONLY: the oracle that the CUDA path is compared against.
The library is built by ``make -C oracle`` (``build()`` below does it).
Parity against the upstream Fortran is unpinned (its source is absent).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libfv3oracle.so")
_lib = None

DP = C.POINTER(C.c_double)


class Bounds(C.Structure):
    _fields_ = [(k, C.c_int) for k in ("is_", "ie", "js", "je", "isd", "ied", "jsd", "jed", "ng")]


class Grid(C.Structure):
    _fields_ = [("dx", DP), ("dy", DP), ("dxa", DP), ("dya", DP), ("area", DP), ("rarea", DP), ("sin_sg", DP),
                ("sw_corner", C.c_int), ("se_corner", C.c_int), ("nw_corner", C.c_int), ("ne_corner", C.c_int),
                ("nested", C.c_int), ("del6_u", DP), ("del6_v", DP), ("da_min", C.c_double)]


class NestBC(C.Structure):
    _fields_ = [(k, DP) for k in ("west_t0", "west_t1", "east_t0", "east_t1", "south_t0", "south_t1", "north_t0",
                                  "north_t1")]


HALO_FN = C.CFUNCTYPE(None, DP, C.c_int, C.c_int, C.c_void_p)

NEST_SIDES = ("west", "east", "south", "north")


def nest_bc_structs(bc: dict, nq: int):
    """(NestBC * nq) for boundary states given as {side: (t0, t1)} with t0, t1 of shape (nq, npz, rows, cols),
    C-contiguous float64; a missing side gives NULL pointers."""
    arr = (NestBC * nq)()
    for iq in range(nq):
        ptrs = []
        for side in NEST_SIDES:
            pair = bc.get(side)
            for t in range(2):
                ptrs.append(_p(pair[t][iq]) if pair is not None else None)
        arr[iq] = NestBC(*ptrs)
    return arr


def build(force: bool = False) -> str:
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < max(
            os.path.getmtime(os.path.join(_HERE, f)) for f in ("fv3_oracle.cpp", "fv3_oracle.h")):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        L.orc_fv_tp_2d.restype = None
        L.orc_tracer_2d.restype = C.c_int
        L.orc_tracer_2d_cube.restype = C.c_int
        L.orc_tracer_2d_nested.restype = C.c_int
        L.orc_mass_sum.restype = C.c_double
        L.orc_mass_sum.argtypes = [DP, DP, DP, C.c_long, C.c_long]
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous, (a.dtype, a.flags)
    return a.ctypes.data_as(DP)


def _f64(a) -> np.ndarray:
    if hasattr(a, "detach"):
        a = a.detach().cpu().numpy()
    return np.ascontiguousarray(a, dtype=np.float64)


def bounds_for(n: int, ng: int = 3) -> Bounds:
    return Bounds(1, n, 1, n, 1 - ng, n + ng, 1 - ng, n + ng, ng)


class GridRef:
    """An orc_grid plus the arrays it points to (kept alive)."""

    def __init__(self, geom, corners=(1, 1, 1, 1), nested=0, da_min=None):
        self.arrays = [_f64(geom.dx), _f64(geom.dy), _f64(geom.dxa), _f64(geom.dya), _f64(geom.area),
                       _f64(geom.rarea), _f64(geom.sin_sg)]
        self.damp = [_f64(geom.del6_u), _f64(geom.del6_v)]
        if da_min is None:
            ng, n = geom.ng, geom.n
            da_min = float(np.min(geom.area[ng:ng + n, ng:ng + n]))
        self.struct = Grid(*[_p(a) for a in self.arrays], *corners, nested, *[_p(a) for a in self.damp],
                           C.c_double(da_min))


def copy_corners(q: np.ndarray, n: int, direction: int, geom, ng: int = 3) -> np.ndarray:
    q = _f64(q).copy()
    g = GridRef(geom)
    lib().orc_copy_corners(_p(q), n + 1, n + 1, direction, C.byref(g.struct), C.byref(bounds_for(n, ng)))
    return q


def _opt(a):
    return _p(a) if a is not None else None


def fv_tp_2d(q, crx, cry, hord, xfx, yfx, geom, ra_x, ra_y, mfx=None, mfy=None, ng: int = 3, lim_fac=1.0,
             mass=None, nord=0, damp_c=0.0, nested=0, da_min=None, corners=(1, 1, 1, 1)):
    """Returns (fx, fy, q_with_corners)."""
    q = _f64(q).copy()
    n = q.shape[-1] - 2 * ng
    fx = np.zeros((n, n + 1))
    fy = np.zeros((n + 1, n))
    g = GridRef(geom, corners=corners, nested=nested, da_min=da_min)
    arrs = [_f64(a) for a in (crx, cry, xfx, yfx, ra_x, ra_y)]
    mx = _f64(mfx) if mfx is not None else None
    my = _f64(mfy) if mfy is not None else None
    ms = _f64(mass) if mass is not None else None
    lib().orc_fv_tp_2d(_p(q), _p(arrs[0]), _p(arrs[1]), n + 1, n + 1, hord, _p(fx), _p(fy), _p(arrs[2]),
                       _p(arrs[3]), C.byref(g.struct), C.byref(bounds_for(n, ng)), _p(arrs[4]), _p(arrs[5]),
                       C.c_double(lim_fac), _opt(mx), _opt(my), _opt(ms), nord, C.c_double(damp_c))
    return fx, fy, q


def fv_tp_2d_tl(q, dq, crx, cry, hord, xfx, yfx, geom, ra_x, ra_y, mfx=None, mfy=None, ng: int = 3, lim_fac=1.0,
                mass=None, nord=0, damp_c=0.0, corners=(1, 1, 1, 1)):
    q = _f64(q)
    dq = _f64(dq)
    n = q.shape[-1] - 2 * ng
    dfx = np.zeros((n, n + 1))
    dfy = np.zeros((n + 1, n))
    g = GridRef(geom, corners=corners)
    arrs = [_f64(a) for a in (crx, cry, xfx, yfx, ra_x, ra_y)]
    mx = _f64(mfx) if mfx is not None else None
    my = _f64(mfy) if mfy is not None else None
    lib().orc_fv_tp_2d_tl(_p(q), _p(dq), _p(arrs[0]), _p(arrs[1]), n + 1, n + 1, hord, _p(dfx), _p(dfy),
                          _p(arrs[2]), _p(arrs[3]), C.byref(g.struct), C.byref(bounds_for(n, ng)), _p(arrs[4]),
                          _p(arrs[5]), C.c_double(lim_fac), _opt(mx), _opt(my),
                          _opt(_f64(mass) if mass is not None else None), nord, C.c_double(damp_c))
    return dfx, dfy


def count_fv_tp_2d(q, crx, cry, hord, xfx, yfx, geom, ra_x, ra_y, mfx, mfy, ng: int = 3) -> dict:
    """Operation counts of one fv_tp_2d call on one tile level (the counting scalar of the oracle)."""
    q = _f64(q)
    n = q.shape[-1] - 2 * ng
    g = GridRef(geom)
    arrs = [_f64(a) for a in (crx, cry, xfx, yfx, ra_x, ra_y, mfx, mfy)]
    c = (C.c_ulonglong * 4)()
    lib().orc_count_fv_tp_2d(_p(q), _p(arrs[0]), _p(arrs[1]), n + 1, n + 1, hord, _p(arrs[2]), _p(arrs[3]),
                             C.byref(g.struct), C.byref(bounds_for(n, ng)), _p(arrs[4]), _p(arrs[5]), _p(arrs[6]),
                             _p(arrs[7]), c)
    return dict(zip(("add", "mul", "div", "cmp"), (int(v) for v in c)))


def count_remap_column(pe1, q1, pe2, iv=0, kord=9) -> dict:
    """Operation counts of the remap of one column (tracer-valued quantities only)."""
    pe1, q1, pe2 = _f64(pe1), _f64(q1), _f64(pe2)
    c = (C.c_ulonglong * 4)()
    lib().orc_count_remap_column(q1.shape[0], _p(pe1), _p(q1), pe2.shape[0] - 1, _p(pe2), iv, kord, c)
    return dict(zip(("add", "mul", "div", "cmp"), (int(v) for v in c)))


def tracer_2d(q, dp1, mfx, mfy, cx, cy, geom, hord=8, q_split=0, halo_fn=None, ng: int = 3, nord_tr=0, trdm=0.0,
              lim_fac=1.0):
    """Single-domain tracer_2d.  q (nq, npz, nd, nd).  Returns (q, dp1, mfx, mfy, cx, cy, nsplt)."""
    q = _f64(q).copy()
    dp1, mfx, mfy, cx, cy = (_f64(a).copy() for a in (dp1, mfx, mfy, cx, cy))
    nq, npz = q.shape[0], q.shape[1]
    n = q.shape[-1] - 2 * ng
    g = GridRef(geom)
    cb = HALO_FN(halo_fn) if halo_fn is not None else HALO_FN()
    nsplt = lib().orc_tracer_2d(_p(q), _p(dp1), _p(mfx), _p(mfy), _p(cx), _p(cy), C.byref(g.struct),
                                C.byref(bounds_for(n, ng)), n + 1, n + 1, npz, nq, hord, q_split, C.c_double(0.0),
                                nord_tr, C.c_double(trdm), C.c_double(lim_fac), cb, None)
    return q, dp1, mfx, mfy, cx, cy, nsplt


def nest_bc_apply(var, bc: dict, step: float, split: float, bounds: Bounds, npx: int, npy: int, iq: int = 0):
    """nested_grid_BC_apply_intT of tracer iq's boundary states on var (npz, njd, nid); returns a copy."""
    var = _f64(var).copy()
    arr = nest_bc_structs(bc, iq + 1)
    lib().orc_nest_bc_apply(_p(var), C.byref(bounds), npx, npy, var.shape[0], C.byref(arr[iq]), C.c_double(step),
                            C.c_double(split))
    return var


def tracer_2d_nested(q, dp1, mfx, mfy, cx, cy, geom, bc, nest_timestep=0, k_split=1, hord=8, q_split=0,
                     halo_fn=None, nord_tr=0, trdm=0.0, lim_fac=1.0, nested=1, bounds: Bounds | None = None,
                     npx: int | None = None, npy: int | None = None, da_min=None, ng: int = 3):
    """tracer_2d_nested on one domain.  q (nq, npz, njd, nid); bc {side: (t0, t1)} (see nest_bc_structs) or
    None.  bounds default to a whole n x n domain.  Returns (q, dp1, mfx, mfy, cx, cy, nsplt, nest_timestep)."""
    q = _f64(q).copy()
    dp1, mfx, mfy, cx, cy = (_f64(a).copy() for a in (dp1, mfx, mfy, cx, cy))
    nq, npz = q.shape[0], q.shape[1]
    if bounds is None:
        n = q.shape[-1] - 2 * ng
        bounds, npx, npy = bounds_for(n, ng), n + 1, n + 1
    g = GridRef(geom, nested=nested, da_min=da_min)
    cb = HALO_FN(halo_fn) if halo_fn is not None else HALO_FN()
    arr = nest_bc_structs(bc, nq) if bc is not None else None
    counter = C.c_int(nest_timestep)
    nsplt = lib().orc_tracer_2d_nested(_p(q), _p(dp1), _p(mfx), _p(mfy), _p(cx), _p(cy), C.byref(g.struct),
                                       C.byref(bounds), npx, npy, npz, nq, hord, q_split, C.c_double(0.0), nord_tr,
                                       C.c_double(trdm), k_split, arr, C.byref(counter), C.c_double(lim_fac), cb,
                                       None)
    return q, dp1, mfx, mfy, cx, cy, nsplt, counter.value


def tracer_2d_1L(q, dp1, mfx, mfy, cx, cy, geom, hord=8, q_split=0, halo_fn=None, ng: int = 3, nord_tr=0,
                 trdm=0.0, lim_fac=1.0):
    """Single-domain tracer_2d_1L (per-level substep counts).  Returns (q, dp1, mfx, mfy, cx, cy, nsplt_levels)."""
    q = _f64(q).copy()
    dp1, mfx, mfy, cx, cy = (_f64(a).copy() for a in (dp1, mfx, mfy, cx, cy))
    nq, npz = q.shape[0], q.shape[1]
    n = q.shape[-1] - 2 * ng
    g = GridRef(geom)
    cb = HALO_FN(halo_fn) if halo_fn is not None else HALO_FN()
    ns = np.zeros(npz, dtype=np.int32)
    lib().orc_tracer_2d_1L(_p(q), _p(dp1), _p(mfx), _p(mfy), _p(cx), _p(cy), C.byref(g.struct),
                           C.byref(bounds_for(n, ng)), n + 1, n + 1, npz, nq, hord, q_split, C.c_double(0.0),
                           nord_tr, C.c_double(trdm), C.c_double(lim_fac), cb, None,
                           ns.ctypes.data_as(C.POINTER(C.c_int)))
    return q, dp1, mfx, mfy, cx, cy, ns


def tracer_2d_cube(q, dp1, mfx, mfy, cx, cy, geoms, topo, hord=8, q_split=0, sync_edges=False, ng: int = 3,
                   nord_tr=0, trdm=0.0, lim_fac=1.0):
    """Six-tile tracer_2d.  q (6, nq, npz, nd, nd).  Returns (q, dp1, nsplt)."""
    q = _f64(q).copy()
    dp1, mfx, mfy, cx, cy = (_f64(a).copy() for a in (dp1, mfx, mfy, cx, cy))
    nq, npz = q.shape[1], q.shape[2]
    n = q.shape[-1] - 2 * ng
    ng_, n_ = geoms[0].ng, geoms[0].n
    da = float(min(np.min(g.area[ng_:ng_ + n_, ng_:ng_ + n_]) for g in geoms))
    refs = [GridRef(g, da_min=da) for g in geoms]
    arr = (Grid * 6)(*[r.struct for r in refs])
    topo = np.ascontiguousarray(topo, dtype=np.int32)
    nsplt = lib().orc_tracer_2d_cube(_p(q), _p(dp1), _p(mfx), _p(mfy), _p(cx), _p(cy), arr, n, npz, nq, hord,
                                     q_split, topo.ctypes.data_as(C.POINTER(C.c_int)), int(sync_edges), nord_tr,
                                     C.c_double(trdm), C.c_double(lim_fac))
    return q, dp1, nsplt


def cube_halo_fill(q, n: int, topo, ng: int = 3) -> np.ndarray:
    q = _f64(q).copy()
    nplanes = int(np.prod(q.shape[1:-2]))
    topo = np.ascontiguousarray(topo, dtype=np.int32)
    lib().orc_cube_halo_fill(_p(q), n, ng, nplanes, topo.ctypes.data_as(C.POINTER(C.c_int)))
    return q


def column_profile(q, delp, iv=0, kord=9, qs=0.0, q_min=0.0) -> np.ndarray:
    q = _f64(q)
    delp = _f64(delp)
    a4 = np.zeros((q.shape[0], 4))
    lib().orc_column_profile(_p(q), _p(delp), q.shape[0], iv, kord, C.c_double(qs), C.c_double(q_min), _p(a4))
    return a4


def remap_column(pe1, q1, pe2, iv=0, kord=9, qs=0.0, q_min=0.0) -> np.ndarray:
    pe1, q1, pe2 = _f64(pe1), _f64(q1), _f64(pe2)
    q2 = np.zeros(pe2.shape[0] - 1)
    lib().orc_remap_column(q1.shape[0], _p(pe1), _p(q1), C.c_double(qs), q2.shape[0], _p(pe2), _p(q2), iv, kord,
                           C.c_double(q_min))
    return q2


def remap_columns(pe1, q1, pe2, iv=0, kord=9, qs=None, q_min=0.0, dp2=None) -> np.ndarray:
    """pe1 (km+1, ncol), q1 (km, ncol), pe2 (kn+1, ncol) -> q2 (kn, ncol); dp2 (kn, ncol): the target
    thicknesses dividing the overlap masses (map1_q2), else the pe2 differences."""
    pe1, q1, pe2 = _f64(pe1), _f64(q1), _f64(pe2)
    km, ncol = q1.shape
    kn = pe2.shape[0] - 1
    q2 = np.zeros((kn, ncol))
    qsa = _f64(qs) if qs is not None else None
    if dp2 is not None:
        d2 = _f64(dp2)
        lib().orc_remap_columns_dp2(ncol, km, _p(pe1), _p(q1), _p(qsa) if qsa is not None else None, kn, _p(pe2),
                                    _p(d2), _p(q2), iv, kord, C.c_double(q_min))
        return q2
    lib().orc_remap_columns(ncol, km, _p(pe1), _p(q1), _p(qsa) if qsa is not None else None, kn, _p(pe2), _p(q2),
                            iv, kord, C.c_double(q_min))
    return q2


def remap_columns_tl(pe1, q1, dq1, pe2, iv=0, kord=9, qs=None, q_min=0.0):
    """Tangent-linear of remap_columns (limiter branches frozen at q1) -> (q2, dq2)."""
    pe1, q1, dq1, pe2 = _f64(pe1), _f64(q1), _f64(dq1), _f64(pe2)
    km, ncol = q1.shape
    kn = pe2.shape[0] - 1
    q2, dq2 = np.zeros((kn, ncol)), np.zeros((kn, ncol))
    qsa = _f64(qs) if qs is not None else None
    lib().orc_remap_columns_tl(ncol, km, _p(pe1), _p(q1), _p(dq1), _p(qsa) if qsa is not None else None, kn,
                               _p(pe2), _p(q2), _p(dq2), iv, kord, C.c_double(q_min))
    return q2, dq2


def map_scalar(km, pe1, q1, qs, kn, pe2, q2, i1, i2, j, ibeg, iend, jbeg, jend, iv, kord, q_min):
    """Row-wise map_scalar on Fortran-shaped arrays (q1 (km, jdim, idim) C-order == (i,j,k) Fortran)."""
    pe1, q1, pe2 = _f64(pe1), _f64(q1), _f64(pe2)
    q2 = _f64(q2).copy()
    qsa = _f64(qs) if qs is not None else None
    lib().orc_map_scalar(km, _p(pe1), _p(q1), _p(qsa) if qsa is not None else None, kn, _p(pe2), _p(q2), i1, i2, j,
                         ibeg, iend, jbeg, jend, iv, kord, C.c_double(q_min))
    return q2


def fillz(q, dp) -> np.ndarray:
    """q (nq, km, im), dp (km, im) (C order of Fortran q(im, km, nq)) -> filled copy of q."""
    q = _f64(q).copy()
    dp = _f64(dp)
    nq, km, im = q.shape
    lib().orc_fillz(im, km, nq, _p(q), _p(dp))
    return q


def pressure_vars(delp, ptop, akap):
    """delp (km, im) -> pe, peln, pk (km+1, im), pkz (km, im)."""
    delp = _f64(delp)
    km, im = delp.shape
    pe, peln, pk = (np.zeros((km + 1, im)) for _ in range(3))
    pkz = np.zeros((km, im))
    lib().orc_pressure_vars(im, km, C.c_double(ptop), C.c_double(akap), _p(delp), _p(pe), _p(peln), _p(pk), _p(pkz))
    return pe, peln, pk, pkz


def mass_sum(q, dp, area) -> float:
    """Neumaier-compensated sum of q*dp*area; q, dp (..., ncell) broadcast area (ncell)."""
    q, dp, area = _f64(q), _f64(dp), _f64(area)
    q, dp = np.broadcast_arrays(q, dp)
    q = np.ascontiguousarray(q)
    dp = np.ascontiguousarray(dp)
    return lib().orc_mass_sum(_p(q), _p(dp), _p(area), q.size, area.size)
