"""Host-side mirror of the FV3 tracer-path interface, backed by libfv3g.so.

The functions keep the Fortran names, argument order and meaning of
``tracer_2d`` (fv_tracer2d.F90), ``fv_tp_2d`` (tp_core.F90) and
``map_scalar`` / ``map1_ppm`` (fv_mapz.F90) of GFDL_atmos_cubed_sphere.
Arrays are numpy float64 in C order with the Fortran shape reversed (a
Fortran ``q(isd:ied, jsd:jed, npz, nq)`` is a numpy ``(nq, npz, njd, nid)``),
so memory order is identical.  ``inout`` arguments are updated in place and a
failing call raises ``Fv3gError`` (the Fortran shim maps it to FATAL).

``CubeState`` is the batched, device-resident six-tile path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import DP, Bounds, Grid, NestBC, StateDesc

__all__ = ["Bounds", "GridStruct", "fv_tp_2d", "tracer_2d", "tracer_2d_1L", "tracer_2d_nested", "NestBoundary",
           "map_scalar", "map1_ppm", "map_scalar_3d", "CubeState", "bounds_for"]


def _p(a):
    if a is None:
        return None
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
        raise TypeError("arrays must be C-contiguous float64 numpy arrays")
    return a.ctypes.data_as(DP)


def bounds_for(n: int, ng: int = 3, is_: int = 1, ie: int | None = None, js: int = 1, je: int | None = None) -> Bounds:
    ie = n if ie is None else ie
    je = n if je is None else je
    return Bounds(is_, ie, js, je, is_ - ng, ie + ng, js - ng, je + ng, ng)


class GridStruct:
    """fv3g_grid built from a tile geometry (keeps its arrays alive)."""

    def __init__(self, geom, corners=(1, 1, 1, 1), nested: int = 0, da_min: float | None = None):
        self.arrays = [np.ascontiguousarray(a, dtype=np.float64)
                       for a in (geom.dx, geom.dy, geom.dxa, geom.dya, geom.area, geom.rarea, geom.sin_sg)]
        self.damp = [np.ascontiguousarray(getattr(geom, f), dtype=np.float64) if hasattr(geom, f) else None
                     for f in ("del6_u", "del6_v")]
        if da_min is None:
            ng, n = geom.ng, geom.n
            da_min = float(np.min(geom.area[ng:ng + n, ng:ng + n]))
        self.struct = Grid(*[_p(a) for a in self.arrays], *corners, nested, _p(self.damp[0]), _p(self.damp[1]),
                           C.c_double(da_min))


def fv_tp_2d(q, crx, cry, npx, npy, hord, fx, fy, xfx, yfx, gridstruct: GridStruct, bd: Bounds, ra_x, ra_y,
             lim_fac=1.0, mfx=None, mfy=None, mass=None, nord=0, damp_c=0.0) -> None:
    _lib.call("fv3g_fv_tp_2d", _p(q), _p(crx), _p(cry), npx, npy, hord, _p(fx), _p(fy), _p(xfx), _p(yfx),
              C.byref(gridstruct.struct), C.byref(bd), _p(ra_x), _p(ra_y), C.c_double(lim_fac), _p(mfx), _p(mfy),
              _p(mass), nord, C.c_double(damp_c))


def tracer_2d(q, dp1, mfx, mfy, cx, cy, gridstruct: GridStruct, bd: Bounds, npx, npy, npz, nq, hord, q_split, dt,
              nord_tr=0, trdm=0.0, lim_fac=1.0, halo_update=None) -> int:
    """Returns nsplt.  halo_update(q) (numpy view of q) refreshes halos per substep."""
    shape = q.shape
    cb = _lib.HALO_FN()
    if halo_update is not None:
        def _cb(ptr, nq_, npz_, ctx):
            arr = np.ctypeslib.as_array(ptr, shape=shape)
            halo_update(arr)
        cb = _lib.HALO_FN(_cb)
    nsplt = C.c_int(0)
    _lib.call("fv3g_tracer_2d", _p(q), _p(dp1), _p(mfx), _p(mfy), _p(cx), _p(cy), C.byref(gridstruct.struct),
              C.byref(bd), npx, npy, npz, nq, hord, q_split, C.c_double(dt), nord_tr, C.c_double(trdm),
              C.c_double(lim_fac), cb, None, C.byref(nsplt))
    return nsplt.value


def tracer_2d_1L(q, dp1, mfx, mfy, cx, cy, gridstruct: GridStruct, bd: Bounds, npx, npy, npz, nq, hord, q_split,
                 dt, nord_tr=0, trdm=0.0, lim_fac=1.0, halo_update=None) -> int:
    """tracer_2d_1L: levels advanced one at a time with their own substep counts; returns the largest."""
    shape = q.shape
    cb = _lib.HALO_FN()
    if halo_update is not None:
        def _cb(ptr, nq_, npz_, ctx):
            halo_update(np.ctypeslib.as_array(ptr, shape=shape))
        cb = _lib.HALO_FN(_cb)
    nsplt = C.c_int(0)
    _lib.call("fv3g_tracer_2d_1L", _p(q), _p(dp1), _p(mfx), _p(mfy), _p(cx), _p(cy), C.byref(gridstruct.struct),
              C.byref(bd), npx, npy, npz, nq, hord, q_split, C.c_double(dt), nord_tr, C.c_double(trdm),
              C.c_double(lim_fac), cb, None, C.byref(nsplt))
    return nsplt.value


class NestBoundary:
    """neststruct%q_BC of every tracer: {side: (t0, t1)} for the sides "west", "east", "south", "north", each
    array (nq, npz, rows, cols) float64 in C order, i.e. per tracer the Fortran strip west (isd:0, jsd:jed, npz),
    east (npx:ied, jsd:jed, npz), south (isd:ied, jsd:0, npz) or north (isd:ied, npy:jed, npz).  A side the
    domain does not read may be left out."""

    SIDES = ("west", "east", "south", "north")

    def __init__(self, strips: dict):
        self.arrays = {k: tuple(np.ascontiguousarray(a, dtype=np.float64) for a in v) for k, v in strips.items()}
        nq = {a.shape[0] for v in self.arrays.values() for a in v}
        if len(nq) != 1:
            raise ValueError("boundary strips disagree on the tracer count")
        self.nq = nq.pop()
        self.structs = (NestBC * self.nq)()
        for iq in range(self.nq):
            ptrs = []
            for side in self.SIDES:
                pair = self.arrays.get(side)
                ptrs += [pair[t][iq].ctypes.data_as(DP) if pair is not None else None for t in range(2)]
            self.structs[iq] = NestBC(*ptrs)


def tracer_2d_nested(q, dp1, mfx, mfy, cx, cy, gridstruct: GridStruct, bd: Bounds, npx, npy, npz, nq, hord,
                     q_split, dt, nord_tr=0, trdm=0.0, k_split=1, q_bc: NestBoundary | None = None,
                     nest_timestep: int = 0, lim_fac=1.0, halo_update=None) -> tuple[int, int]:
    """tracer_2d_nested: on a nested grid the outer-side halos take q_bc interpolated to each substep's start.
    Returns (nsplt, the advanced nest_timestep)."""
    if q_bc is not None and q_bc.nq != nq:
        raise ValueError(f"q_bc holds {q_bc.nq} tracers, nq is {nq}")
    shape = q.shape
    cb = _lib.HALO_FN()
    if halo_update is not None:
        def _cb(ptr, nq_, npz_, ctx):
            halo_update(np.ctypeslib.as_array(ptr, shape=shape))
        cb = _lib.HALO_FN(_cb)
    nsplt = C.c_int(0)
    counter = C.c_int(nest_timestep)
    _lib.call("fv3g_tracer_2d_nested", _p(q), _p(dp1), _p(mfx), _p(mfy), _p(cx), _p(cy), C.byref(gridstruct.struct),
              C.byref(bd), npx, npy, npz, nq, hord, q_split, C.c_double(dt), nord_tr, C.c_double(trdm), k_split,
              q_bc.structs if q_bc is not None else None, C.byref(counter), C.c_double(lim_fac), cb, None,
              C.byref(nsplt))
    return nsplt.value, counter.value


def map_scalar(km, pe1, q1, qs, kn, pe2, q2, i1, i2, j, ibeg, iend, jbeg, jend, iv, kord, q_min) -> None:
    _lib.call("fv3g_map_scalar", km, _p(pe1), _p(q1), _p(qs), kn, _p(pe2), _p(q2), i1, i2, j, ibeg, iend, jbeg, jend,
              iv, kord, C.c_double(q_min))


def map1_ppm(km, pe1, q1, qs, kn, pe2, q2, i1, i2, j, ibeg, iend, jbeg, jend, iv, kord) -> None:
    _lib.call("fv3g_map1_ppm", km, _p(pe1), _p(q1), _p(qs), kn, _p(pe2), _p(q2), i1, i2, j, ibeg, iend, jbeg, jend,
              iv, kord)


def fv_tp_2d_tl(q, q_tl, crx, cry, npx, npy, hord, fx, fx_tl, fy, fy_tl, xfx, yfx, gridstruct: GridStruct,
                bd: Bounds, ra_x, ra_y, lim_fac=1.0, mfx=None, mfy=None, mass=None, nord=0, damp_c=0.0) -> None:
    """Tangent-linear fv_tp_2d (Courant numbers and mass fluxes frozen); fx / fy may be None."""
    _lib.call("fv3g_fv_tp_2d_tl", _p(q), _p(q_tl), _p(crx), _p(cry), npx, npy, hord, _p(fx), _p(fx_tl), _p(fy),
              _p(fy_tl), _p(xfx), _p(yfx), C.byref(gridstruct.struct), C.byref(bd), _p(ra_x), _p(ra_y),
              C.c_double(lim_fac), _p(mfx), _p(mfy), _p(mass), nord, C.c_double(damp_c))


def fv_tp_2d_ad(q, q_ad, crx, cry, npx, npy, hord, fx_ad, fy_ad, xfx, yfx, gridstruct: GridStruct, bd: Bounds,
                ra_x, ra_y, lim_fac=1.0, mfx=None, mfy=None, mass=None, nord=0, damp_c=0.0) -> None:
    """Adjoint fv_tp_2d at trajectory q: q_ad += J^T (fx_ad, fy_ad); fx_ad, fy_ad are zeroed."""
    _lib.call("fv3g_fv_tp_2d_ad", _p(q), _p(q_ad), _p(crx), _p(cry), npx, npy, hord, _p(fx_ad), _p(fy_ad), _p(xfx),
              _p(yfx), C.byref(gridstruct.struct), C.byref(bd), _p(ra_x), _p(ra_y), C.c_double(lim_fac), _p(mfx),
              _p(mfy), _p(mass), nord, C.c_double(damp_c))


def map1_ppm_tl(km, pe1, q1, q1_tl, qs, kn, pe2, q2, q2_tl, i1, i2, j, ibeg, iend, jbeg, jend, iv, kord) -> None:
    _lib.call("fv3g_map1_ppm_tl", km, _p(pe1), _p(q1), _p(q1_tl), _p(qs), kn, _p(pe2), _p(q2), _p(q2_tl), i1, i2, j,
              ibeg, iend, jbeg, jend, iv, kord)


def map1_ppm_ad(km, pe1, q1, q1_ad, qs, kn, pe2, q2_ad, i1, i2, j, ibeg, iend, jbeg, jend, iv, kord) -> None:
    _lib.call("fv3g_map1_ppm_ad", km, _p(pe1), _p(q1), _p(q1_ad), _p(qs), kn, _p(pe2), _p(q2_ad), i1, i2, j, ibeg,
              iend, jbeg, jend, iv, kord)


def map1_q2(km, pe1, q1, kn, pe2, q2, dp2, i1, i2, iv, kord, j, ibeg, iend, jbeg, jend, q_min=0.0) -> None:
    """map1_q2: row j of q1 onto pe2 with the target thicknesses dp2 (i1:i2, kn); q2 (kn, i2-i1+1) C order."""
    _lib.call("fv3g_map1_q2", km, _p(pe1), _p(q1), kn, _p(pe2), _p(q2), _p(dp2), i1, i2, iv, kord, j, ibeg, iend, jbeg,
              jend, C.c_double(q_min))


def fillz(im, km, nq, q, dp) -> None:
    """q (nq, km, im) (Fortran q(im, km, nq)) filled in place; dp (km, im)."""
    _lib.call("fv3g_fillz", im, km, nq, _p(q), _p(dp))


def pressure_vars(im, km, ptop, akap, delp, pe, peln, pk, pkz) -> None:
    _lib.call("fv3g_pressure_vars", im, km, C.c_double(ptop), C.c_double(akap), _p(delp), _p(pe), _p(peln), _p(pk),
              _p(pkz))


def map_scalar_3d(km, pe1, q1, qs, kn, pe2, q2, i1, i2, j1, j2, ibeg, iend, jbeg, jend, nq, iv, kord, q_min) -> None:
    _lib.call("fv3g_map_scalar_3d", km, _p(pe1), _p(q1), _p(qs), kn, _p(pe2), _p(q2), i1, i2, j1, j2, ibeg, iend,
              jbeg, jend, nq, iv, kord, C.c_double(q_min))


def _stream(stream):
    """C-ABI stream argument: None -> the state's own stream; a CUDA stream
    handle otherwise.  Handle 0 (torch's default, the legacy NULL stream) is
    passed as cudaStreamLegacy so that work stays ordered with it."""
    if stream is None:
        return C.c_void_p(0)
    return C.c_void_p(1 if int(stream) == 0 else int(stream))


class CubeState:
    """ntiles (6: the cube; 1: one face with a prescribed halo ring; with independent_tiles, a batch of such
    single faces of one size, advanced with one launch per phase) x npz levels x nq tracers resident in HBM
    (fv3g_state)."""

    def __init__(self, n: int, npz: int, nq: int, *, precision: str = "fp64", hord: int = 8, kord: int = 9,
                 iv: int = 0, q_min: float = 0.0, warps_per_cta: int = 0, ntiles: int = 6, nord_tr: int = 0,
                 trdm: float = 0.0, lim_fac: float = 1.0, fill: bool = False, edge_sync: bool = False,
                 mass_fix: bool = False, independent_tiles: bool = False):
        L = _lib.load()
        self.n, self.npz, self.nq, self.ntiles = n, npz, nq, ntiles
        self.nd = n + 6
        self.precision = precision
        prec = _lib.FV3G_FP64 if precision == "fp64" else _lib.FV3G_MIXED
        desc = StateDesc(n, ntiles, npz, nq, prec, hord, kord, iv, q_min, warps_per_cta, nord_tr, trdm, lim_fac,
                         int(fill), int(edge_sync), int(mass_fix), int(independent_tiles))
        self._h = C.c_void_p()
        _lib.check(L.fv3g_state_create(C.byref(desc), C.byref(self._h)), "fv3g_state_create")
        self._grids = []

    def close(self):
        if self._h:
            _lib.load().fv3g_state_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------- setup
    def set_grid(self, geoms) -> None:
        ng, n = geoms[0].ng, geoms[0].n
        da = float(min(np.min(g.area[ng:ng + n, ng:ng + n]) for g in geoms))  # over the cube
        for t, g in enumerate(geoms):
            gs = GridStruct(g, da_min=da)
            self._grids.append(gs)
            _lib.call("fv3g_state_set_grid", self._h, t, C.byref(gs.struct))

    def set_levels(self, ak, bk) -> None:
        self._ak = np.ascontiguousarray(ak, dtype=np.float64)
        self._bk = np.ascontiguousarray(bk, dtype=np.float64)
        _lib.call("fv3g_state_set_levels", self._h, _p(self._ak), _p(self._bk))

    def upload(self, field: str, host) -> None:
        a = np.ascontiguousarray(host, dtype=np.float64)
        _lib.call("fv3g_upload", self._h, _lib.FIELDS[field], _p(a))

    def download(self, field: str) -> np.ndarray:
        out = np.empty(self.field_shape(field), dtype=np.float64)
        _lib.call("fv3g_download", self._h, _lib.FIELDS[field], _p(out))
        return out

    def upload_device(self, field: str, dptr: int, stream=None) -> None:
        _lib.call("fv3g_upload_device", self._h, _lib.FIELDS[field], C.c_void_p(dptr), _stream(stream))

    def download_device(self, field: str, dptr: int, stream=None) -> None:
        _lib.call("fv3g_download_device", self._h, _lib.FIELDS[field], C.c_void_p(dptr), _stream(stream))

    def field_shape(self, field: str) -> tuple:
        n, nd, npz, nq, t = self.n, self.nd, self.npz, self.nq, self.ntiles
        return {"Q": (t, nq, npz, nd, nd), "Q_REMAPPED": (t, nq, npz, nd, nd), "DELP": (t, npz, nd, nd),
                "DELP_OUT": (t, npz, nd, nd), "CX": (t, npz, nd, n + 1), "CY": (t, npz, n + 1, nd),
                "MFX": (t, npz, n, n + 1), "MFY": (t, npz, n + 1, n)}[field]

    def load_problem(self, prob) -> None:
        """Upload a synth.Problem (grid, levels and every input field)."""
        self.set_grid(prob.geoms)
        self.set_levels(prob.ak, prob.bk)
        for name, val in (("Q", prob.q), ("DELP", prob.dp), ("CX", prob.cx), ("CY", prob.cy), ("MFX", prob.mfx),
                          ("MFY", prob.mfy)):
            self.upload(name, val.detach().cpu().numpy() if hasattr(val, "detach") else val)

    # ------------------------------------------------------------ compute
    def tracer_2d(self, q_split: int, stream=None) -> None:
        _lib.call("fv3g_tracer_2d_batched", self._h, q_split, _stream(stream))

    def remap(self, stream=None) -> None:
        _lib.call("fv3g_remap_batched", self._h, _stream(stream))

    def fillz(self, stream=None) -> None:
        """fillz on the remapped tracers."""
        _lib.call("fv3g_fillz_batched", self._h, _stream(stream))

    def autotune(self) -> int:
        """Pick the advection CTA widths by timing a substep; returns the interior width."""
        w = C.c_int(0)
        _lib.call("fv3g_state_autotune", self._h, C.byref(w))
        return w.value

    def nsplt(self) -> int:
        """Substeps of the last tracer_2d (q_split, or the count derived from the Courant maximum)."""
        n = C.c_int(0)
        _lib.call("fv3g_state_nsplt", self._h, C.byref(n))
        return n.value

    def set_tracer_pairs(self, on: bool) -> None:
        """FP32 states with hord 8: advance the tracers two per warp (True) or one per warp (False)."""
        _lib.call("fv3g_state_set_tracer_pairs", self._h, int(bool(on)))

    def set_mass_fix(self, on: bool) -> None:
        """Restore each tracer's global mass after every step (True) or leave it as transported (False)."""
        _lib.call("fv3g_state_set_mass_fix", self._h, int(bool(on)))

    def set_remap_form(self, form: int) -> None:
        """Remap kernel: 0 warp per column (default), 1 thread per column for FP32 kord-9 states of 16+ levels."""
        _lib.call("fv3g_state_set_remap_form", self._h, int(form))

    def remap_form(self) -> int:
        f = C.c_int(0)
        _lib.call("fv3g_state_remap_form", self._h, C.byref(f))
        return f.value

    def tracer_pairs(self) -> bool:
        on = C.c_int(0)
        _lib.call("fv3g_state_tracer_pairs", self._h, C.byref(on))
        return bool(on.value)

    def widths(self) -> tuple:
        """(interior, edge-ring) advection CTA widths in warps."""
        w, r = C.c_int(0), C.c_int(0)
        _lib.call("fv3g_state_widths", self._h, C.byref(w), C.byref(r))
        return w.value, r.value

    def step(self, q_split: int, use_graph: bool = True, stream=None) -> None:
        _lib.call("fv3g_step", self._h, q_split, int(use_graph), _stream(stream))

    def step_tl(self, q_split: int, dq_in: int, dq_out: int, parts: int = 3, stream=None) -> None:
        """fv3g_state_step_tl: dq_out = J dq_in for the step about the state's inputs (FP64 six-tile state);
        device pointers (ints) of Q-shaped FP64 arrays; parts 1 tracer_2d, 2 remap, 3 both."""
        _lib.call("fv3g_state_step_tl", self._h, q_split, parts, C.c_void_p(dq_in), C.c_void_p(dq_out),
                  _stream(stream))

    def step_ad(self, q_split: int, q_ad_out: int, q_ad_in: int, parts: int = 3, stream=None) -> None:
        """fv3g_state_step_ad: q_ad_in = J^T q_ad_out (hand-written reverse sweeps; kord 4)."""
        _lib.call("fv3g_state_step_ad", self._h, q_split, parts, C.c_void_p(q_ad_out), C.c_void_p(q_ad_in),
                  _stream(stream))

    def remap_fields(self, fields_in: int, fields_out: int, nfield: int, kind: int = 0, iv: int = 1, kord: int = 9,
                     q_min: float = 0.0, log_p: bool = False, stream=None) -> None:
        """fv3g_state_remap_fields: device pointers (ints) of (ntiles, nfield, npz, nd, nd) arrays of the state's
        element type; kind 0 cells, 1 u faces, 2 v faces."""
        _lib.call("fv3g_state_remap_fields", self._h, C.c_void_p(fields_in), C.c_void_p(fields_out), nfield, kind, iv,
                  kord, C.c_double(q_min), int(bool(log_p)), _stream(stream))

    def step_host(self, q_split: int, q_in: int, fields: dict, q_out: int, host_f32: bool, groups: int = 0,
                  stream=None) -> None:
        """fv3g_step_host: host pointers (ints) of Q, of fields["DELP"/"CX"/"CY"/"MFX"/"MFY"] and of the output;
        transfers of tracer groups overlap the compute.  With a stream the call only enqueues."""
        s = None if stream is None else _stream(stream)
        _lib.call("fv3g_step_host", self._h, q_split, C.c_void_p(q_in), C.c_void_p(fields["DELP"]),
                  C.c_void_p(fields["CX"]), C.c_void_p(fields["CY"]), C.c_void_p(fields["MFX"]),
                  C.c_void_p(fields["MFY"]), C.c_void_p(q_out), int(host_f32), groups, s)

    def handle(self):
        return self._h

    def mass(self, field: str = "Q", stream=None) -> np.ndarray:
        out = np.zeros(self.nq, dtype=np.float64)
        _lib.call("fv3g_mass_sum", self._h, _lib.FIELDS[field], _p(out), _stream(stream))
        return out

    # ------------------------------------------------ host copies / timing
    def upload_async(self, field: str, host_ptr: int, host_f32: bool, stream=None) -> None:
        _lib.call("fv3g_upload_async", self._h, _lib.FIELDS[field], C.c_void_p(host_ptr), int(host_f32),
                  _stream(stream))

    def download_async(self, field: str, host_ptr: int, host_f32: bool, stream=None) -> None:
        _lib.call("fv3g_download_async", self._h, _lib.FIELDS[field], C.c_void_p(host_ptr), int(host_f32),
                  _stream(stream))

    def sync(self, stream=None) -> None:
        _lib.call("fv3g_stream_sync", self._h, _stream(stream))

    def set_timing(self, enable: bool) -> None:
        _lib.call("fv3g_set_timing", self._h, int(enable))

    KERNEL_KINDS = ("prologue", "substep", "edge_fix", "remap", "halo")

    def kernel_times(self) -> dict:
        """{kind: (total ms, kernel launches)} of the last completed step."""
        ms = (C.c_double * len(self.KERNEL_KINDS))()
        cnt = (C.c_int * len(self.KERNEL_KINDS))()
        _lib.call("fv3g_kernel_times", self._h, ms, cnt)
        return {k: (ms[i], cnt[i]) for i, k in enumerate(self.KERNEL_KINDS)}

    def error_code(self) -> int:
        code = C.c_int(0)
        _lib.call("fv3g_state_error", self._h, C.byref(code))
        return code.value


class Ensemble:
    """Independent states advanced together by one graph per step (fv3g_ensemble)."""

    def __init__(self, members):
        L = _lib.load()
        self.members = list(members)
        arr = (C.c_void_p * len(self.members))(*[m.handle() for m in self.members])
        self._h = C.c_void_p()
        _lib.check(L.fv3g_ensemble_create(arr, len(self.members), C.byref(self._h)), "fv3g_ensemble_create")

    def step(self, q_split: int, stream=None) -> None:
        _lib.call("fv3g_ensemble_step", self._h, q_split, _stream(stream))

    def close(self):
        if self._h:
            _lib.load().fv3g_ensemble_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
