"""Restart files of the tracer path through libfv3g: ``fv_tracer.res.tile<t>.nc`` (the tracers) and
``fv_core.res.tile<t>.nc`` (``delp``), plus ``ak``/``bk`` of ``fv_core.res.nc``, as fv3atm reads them at start-up
and writes them at restart times (atmos_model.F90:105,1149-1166), in the layout of the write component
(io/module_write_restart_netcdf.F90:244-317,444-530): dimensions ``xaxis_1``, ``yaxis_1``, ``zaxis_1`` and the
unlimited ``Time``; every field ``(Time, zaxis_1, yaxis_1, xaxis_1)`` with a ``checksum`` attribute (FMS
``mpp_chksum`` as ``'(Z16)'``).

Containers: netCDF classic (CDF-1), 64-bit offset (CDF-2) and 64-bit data (CDF-5).  The header is parsed by the
library on the host; the values go to the GPU as they lie in the file and one kernel swaps the byte order,
converts to the state's precision, places them in the halo-padded planes and sums the checksum.  Halos are not
in the files: the six-tile state rebuilds them before each substep; a one-face state needs its ring set.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import DP

NC_FLOAT, NC_DOUBLE = 5, 6
_TYPES = {1: np.int8, 2: np.uint8, 3: np.int16, 4: np.int32, 5: np.float32, 6: np.float64, 7: np.uint8, 8: np.uint16,
          9: np.uint32, 10: np.int64, 11: np.uint64}
AXES = ("xaxis_1", "xaxis_2", "yaxis_1", "yaxis_2", "zaxis_1", "Time")


def tracer_file(directory: str, tile: int) -> str:
    return os.path.join(directory, f"fv_tracer.res.tile{tile + 1}.nc")


def core_file(directory: str, tile: int) -> str:
    return os.path.join(directory, f"fv_core.res.tile{tile + 1}.nc")


class NcFile:
    """An open restart file (fv3g_ncfile)."""

    def __init__(self, path: str):
        self.path = path
        self._h = C.c_void_p()
        _lib.call("fv3g_nc_open", path.encode(), C.byref(self._h))

    def close(self) -> None:
        if self._h:
            _lib.load().fv3g_nc_close(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def variables(self) -> dict:
        """{name: (numpy dtype, shape, is_record)} in file order; a record dimension counts the records."""
        n = C.c_int(0)
        _lib.call("fv3g_nc_nvars", self._h, C.byref(n))
        out = {}
        for i in range(n.value):
            name = C.create_string_buffer(256)
            t, nd, rec = C.c_int(0), C.c_int(0), C.c_int(0)
            shape = (C.c_longlong * 8)()
            _lib.call("fv3g_nc_var_info", self._h, i, name, 256, C.byref(t), C.byref(nd), shape, C.byref(rec))
            out[name.value.decode()] = (np.dtype(_TYPES[t.value]), tuple(shape[:min(nd.value, 8)]), bool(rec.value))
        return out

    def checksum(self, name: str):
        """The variable's checksum attribute as an unsigned 64-bit int, or None."""
        v, present = C.c_ulonglong(0), C.c_int(0)
        _lib.call("fv3g_nc_checksum", self._h, name.encode(), C.byref(v), C.byref(present))
        return v.value if present.value else None

    def read(self, name: str, record: int = 0) -> np.ndarray:
        """One record (or the whole fixed variable) on the host, as float64."""
        vs = self.variables()
        if name not in vs:  # the library reports the missing variable
            _lib.call("fv3g_nc_read", self._h, name.encode(), record, np.zeros(1).ctypes.data_as(DP), C.c_longlong(1))
        dtype, shape, rec = vs[name]
        shape = shape[1:] if rec else shape
        out = np.empty(shape, dtype=np.float64)
        _lib.call("fv3g_nc_read", self._h, name.encode(), record, out.ctypes.data_as(DP), C.c_longlong(out.size))
        return out

    def field_names(self) -> list:
        """The 3-D fields (zaxis, yaxis, xaxis) of the file, axes excluded, in file order."""
        return [k for k, (dt, shp, rec) in self.variables().items()
                if k not in AXES and len(shp) - int(rec) == 3 and dt.kind == "f"]


def _names(names):
    arr = (C.c_char_p * len(names))(*[s.encode() for s in names])
    return arr


def read_state(state, field: str, tile: int, f, names, slots=None, verify: bool = True) -> list:
    """Load variables `names` of file f (an NcFile or a path) into tile `tile` of `state` ("Q": tracer slots,
    default 0..len-1; "DELP": one variable).  Returns the checksums of the data read."""
    own = not isinstance(f, NcFile)
    nc = NcFile(f) if own else f
    try:
        nv = len(names)
        sl = None
        if field == "Q":
            sl = (C.c_int * nv)(*(range(nv) if slots is None else slots))
        sums = (C.c_ulonglong * nv)()
        _lib.call("fv3g_state_read_restart", state.handle(), _lib.FIELDS[field], tile, nc._h, _names(names), sl, nv,
                  int(verify), sums)
        return list(sums)
    finally:
        if own:
            nc.close()


def write_state(state, field: str, tile: int, path: str, names, slots=None, dtype: str = "double",
                version: int = 2) -> list:
    """Write tile `tile` of a state field (the latest values) to a new file; dtype "double" or "float",
    version 1, 2 or 5.  Returns the checksums written."""
    nv = len(names)
    sl = None
    if field == "Q":
        sl = (C.c_int * nv)(*(range(nv) if slots is None else slots))
    sums = (C.c_ulonglong * nv)()
    _lib.call("fv3g_state_write_restart", state.handle(), _lib.FIELDS[field], tile, path.encode(), _names(names), sl,
              nv, NC_DOUBLE if dtype == "double" else NC_FLOAT, version, sums)
    return list(sums)


def load_restart(state, directory: str, tracer_names=None, verify: bool = True, delp: bool = True) -> list:
    """Read every tile's tracers (the first nq fields of fv_tracer.res.tile<t>.nc unless names are given) and
    delp (fv_core.res.tile<t>.nc) into the state, and ak/bk from fv_core.res.nc when it is there.  Returns the
    tracer names."""
    for t in range(state.ntiles):
        with NcFile(tracer_file(directory, t)) as f:
            names = list(tracer_names) if tracer_names is not None else f.field_names()[:state.nq]
            read_state(state, "Q", t, f, names, verify=verify)
        if delp:
            read_state(state, "DELP", t, core_file(directory, t), ["delp"], verify=verify)
    levels = os.path.join(directory, "fv_core.res.nc")
    if os.path.exists(levels):
        with NcFile(levels) as f:
            state.set_levels(f.read("ak").ravel(), f.read("bk").ravel())
    return names


def save_restart(state, directory: str, tracer_names, dtype: str = "double", version: int = 2,
                 delp: bool = False) -> None:
    """Write fv_tracer.res.tile<t>.nc (and, with delp, an fv_core.res.tile<t>.nc holding delp) for every tile."""
    os.makedirs(directory, exist_ok=True)
    for t in range(state.ntiles):
        write_state(state, "Q", t, tracer_file(directory, t), list(tracer_names), dtype=dtype, version=version)
        if delp:
            write_state(state, "DELP", t, core_file(directory, t), ["delp"], dtype=dtype, version=version)
