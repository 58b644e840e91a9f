"""Restart files written by scipy's independent netCDF classic writer (CDF-1, CDF-2) in the write component's
layout (io/module_write_restart_netcdf.F90:244-317), for checking the library's reader and writer."""
from __future__ import annotations

import numpy as np

from oracle.restart_oracle import mpp_chksum, z16


def write_fields(path, fields: dict, version: int = 2, core: bool = False, checksum=True, extra: dict | None = None):
    """fields {name: (npz, n, n) float32/float64}; core: the fv_core.res layout (axes xaxis_1/2, yaxis_1/2, the
    cell fields on (yaxis_2, xaxis_1)); extra {name: (array, dims)} written as they are."""
    from scipy.io import netcdf_file
    first = next(iter(fields.values()))
    npz, n = first.shape[0], first.shape[-1]
    f = netcdf_file(path, "w", version=version)
    f.createDimension("Time", None)  # scipy wants the record dimension defined first
    axes = [("xaxis_1", n, "X")]
    if core:
        axes += [("xaxis_2", n + 1, "X"), ("yaxis_1", n + 1, "Y"), ("yaxis_2", n, "Y")]
    else:
        axes += [("yaxis_1", n, "Y")]
    axes += [("zaxis_1", npz, "Z")]
    for name, length, ax in axes:
        f.createDimension(name, length)
    for name, length, ax in axes:
        v = f.createVariable(name, "d", (name,))
        v.axis = ax
        v[:] = np.arange(1, length + 1, dtype=np.float64)
    t = f.createVariable("Time", "d", ("Time",))
    t.cartesian_axis, t.units, t.long_name = "T", "time level", "Time"
    t[:] = np.array([1.0])
    ycell = "yaxis_2" if core else "yaxis_1"
    for name, a in fields.items():
        v = f.createVariable(name, a.dtype.char, ("Time", "zaxis_1", ycell, "xaxis_1"))
        v[:] = a[None]
        if checksum is True:
            v.checksum = z16(mpp_chksum(a))
        elif isinstance(checksum, dict) and name in checksum:
            v.checksum = checksum[name]
    for name, (a, dims) in (extra or {}).items():
        v = f.createVariable(name, a.dtype.char, dims)
        v[:] = a
    f.NumFilesInSet = np.int32(1)
    f.close()


def read_fields(path) -> dict:
    """{name: (data without the record dimension, checksum attribute or None)} of every 4-D field."""
    from scipy.io import netcdf_file
    out = {}
    with netcdf_file(path, "r", mmap=False) as f:
        for name, v in f.variables.items():
            if v.dimensions and v.dimensions[0] == "Time" and len(v.dimensions) == 4:
                ck = getattr(v, "checksum", None)
                out[name] = (np.array(v[0]), ck.decode() if isinstance(ck, bytes) else ck)
    return out
