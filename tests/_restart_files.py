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


def write_cdf5(path, fields: dict, checksum: bool = True):
    """A CDF-5 (64-bit data) file in the write component's layout, packed by hand from the published format
    (scipy writes CDF-1/2 only): big-endian, 8-byte counts, sizes, dimension ids and offsets."""
    import struct
    first = next(iter(fields.values()))
    npz, n = first.shape[0], first.shape[-1]
    dims = [("xaxis_1", n), ("yaxis_1", n), ("zaxis_1", npz), ("Time", 0)]

    def name(s):
        b = s.encode()
        return struct.pack(">q", len(b)) + b + b"\0" * (-len(b) % 4)

    def text_attr(k, v):
        b = v.encode()
        return name(k) + struct.pack(">iq", 2, len(b)) + b + b"\0" * (-len(b) % 4)

    # (name, dimids, attrs, nc_type, bytes per record or in all, record, data bytes)
    vars_ = [(a, [i], [("axis", a[0].upper())], 6, 8 * ln, False,
              np.arange(1, ln + 1, dtype=">f8").tobytes()) for i, (a, ln) in enumerate(dims[:3])]
    vars_.append(("Time", [3], [("cartesian_axis", "T")], 6, 8, True, np.array([1.0], ">f8").tobytes()))
    for k, a in fields.items():
        t = 6 if a.dtype == np.float64 else 5
        attrs = [("checksum", z16(mpp_chksum(a)))] if checksum else []
        vars_.append((k, [3, 2, 1, 0], attrs, t, a.nbytes, True, a.astype(a.dtype.newbyteorder(">")).tobytes()))

    def header(begins):
        h = b"CDF\x05" + struct.pack(">q", 1)
        h += struct.pack(">iq", 10, len(dims)) + b"".join(name(d) + struct.pack(">q", ln) for d, ln in dims)
        h += struct.pack(">iq", 0, 0)  # no global attributes
        h += struct.pack(">iq", 11, len(vars_))
        for (vn, ids, attrs, t, nb, rec, _), beg in zip(vars_, begins):
            h += name(vn) + struct.pack(">q", len(ids)) + b"".join(struct.pack(">q", i) for i in ids)
            h += (struct.pack(">iq", 12, len(attrs)) + b"".join(text_attr(k, v) for k, v in attrs)) if attrs \
                else struct.pack(">iq", 0, 0)
            h += struct.pack(">iqq", t, nb + (-nb % 4), beg)
        return h

    off = len(header([0] * len(vars_)))
    begins = [0] * len(vars_)
    for i, v in enumerate(vars_):  # the fixed variables first, then the record section
        if not v[5]:
            begins[i] = off
            off += v[4] + (-v[4] % 4)
    for i, v in enumerate(vars_):
        if v[5]:
            begins[i] = off
            off += v[4] + (-v[4] % 4)
    with open(path, "wb") as f:
        f.write(header(begins))
        for (vn, ids, attrs, t, nb, rec, data), beg in zip(vars_, begins):
            f.seek(beg)
            f.write(data + b"\0" * (-len(data) % 4))
