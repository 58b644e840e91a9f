"""FMS ``mpp_chksum`` and the text of a restart file's ``checksum`` attribute, restated in numpy.

TEST INFRASTRUCTURE ONLY: the oracle of the restart reader and writer.

``mpp_chksum`` (FMS, called by io/module_write_restart_netcdf.F90:444-500 on the field it writes) sums the
values' bit patterns as integers: an FP64 array as 64-bit integers, an FP32 array as 32-bit integers widened
with their sign to 64 bits; the sum wraps modulo 2^64.  The attribute is that integer written with the Fortran
edit descriptor ``Z16`` into a 32-character variable (:101,530): upper-case hexadecimal digits right-justified
in 16 columns, then 16 blanks.  FMS's own source is not in the reference tree, so this follows its published
behaviour; parity with a Fortran-written file is unpinned.
"""
from __future__ import annotations

import numpy as np


def mpp_chksum(a) -> int:
    """The checksum of an FP64 or FP32 array as an unsigned 64-bit value (two's complement of the sum)."""
    a = np.ascontiguousarray(a)
    if a.dtype == np.float64:
        bits = a.view(np.uint64).ravel()
    elif a.dtype == np.float32:
        bits = a.view(np.int32).astype(np.int64).view(np.uint64).ravel()
    else:
        raise TypeError(f"mpp_chksum of {a.dtype}")
    return int(np.add.reduce(bits, dtype=np.uint64)) if bits.size else 0


def z16(v: int) -> str:
    """The attribute text of checksum v."""
    return format(v & 0xFFFFFFFFFFFFFFFF, "X").rjust(16) + " " * 16
