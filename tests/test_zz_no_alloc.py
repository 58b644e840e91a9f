"""fv3g_remap_columns_noalloc: the column remap for callers that cannot let the
library allocate device memory (they own their device arrays and forbid
cudaMalloc/cudaFree inside their time loop).  Its scratch is a fixed device
array shared by all calls, so it is checked against the allocating entry
fv3g_map_scalar_3d on two calls in a row with different data.

This file is collected last so that a failure here, in a run that stops at the
first failure, comes after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from fv3atm_gb300 import _lib, api
from fv3atm_gb300 import grid as G

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def _columns(seed, km, ncol, nfield):
    rng = np.random.default_rng(seed)
    ak, bk = G.hybrid_levels(km)
    ps = rng.uniform(95000.0, 103000.0, ncol)
    dref = np.diff(ak)[:, None] + np.diff(bk)[:, None] * ps[None]
    dp = dref * (1.0 + 0.1 * rng.uniform(-1.0, 1.0, dref.shape))
    pe1 = np.ascontiguousarray(np.concatenate([np.full((1, ncol), ak[0]), ak[0] + np.cumsum(dp, 0)]))
    pe2 = np.ascontiguousarray(ak[:, None] + bk[:, None] * pe1[-1][None])
    q1 = np.ascontiguousarray(np.abs(rng.standard_normal((nfield, km, ncol))) + 0.05)
    return pe1, pe2, q1


def _device(pe1, q1, pe2, qs):
    import torch
    d = {k: torch.as_tensor(v, device="cuda") for k, v in (("pe1", pe1), ("pe2", pe2), ("q1", q1))}
    if qs is not None:
        d["qs"] = torch.as_tensor(qs, device="cuda")
    nfield, _, ncol = q1.shape
    d["q2"] = torch.full((nfield, pe2.shape[0] - 1, ncol), -1.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    return d


def _call(d, iv, kord, q_min):
    nfield, km, ncol = d["q1"].shape
    kn = d["pe2"].shape[0] - 1
    qs = C.c_void_p(d["qs"].data_ptr()) if "qs" in d else None
    _lib.call("fv3g_remap_columns_noalloc", ncol, km, C.c_void_p(d["pe1"].data_ptr()),
              C.c_void_p(d["q1"].data_ptr()), qs, kn, C.c_void_p(d["pe2"].data_ptr()),
              C.c_void_p(d["q2"].data_ptr()), nfield, iv, kord, C.c_double(q_min), None)


def _noalloc(pe1, q1, pe2, iv, kord, q_min, qs=None):
    import torch
    d = _device(pe1, q1, pe2, qs)
    _call(d, iv, kord, q_min)
    torch.cuda.synchronize()
    return d["q2"].cpu().numpy()


def _allocating(pe1, q1, pe2, iv, kord, q_min, qs=None):
    nfield, km, ncol = q1.shape
    kn = pe2.shape[0] - 1
    q2 = np.zeros((nfield, kn, 1, ncol))
    qsa = None if qs is None else np.ascontiguousarray(qs[None, :])
    api.map_scalar_3d(km, pe1, np.ascontiguousarray(q1[:, :, None, :]), qsa, kn, pe2, q2, 1, ncol, 1, 1, 1, ncol,
                      1, 1, nfield, iv, kord, q_min)
    return q2[:, :, 0, :]


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def test_noalloc_remap_matches_allocating_entry_twice(cuda):
    for call, (seed, km, ncol, nfield, kord, iv) in enumerate(((1, 127, 1000, 3, 9, 0), (2, 63, 257, 2, 4, 1))):
        pe1, pe2, q1 = _columns(seed, km, ncol, nfield)
        got = _noalloc(pe1, q1, pe2, iv, kord, 0.1)
        want = _allocating(pe1, q1, pe2, iv, kord, 0.1)
        assert _rel(got, want) <= FP64_TOL, (call, _rel(got, want))


def test_noalloc_remap_at_its_limits_with_surface_values(cuda):
    """The full fixed array (1024 columns, 128 layers on both sides) and iv = -2, whose bottom interface is the
    caller's device array qs, against fv3g_map_scalar_3d given the same qs."""
    rng = np.random.default_rng(11)
    for call, kord in enumerate((4, 9)):
        pe1, pe2, q1 = _columns(20 + call, 128, 1024, 2)
        qs = q1[:, -1, :].mean(0) + 0.01 * rng.standard_normal(1024)
        got = _noalloc(pe1, q1, pe2, -2, kord, 0.0, qs=qs)
        want = _allocating(pe1, q1, pe2, -2, kord, 0.0, qs=qs)
        assert _rel(got, want) <= FP64_TOL, (kord, _rel(got, want))


def test_noalloc_remap_allocates_no_device_memory(cuda):
    """After a first call (which looks up the fixed array's address), further calls leave the device's free
    memory and torch's allocator untouched."""
    import torch
    pe1, pe2, q1 = _columns(5, 127, 1000, 3)
    d = _device(pe1, q1, pe2, None)
    _call(d, 0, 9, 0.0)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    stats0 = torch.cuda.memory_stats()
    for _ in range(3):
        _call(d, 0, 9, 0.0)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    stats1 = torch.cuda.memory_stats()
    assert free1 == free0
    for key in ("allocation.all.allocated", "reserved_bytes.all.current", "allocated_bytes.all.current"):
        assert stats1.get(key) == stats0.get(key), key


def test_noalloc_remap_rejects_oversized_requests(cuda):
    with pytest.raises(_lib.Fv3gError, match="1024 columns"):
        _lib.call("fv3g_remap_columns_noalloc", 1025, 10, C.c_void_p(8), C.c_void_p(8), None, 10, C.c_void_p(8),
                  C.c_void_p(8), 1, 0, 9, C.c_double(0.0), None)
    with pytest.raises(_lib.Fv3gError, match="layers"):
        _lib.call("fv3g_remap_columns_noalloc", 10, 129, C.c_void_p(8), C.c_void_p(8), None, 10, C.c_void_p(8),
                  C.c_void_p(8), 1, 0, 9, C.c_double(0.0), None)
    with pytest.raises(_lib.Fv3gError, match="qs"):
        _lib.call("fv3g_remap_columns_noalloc", 10, 10, C.c_void_p(8), C.c_void_p(8), None, 10, C.c_void_p(8),
                  C.c_void_p(8), 1, -2, 9, C.c_double(0.0), None)
