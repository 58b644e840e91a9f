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


def _noalloc(pe1, q1, pe2, iv, kord, q_min):
    import torch
    nfield, km, ncol = q1.shape
    kn = pe2.shape[0] - 1
    d = {k: torch.as_tensor(v, device="cuda") for k, v in (("pe1", pe1), ("pe2", pe2), ("q1", q1))}
    q2 = torch.full((nfield, kn, ncol), -1.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    _lib.call("fv3g_remap_columns_noalloc", ncol, km, C.c_void_p(d["pe1"].data_ptr()),
              C.c_void_p(d["q1"].data_ptr()), None, kn, C.c_void_p(d["pe2"].data_ptr()), C.c_void_p(q2.data_ptr()),
              nfield, iv, kord, C.c_double(q_min), None)
    torch.cuda.synchronize()
    return q2.cpu().numpy()


def _allocating(pe1, q1, pe2, iv, kord, q_min):
    nfield, km, ncol = q1.shape
    kn = pe2.shape[0] - 1
    q2 = np.zeros((nfield, kn, 1, ncol))
    api.map_scalar_3d(km, pe1, np.ascontiguousarray(q1[:, :, None, :]), None, kn, pe2, q2, 1, ncol, 1, 1, 1, ncol,
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


def test_noalloc_remap_rejects_oversized_requests(cuda):
    with pytest.raises(_lib.Fv3gError, match="1024 columns"):
        _lib.call("fv3g_remap_columns_noalloc", 1025, 10, C.c_void_p(8), C.c_void_p(8), None, 10, C.c_void_p(8),
                  C.c_void_p(8), 1, 0, 9, C.c_double(0.0), None)
    with pytest.raises(_lib.Fv3gError, match="layers"):
        _lib.call("fv3g_remap_columns_noalloc", 10, 129, C.c_void_p(8), C.c_void_p(8), None, 10, C.c_void_p(8),
                  C.c_void_p(8), 1, 0, 9, C.c_double(0.0), None)
