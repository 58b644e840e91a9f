"""The named configurations at their full sizes, checked through properties that
do not need the CPU oracle at that size (the oracle parity tests run on the
same code at smaller sizes):

* six C192 tiles, 127 levels, 9 tracers, tracer_2d n_split 3, hord 8: FP64
  global mass conservation, no new extrema, and the FP32-mixed path within
  1e-5 of the FP64 path per tracer.
"""
import numpy as np
import pytest

from fv3atm_gb300 import api
from fv3atm_gb300 import synth as S

from ._helpers import cube_mass, interior, rel_l2

pytestmark = pytest.mark.gpu


def _state(P, precision):
    import torch
    st = api.CubeState(P.n, P.npz, P.nq, precision=precision)
    st.set_grid(P.geoms)
    st.set_levels(P.ak, P.bk)
    dt = torch.float64 if precision == "fp64" else torch.float32
    cur = torch.cuda.current_stream().cuda_stream
    for name, val in (("Q", P.q), ("DELP", P.dp), ("CX", P.cx), ("CY", P.cy), ("MFX", P.mfx), ("MFY", P.mfy)):
        v = val.to(device="cuda", dtype=dt).contiguous()
        st.upload_device(name, v.data_ptr(), stream=cur)
        torch.cuda.synchronize()
    return st


def test_c192_l127_nine_tracers_fp64_vs_mixed(cuda):
    P = S.make_problem(192, 127, 9, seed=1192, cmax=0.8, pert_amp=10.0, device="cuda")
    n = P.n
    q0 = interior(P.q.cpu().numpy(), n)
    outs = {}
    for prec in ("fp64", "mixed"):
        st = _state(P, prec)
        m0 = st.mass("Q")
        st.tracer_2d(3)
        st.sync()
        outs[prec] = (interior(st.download("Q"), n), m0, st.mass("Q"))
        st.close()
    q64, m0, m1 = outs["fp64"]
    assert np.all(np.abs(m1 - m0) <= 1e-13 * np.abs(m0)), (m1 - m0) / m0
    for iq in range(P.nq):
        assert q64[:, iq].min() >= q0[:, iq].min() - 1e-14
        assert q64[:, iq].max() <= q0[:, iq].max() + 1e-14
        assert rel_l2(outs["mixed"][0][:, iq], q64[:, iq]) <= 1e-5
