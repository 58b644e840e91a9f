"""The named configurations at their full sizes against the FP64 CPU oracle:

* six C192 tiles, 127 levels, 9 tracers, tracer_2d n_split 3, hord 8 (FP64 plain vs FP32-mixed): every
  tracer of both paths against the oracle, FP64 global mass, no new extrema;
* six C384 tiles, 127 levels, 20 tracers, tracer_2d n_split 3 + the kord-9 remap, FP32-mixed (the operational
  size): the state advances all 20 tracers, the oracle two of them (the problem draws its tracers one by one,
  so those two are the first two of the 20), and the global mass drift of every tracer over the step;
* the uneven ensemble, 32 single-tile members (16 x C48 L32, 10 x C96 L64, 6 x C192 L127), 4 tracers each,
  n_split 2, one graph per ensemble step, FP32-mixed: every member against the oracle's single-tile step.
"""
import numpy as np
import pytest

import oracle as O
from fv3atm_gb300 import api
from fv3atm_gb300 import synth as S

from ._helpers import cube_mass, final_dp, interior, rel_l2, remap_reference

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-5
# One step of the mixed path moves a tracer's global mass by a few 1e-10 at most (the FP32 rounding of each
# stored value does not average out over the few cells that carry a localised tracer's mass); measured
# 2e-12 .. 1.6e-10 at C384 L127 x 20.
MIXED_MASS_STEP = 1e-9
# kord 9's extremum detection switches a layer between a flat and a curved profile (a two-grid-length wave,
# decided by the signs of the jumps between layer means); where two means agree to FP32 rounding the mixed path
# can take the other side of the switch than the FP64 oracle, and that layer moves by O(its jump).  Such layers
# are rare, but one of them is a larger part of a small member's norm: per member the error stays below 1e-4
# (C48 L32 members), their mean below 1e-5.
FLIP_MEMBER_TOL = 1e-4


def _host(t):
    return np.ascontiguousarray(t.detach().cpu().numpy())


def _state(P, precision, **kw):
    import torch
    st = api.CubeState(P.n, P.npz, P.nq, precision=precision, **kw)
    st.set_grid(P.geoms)
    st.set_levels(P.ak, P.bk)
    dt = torch.float64 if precision == "fp64" else torch.float32
    cur = torch.cuda.current_stream().cuda_stream
    for name, val in (("Q", P.q), ("DELP", P.dp), ("CX", P.cx), ("CY", P.cy), ("MFX", P.mfx), ("MFY", P.mfy)):
        v = val.to(device="cuda", dtype=dt).contiguous()
        st.upload_device(name, v.data_ptr(), stream=cur)
        torch.cuda.synchronize()
    return st


def test_c192_l127_nine_tracers_against_the_oracle(cuda):
    P = S.make_problem(192, 127, 9, seed=1192, cmax=0.8, pert_amp=10.0, device="cuda")
    n = P.n
    h = {k: _host(getattr(P, k)) for k in ("q", "dp", "mfx", "mfy", "cx", "cy")}
    q_ref, dp_last, ns = O.tracer_2d_cube(h["q"], h["dp"], h["mfx"], h["mfy"], h["cx"], h["cy"], P.geoms, P.topo,
                                          hord=8, q_split=3)
    q0 = interior(h["q"], n)
    for prec, tol in (("fp64", FP64_TOL), ("mixed", MIXED_TOL)):
        st = _state(P, prec)
        m0 = st.mass("Q")
        st.tracer_2d(3)
        st.sync()
        q = interior(st.download("Q"), n)
        m1 = st.mass("Q")
        st.close()
        for iq in range(P.nq):
            assert rel_l2(q[:, iq], interior(q_ref[:, iq], n)) <= tol, (prec, iq)
        if prec == "fp64":
            assert np.all(np.abs(m1 - m0) <= 1e-13 * np.abs(m0)), (m1 - m0) / m0
            for iq in range(P.nq):
                assert q[:, iq].min() >= q0[:, iq].min() - 1e-14
                assert q[:, iq].max() <= q0[:, iq].max() + 1e-14
        else:
            assert np.all(np.abs(m1 - m0) <= MIXED_MASS_STEP * np.abs(m0)), (m1 - m0) / m0
    # the oracle conserves the mass of its own result as well
    dpf = final_dp(dp_last, h["mfx"], h["mfy"], P.geoms, ns, n)
    mo0, mo1 = cube_mass(h["q"], h["dp"], P.geoms, n), cube_mass(q_ref, dpf, P.geoms, n)
    assert np.all(np.abs(mo1 - mo0) <= 1e-13 * np.abs(mo0))


def test_c384_l127_twenty_tracers_step_against_the_oracle(cuda):
    import torch
    P = S.make_problem(384, 127, 20, seed=2000, cmax=0.8, pert_amp=10.0, dp_noise=0.10, device="cuda")
    n, ntr = P.n, 2
    st = _state(P, "mixed")
    m0 = st.mass("Q")
    st.step(3, use_graph=False)
    st.sync()
    m1 = st.mass("Q_REMAPPED")
    got = torch.empty(st.field_shape("Q_REMAPPED"), dtype=torch.float32, device="cuda")
    st.download_device("Q_REMAPPED", got.data_ptr(), stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = got[:, :ntr].cpu().numpy().astype(np.float64)
    st.close()
    assert np.all(np.abs(m1 - m0) <= MIXED_MASS_STEP * np.abs(m0)), (m1 - m0) / m0
    h = {k: _host(getattr(P, k)) for k in ("dp", "mfx", "mfy", "cx", "cy")}
    q = _host(P.q[:, :ntr])
    geoms, topo, ak, bk = P.geoms, P.topo, P.ak, P.bk
    del P
    torch.cuda.empty_cache()
    q1, dp_last, ns = O.tracer_2d_cube(q, h["dp"], h["mfx"], h["mfy"], h["cx"], h["cy"], geoms, topo, hord=8,
                                       q_split=3)
    dpf = final_dp(dp_last, h["mfx"], h["mfy"], geoms, ns, n)
    want, _, _, _ = remap_reference(q1, dpf, ak, bk, n)
    for iq in range(ntr):
        assert rel_l2(interior(got[:, iq], n), interior(want[:, iq], n)) <= MIXED_TOL, iq


def test_ensemble_members_against_the_oracle(cuda):
    import torch
    from .test_gpu_ensemble import _oracle_single_tile
    spec = [(48, 32)] * 16 + [(96, 64)] * 10 + [(192, 127)] * 6
    probs, states = [], []
    for k, (n, npz) in enumerate(spec):
        P = S.make_problem(n, npz, 4, ntiles=1, seed=5000 + k, cmax=0.7)
        st = api.CubeState(n, npz, 4, precision="mixed", ntiles=1)
        st.load_problem(P)
        probs.append(P)
        states.append(st)
    ens = api.Ensemble(states)
    ens.step(2)
    torch.cuda.synchronize()
    errs = []
    for P, st in zip(probs, states):
        want = _oracle_single_tile(P, 2)
        got = st.download("Q_REMAPPED")
        errs.append(max(rel_l2(interior(got[:, iq], P.n), interior(want[:, iq], P.n)) for iq in range(4)))
    ens.close()
    for st in states:
        st.close()
    assert max(errs) <= FLIP_MEMBER_TOL, errs
    assert sum(errs) / len(errs) <= MIXED_TOL, errs
