"""The FP32 thread-per-column remap (remap form 1: FP32 kord-9 states with 16 levels or more) against the FP64
oracle remap of the same advected field, and against the warp-per-column kernel (form 0, the default).

The remap alone is checked: the oracle remaps the GPU's own advected tracers on the GPU's own Lagrangian
thickness, so the FP32 transport error does not enter.  Tolerance: relative L2 <= 2e-6 per tracer (FP32
storage of the result and of the interface solve), the same between the two kernels."""
import numpy as np
import pytest

from fv3atm_gb300 import api
from fv3atm_gb300 import synth as S

from ._helpers import interior, rel_l2, remap_reference

pytestmark = pytest.mark.gpu

REMAP_TOL = 2e-6


def _advect_then_remap(P, form, iv=0, q_min=0.0):
    st = api.CubeState(P.n, P.npz, P.nq, precision="mixed", iv=iv, q_min=q_min)
    try:
        st.load_problem(P)
        st.set_remap_form(form)
        assert st.remap_form() == form
        st.tracer_2d(3)
        q_adv = st.download("Q")
        dp = st.download("DELP_OUT")
        st.remap()
        return q_adv, dp, st.download("Q_REMAPPED")
    finally:
        st.close()


@pytest.mark.parametrize("npz", [16, 43, 128])
@pytest.mark.parametrize("iv,q_min", [(0, 0.0), (1, 1e-6), (-1, 0.0)])
def test_column_remap_matches_oracle_and_warp_kernel(cuda, npz, iv, q_min):
    # 5 tracers: the last pass of two fields repeats the fifth and stores nothing
    P = S.make_problem(24, npz, 5, seed=21 + npz, cmax=0.8)
    q_adv, dp, q_col = _advect_then_remap(P, 1, iv, q_min)
    _, _, q_warp = _advect_then_remap(P, 0, iv, q_min)
    q_ref, _, _, _ = remap_reference(q_adv, dp, P.ak, P.bk, P.n, kord=9, iv=iv)
    for iq in range(P.nq):
        a, w, r = (interior(x[:, iq], P.n) for x in (q_col, q_warp, q_ref))
        e_or, e_w = rel_l2(a, r), rel_l2(a, w)
        assert e_or <= REMAP_TOL, (iq, e_or)
        assert e_w <= REMAP_TOL, (iq, e_w)
        # positivity (iv 0) and the floor (iv 1) up to the rounding of a difference of two float-float
        # partial masses inside a thin target layer
        slack = 1e-7 * np.abs(r).max()
        if iv == 0:
            assert a.min() >= min(0.0, r.min()) - slack, (iq, a.min())
        if iv == 1:
            assert a.min() >= min(q_min, r.min()) - slack, (iq, a.min())


def test_column_remap_not_used_below_16_levels(cuda):
    """Fewer than 16 levels: the state runs the warp kernel whatever the form, bit for bit."""
    P = S.make_problem(20, 15, 3, seed=5, cmax=0.8)
    _, _, a = _advect_then_remap(P, 0)
    _, _, b = _advect_then_remap(P, 1)
    assert np.array_equal(interior(a, P.n), interior(b, P.n))


def test_column_remap_conserves_column_mass(cuda):
    """The target layer means are differences of float-float masses below their interfaces, so every
    column's mass telescopes: sum q2 dp2 = sum q1 dp1 to the FP32 rounding of the stored means."""
    P = S.make_problem(24, 64, 4, seed=8, cmax=0.8)
    q_adv, dp, q2 = _advect_then_remap(P, 1)
    _, dp2, _, _ = remap_reference(q_adv, dp, P.ak, P.bk, P.n)
    n = P.n
    for iq in range(P.nq):
        m1 = (interior(q_adv[:, iq], n) * interior(dp, n)).sum(axis=1)
        m2 = (interior(q2[:, iq], n) * dp2).sum(axis=1)  # dp2: interior columns only
        scale = (np.abs(interior(q_adv[:, iq], n)) * interior(dp, n)).sum(axis=1)
        err = np.abs(m2 - m1) / np.maximum(scale, 1e-300)
        assert err.max() <= 2e-7, (iq, err.max())


def test_remap_form_is_validated(cuda):
    st = api.CubeState(12, 16, 1, precision="mixed")
    try:
        with pytest.raises(Exception):
            st.set_remap_form(2)
        assert st.remap_form() == 0
    finally:
        st.close()


def test_column_remap_host_step_groups_equal_device_step(cuda):
    """Both fields of a pass round alike (no automatic multiply-add contraction in the kernel), so the tracer
    groups of the pipelined host step, which pair the tracers differently, remap bit for bit alike."""
    import torch
    P = S.make_problem(24, 20, 5, seed=13, cmax=0.8)
    st = api.CubeState(P.n, P.npz, P.nq, precision="mixed")
    try:
        st.load_problem(P)
        st.set_remap_form(1)
        st.step(2)
        want = st.download("Q_REMAPPED")
        src = {"Q": P.q, "DELP": P.dp, "CX": P.cx, "CY": P.cy, "MFX": P.mfx, "MFY": P.mfy}
        host = {k: torch.as_tensor(v).to(torch.float32).contiguous().pin_memory() for k, v in src.items()}
        out = torch.zeros(st.field_shape("Q_REMAPPED"), dtype=torch.float32).pin_memory()
        for groups in (1, 3):
            out.zero_()
            st.step_host(2, host["Q"].data_ptr(), {k: h.data_ptr() for k, h in host.items()}, out.data_ptr(),
                         True, groups)
            assert np.array_equal(out.numpy().astype(np.float64), want), groups
    finally:
        st.close()
