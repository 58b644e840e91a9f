"""Tangent-linear and adjoint of the whole transport step on the device at the C4 size: six C96 tiles, 64
levels, 4 tracers, 6 substeps of tracer_2d (hord 5), then the kord-4 remap (fv3g_state_step_tl /
fv3g_state_step_ad).

The adjoint is the hand-written reverse sweep (transposed PPM stencils, copy_corners and cube-halo
transposes, the kord-4 column remap reversed); the tangent-linear model applies the same stencils forward
and runs the remap kernel on value/tangent pairs.  Both recompute each substep's trajectory from a
checkpoint of its input.

Checks:
* the dot-product test <J x, y> = <x, J^T y> on the full state of the seeded C4 trajectory (bells and
  Gaussians plus 1 % noise), x ~ N(0,1) x 1e-3 of each tracer's RMS, for tracer_2d, the remap and both;
* with every branch frozen the step is linear and homogeneous in q, so J q reproduces the production
  forward step to round-off;
* finite differences of the production FP64 step against J x at every step size 1e-4 .. 1e-8, each
  asserted against the bound 1e-3 (eps / 1e-4) + 1e-12 / eps (branch crossings along the segment, then
  round-off of the differenced steps).  The perturbation is relative to the local field, x = 1e-3 q r with
  r ~ N(0,1): an additive perturbation of 1e-3 of the RMS dwarfs the trajectory where q is tiny or zero
  (Gaussian tails, clipped plateaus), so the limiter and 2-dx filter there switch on the perturbation's
  own shape and the difference quotient measures another piece of the piecewise-linear map at every
  step size.  hord 5's 2-dx filter is discontinuous (a face flux jumps between the upwind and the
  parabolic value where bl br changes sign), so on the noisy trajectory its finite differences do not
  converge; they run on the smooth part of the trajectory (Gaussians without noise), and hord 8, whose
  limiter is continuous, runs on the noisy trajectory itself."""
import time

import numpy as np
import pytest

from fv3atm_gb300 import api
from fv3atm_gb300 import synth as S

pytestmark = pytest.mark.gpu

N, NPZ, NQ, NSUB = 96, 64, 4, 6
FD_STEPS = (1e-4, 1e-5, 1e-6, 1e-7, 1e-8)


def _interior(a):
    return a[..., 3:3 + N, 3:3 + N]


def _state(P, hord):
    st = api.CubeState(N, NPZ, NQ, precision="fp64", hord=hord, kord=4, iv=0)
    st.load_problem(P)
    q0 = np.ascontiguousarray(P.q.detach().cpu().numpy() if hasattr(P.q, "detach") else P.q, dtype=np.float64)
    return st, q0


@pytest.fixture(scope="module")
def noisy(cuda):
    return S.make_problem(N, NPZ, NQ, seed=4004, cmax=0.8)


@pytest.fixture(scope="module")
def c4(noisy):
    st, q0 = _state(noisy, 5)
    yield st, q0
    st.close()


def _rms_perturbation(q0, rng):
    x = np.zeros_like(q0)
    for iq in range(NQ):
        rms = float(np.sqrt(np.mean(_interior(q0[:, iq]) ** 2)))
        _interior(x[:, iq])[...] = rng.standard_normal(_interior(x[:, iq]).shape) * (1e-3 * rms)
    return x


def _tl(st, q0, x, parts=3):
    import torch
    st.upload("Q", q0)
    dx = torch.as_tensor(x, device="cuda")
    out = torch.zeros_like(dx)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st.step_tl(NSUB, dx.data_ptr(), out.data_ptr(), parts=parts)
    torch.cuda.synchronize()
    return out.cpu().numpy(), time.perf_counter() - t0


def _ad(st, q0, y, parts=3):
    import torch
    st.upload("Q", q0)
    dy = torch.as_tensor(y, device="cuda")
    out = torch.zeros_like(dy)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st.step_ad(NSUB, dy.data_ptr(), out.data_ptr(), parts=parts)
    torch.cuda.synchronize()
    return out.cpu().numpy(), time.perf_counter() - t0


def _forward(st, q, parts=3):
    st.upload("Q", q)
    t0 = time.perf_counter()
    if parts == 1:
        st.tracer_2d(NSUB)
        st.sync()
        return _interior(st.download("Q")), time.perf_counter() - t0
    st.step(NSUB, use_graph=False)
    st.sync()
    return _interior(st.download("Q_REMAPPED")), time.perf_counter() - t0


@pytest.mark.parametrize("parts", [1, 2, 3])
def test_c4_dot_product_full_state(c4, parts):
    st, q0 = c4
    rng = np.random.default_rng(41 + parts)
    x = _rms_perturbation(q0, rng)
    y = np.zeros_like(q0)
    _interior(y)[...] = rng.standard_normal(_interior(y).shape)
    jx, t_tl = _tl(st, q0, x, parts)
    jty, t_ad = _ad(st, q0, y, parts)
    assert np.all(jty[..., :3, :] == 0) and np.all(jty[..., :, :3] == 0), "halo cells of the adjoint are zero"
    lhs = float(np.sum(_interior(jx) * _interior(y)))
    rhs = float(np.sum(_interior(x) * _interior(jty)))
    rel = abs(lhs - rhs) / max(abs(lhs), abs(rhs))
    msg = f"\nC4 dot product (parts {parts}): <Jx,y>={lhs:.17e} <x,J^T y>={rhs:.17e} rel={rel:.3e}"
    if parts == 3:
        _, t_fw = _forward(st, q0)
        msg += (f"; forward step {t_fw * 1e3:.1f} ms, TL {t_tl * 1e3:.1f} ms, AD {t_ad * 1e3:.1f} ms "
                f"(AD / TL {t_ad / t_tl:.2f})")
    print(msg)
    assert rel <= 1e-12, rel


@pytest.mark.parametrize("hord", [5, 8])
def test_c4_tangent_linear_reproduces_the_step(noisy, hord):
    """The transport with its branches frozen is linear and homogeneous in q: J q = F(q)."""
    import torch
    st, q0 = _state(noisy, hord)
    try:
        ref, _ = _forward(st, q0, parts=1)
        jq, _ = _tl(st, q0, q0, parts=1)
        rel = float(np.linalg.norm(_interior(jq) - ref) / np.linalg.norm(ref))
        assert rel <= 1e-14, rel
    finally:
        st.close()
        torch.cuda.empty_cache()


@pytest.mark.parametrize("traj,hord", [("smooth", 5), ("noisy", 8)])
def test_c4_finite_differences_every_step(noisy, traj, hord):
    P = noisy if traj == "noisy" else S.make_problem(N, NPZ, NQ, seed=4004, cmax=0.8, tracer_kind="gauss",
                                                       noise=0.0)
    st, q0 = _state(P, hord)
    try:
        rng = np.random.default_rng(42)
        x = 1e-3 * q0 * rng.standard_normal(q0.shape)
        jx, _ = _tl(st, q0, x)
        tl = _interior(jx)
        base, _ = _forward(st, q0)
        errs = {}
        for eps in FD_STEPS:
            fd = (_forward(st, q0 + eps * x)[0] - base) / eps
            errs[eps] = float(np.linalg.norm(fd - tl) / np.linalg.norm(tl))
        print(f"\nC4 finite differences ({traj} trajectory, hord {hord}, kord 4), rel L2 of "
              "(F(q + eps x) - F(q))/eps - J x: " + ", ".join(f"{e:.0e}: {v:.3e}" for e, v in errs.items()))
        for eps, err in errs.items():
            bound = 1e-3 * (eps / 1e-4) + 1e-12 / eps
            assert err <= bound, (eps, err, bound)
    finally:
        st.close()
