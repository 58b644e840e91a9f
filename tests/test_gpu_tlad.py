"""Tangent-linear and adjoint entries (fv3g_fv_tp_2d_tl/_ad, fv3g_map1_ppm_tl/_ad)
against the FP64 oracle's tangent-linear model, by dot-product tests, and by
torch.autograd.gradcheck through adjoint-backed autograd functions.

Tolerances: tangent-linear vs oracle relative L2 <= 1e-12; dot-product
<TL dq, w> vs <dq, AD w> relative difference <= 1e-12.
"""
import numpy as np
import pytest

import oracle as O
from fv3atm_gb300 import api
from fv3atm_gb300 import grid as G
from fv3atm_gb300 import synth as S

from ._helpers import area_fluxes, ra_xy, rel_l2

pytestmark = pytest.mark.gpu

TL_TOL = 1e-12
DOT_TOL = 1e-12


@pytest.fixture(scope="module")
def tile_prob():
    # n = 30: a full 26-cell CTA tile and a partial one; every tile corner is a cube corner
    return S.make_problem(30, 3, 2, seed=21, cmax=0.8)


def _smooth(shape, seed):
    """A tracer without flat spots or exact ties: the hord-8 limiter has a kink at
    every flat cell, where two tangent-linear models may pick different one-sided
    derivatives (the dot-product tests below use the clipped synthetic tracers)."""
    rng = np.random.default_rng(seed)
    jj, ii = np.meshgrid(np.arange(shape[0]), np.arange(shape[1]), indexing="ij")
    return np.ascontiguousarray(1.5 + 0.5 * np.sin(0.3 * ii) * np.cos(0.2 * jj) + 0.05 * rng.standard_normal(shape))


def _wave(shape):
    """A smooth positive tracer (no 2-dx extrema, no constant line): hord 5's filter is away from its
    switch everywhere, so finite differences of the scheme see the tangent-linear model's linear map.
    (On a constant line bl = br = 0 exactly and the filter sits on its switch.)"""
    jj, ii = np.meshgrid(np.arange(shape[0]), np.arange(shape[1]), indexing="ij")
    return np.ascontiguousarray(1.5 + 0.5 * np.sin(0.3 * ii + 0.4) * np.cos(0.2 * jj + 0.3))


def _inputs(P, t=1, k=1, iq=0, smooth=False):
    g = P.geoms[t]
    cx, cy = P.cx[t, k].numpy(), P.cy[t, k].numpy()
    xfx, yfx = area_fluxes(cx, cy, g)
    rax, ray = ra_xy(xfx, yfx, g)
    q = np.ascontiguousarray(P.q[t, iq, k].numpy())
    if smooth:
        q = _smooth(q.shape, 100 * t + k)
    return dict(n=P.n, g=g, q=q, cx=cx, cy=cy, xfx=xfx, yfx=yfx, rax=rax, ray=ray, mfx=P.mfx[t, k].numpy(),
                mfy=P.mfy[t, k].numpy())


LIM_FAC = {1: 2.5, 5: 1.0, 8: 1.0}  # hord 1 runs with a lim_fac other than 1


def _tl(d, dq, hord, mass=True):
    n = d["n"]
    fx, fxt, fy, fyt = np.zeros((n, n + 1)), np.zeros((n, n + 1)), np.zeros((n + 1, n)), np.zeros((n + 1, n))
    api.fv_tp_2d_tl(d["q"], dq, d["cx"], d["cy"], n + 1, n + 1, hord, fx, fxt, fy, fyt, d["xfx"], d["yfx"],
                    api.GridStruct(d["g"]), api.bounds_for(n), d["rax"], d["ray"], LIM_FAC[hord],
                    d["mfx"] if mass else None, d["mfy"] if mass else None)
    return fx, fxt, fy, fyt


def _ad(d, q_ad, wx, wy, hord, mass=True):
    n = d["n"]
    fx_ad, fy_ad = wx.copy(), wy.copy()
    api.fv_tp_2d_ad(d["q"], q_ad, d["cx"], d["cy"], n + 1, n + 1, hord, fx_ad, fy_ad, d["xfx"], d["yfx"],
                    api.GridStruct(d["g"]), api.bounds_for(n), d["rax"], d["ray"], LIM_FAC[hord],
                    d["mfx"] if mass else None, d["mfy"] if mass else None)
    return fx_ad, fy_ad


@pytest.mark.parametrize("hord", [1, 5, 8])
def test_fv_tp_2d_tl_matches_oracle(cuda, tile_prob, hord):
    d = _inputs(tile_prob, smooth=True)
    dq = np.random.default_rng(1).standard_normal(d["q"].shape)
    fx, fxt, fy, fyt = _tl(d, dq, hord)
    rfx, rfy = O.fv_tp_2d_tl(d["q"], dq, d["cx"], d["cy"], hord, d["xfx"], d["yfx"], d["g"], d["rax"], d["ray"],
                             d["mfx"], d["mfy"], lim_fac=LIM_FAC[hord])
    assert rel_l2(fxt, rfx) <= TL_TOL and rel_l2(fyt, rfy) <= TL_TOL
    ffx, ffy, _ = O.fv_tp_2d(d["q"], d["cx"], d["cy"], hord, d["xfx"], d["yfx"], d["g"], d["rax"], d["ray"],
                             d["mfx"], d["mfy"], lim_fac=LIM_FAC[hord])
    assert rel_l2(fx, ffx) <= TL_TOL and rel_l2(fy, ffy) <= TL_TOL  # the trajectory fluxes


def test_fv_tp_2d_tl_is_linear_and_rejects_higher_order_damping(cuda, tile_prob):
    """hord 5's 2-dx filter is frozen at the trajectory, so the tangent-linear model is a linear map; its
    damping is del-2 only."""
    d = _inputs(tile_prob)
    rng = np.random.default_rng(2)
    x, y = rng.standard_normal(d["q"].shape), rng.standard_normal(d["q"].shape)
    tx, ty, tz = (_tl(d, v, 5) for v in (x, y, 2.0 * x - 3.0 * y))
    for c in (1, 3):
        assert rel_l2(tz[c], 2.0 * tx[c] - 3.0 * ty[c]) <= TL_TOL
    from fv3atm_gb300._lib import Fv3gError
    n = d["n"]
    with pytest.raises(Fv3gError, match="nord 0 only"):
        api.fv_tp_2d_tl(d["q"], x, d["cx"], d["cy"], n + 1, n + 1, 8, None, np.zeros((n, n + 1)), None,
                        np.zeros((n + 1, n)), d["xfx"], d["yfx"], api.GridStruct(d["g"]), api.bounds_for(n), d["rax"],
                        d["ray"], 1.0, d["mfx"], d["mfy"], np.ones_like(d["q"]), 1, 0.1)


@pytest.mark.parametrize("with_mfx", [True, False])
def test_fv_tp_2d_tl_ad_with_del2_damping(cuda, tile_prob, with_mfx):
    """damp_c > 1e-4, nord 0: the tangent-linear fluxes equal the oracle's (damping included, mass-weighted
    with mass fluxes), and the adjoint passes the dot-product test."""
    d = _inputs(tile_prob, t=4, k=2, iq=1, smooth=True)
    n = d["n"]
    mass = np.ascontiguousarray(tile_prob.dp[4, 2].numpy())
    mx, my = (d["mfx"], d["mfy"]) if with_mfx else (None, None)
    rng = np.random.default_rng(11)
    dq = rng.standard_normal(d["q"].shape)
    gs = api.GridStruct(d["g"])
    fx, fxt, fy, fyt = np.zeros((n, n + 1)), np.zeros((n, n + 1)), np.zeros((n + 1, n)), np.zeros((n + 1, n))
    api.fv_tp_2d_tl(d["q"], dq, d["cx"], d["cy"], n + 1, n + 1, 8, fx, fxt, fy, fyt, d["xfx"], d["yfx"], gs,
                    api.bounds_for(n), d["rax"], d["ray"], 1.0, mx, my, mass, 0, 0.12)
    rfx, rfy = O.fv_tp_2d_tl(d["q"], dq, d["cx"], d["cy"], 8, d["xfx"], d["yfx"], d["g"], d["rax"], d["ray"], mx,
                             my, mass=mass, nord=0, damp_c=0.12)
    r0x, _ = O.fv_tp_2d_tl(d["q"], dq, d["cx"], d["cy"], 8, d["xfx"], d["yfx"], d["g"], d["rax"], d["ray"], mx, my)
    assert rel_l2(rfx, r0x) > 1e-6  # the damping is visible at this tolerance
    assert rel_l2(fxt, rfx) <= TL_TOL and rel_l2(fyt, rfy) <= TL_TOL
    wx, wy = rng.standard_normal((n, n + 1)), rng.standard_normal((n + 1, n))
    q_ad = np.zeros_like(d["q"])
    fx_ad, fy_ad = wx.copy(), wy.copy()
    api.fv_tp_2d_ad(d["q"], q_ad, d["cx"], d["cy"], n + 1, n + 1, 8, fx_ad, fy_ad, d["xfx"], d["yfx"], gs,
                    api.bounds_for(n), d["rax"], d["ray"], 1.0, mx, my, mass, 0, 0.12)
    lhs = float((fxt * wx).sum() + (fyt * wy).sum())
    rhs = float((q_ad * dq).sum())
    assert abs(lhs - rhs) <= DOT_TOL * abs(lhs), (lhs, rhs)


@pytest.mark.parametrize("hord", [1, 5, 8])
@pytest.mark.parametrize("mass", [True, False])
def test_fv_tp_2d_adjoint_dot_product(cuda, tile_prob, hord, mass):
    d = _inputs(tile_prob, t=4, k=2, iq=1)
    n = d["n"]
    rng = np.random.default_rng(3)
    dq = rng.standard_normal(d["q"].shape)
    wx, wy = rng.standard_normal((n, n + 1)), rng.standard_normal((n + 1, n))
    _, fxt, _, fyt = _tl(d, dq, hord, mass)
    q_ad0 = rng.standard_normal(d["q"].shape)
    q_ad = q_ad0.copy()
    fx_ad, fy_ad = _ad(d, q_ad, wx, wy, hord, mass)
    lhs = float((fxt * wx).sum() + (fyt * wy).sum())
    rhs = float(((q_ad - q_ad0) * dq).sum())  # the adjoint increments q_ad
    assert abs(lhs - rhs) <= DOT_TOL * abs(lhs), (lhs, rhs)
    assert not fx_ad.any() and not fy_ad.any()  # output adjoints consumed


def test_fv_tp_2d_adjoint_equals_oracle_jacobian_transpose(cuda):
    """On a 12-cell tile (cube corners and edges in every sweep), the adjoint equals
    J^T w with J assembled column by column from the oracle's tangent-linear model."""
    P = S.make_problem(12, 2, 1, seed=5, cmax=0.7)
    d = _inputs(P, t=0, k=1, iq=0, smooth=True)
    n, hord = d["n"], 8
    rng = np.random.default_rng(4)
    wx, wy = rng.standard_normal((n, n + 1)), rng.standard_normal((n + 1, n))
    ref = np.zeros_like(d["q"])
    e = np.zeros_like(d["q"])
    for idx in np.ndindex(*e.shape):
        e[idx] = 1.0
        dfx, dfy = O.fv_tp_2d_tl(d["q"], e, d["cx"], d["cy"], hord, d["xfx"], d["yfx"], d["g"], d["rax"], d["ray"],
                                 d["mfx"], d["mfy"])
        ref[idx] = (dfx * wx).sum() + (dfy * wy).sum()
        e[idx] = 0.0
    q_ad = np.zeros_like(d["q"])
    _ad(d, q_ad, wx, wy, hord)
    assert rel_l2(q_ad, ref) <= TL_TOL


# ------------------------------------------------------------------ map1_ppm
def _row(km=32, ni=12, seed=0):
    rng = np.random.default_rng(seed)
    ak, bk = G.hybrid_levels(km)
    ps = rng.uniform(95000.0, 103000.0, ni)
    dref = np.diff(ak)[:, None] + np.diff(bk)[:, None] * ps[None]
    dp = dref * (1.0 + 0.1 * rng.uniform(-1.0, 1.0, dref.shape))
    pe1 = np.ascontiguousarray(np.concatenate([np.full((1, ni), ak[0]), ak[0] + np.cumsum(dp, 0)]))
    pe2 = np.ascontiguousarray(ak[:, None] + bk[:, None] * pe1[-1][None])
    q1 = np.ascontiguousarray(np.sin(np.linspace(0, 3, km))[:, None] + 0.2 * rng.standard_normal((km, ni)) + 1.5)
    return pe1, pe2, q1, rng


@pytest.mark.parametrize("kord,iv", [(4, -1), (4, 0), (9, 0)])
def test_map1_ppm_tl_matches_oracle(cuda, kord, iv):
    pe1, pe2, q1, rng = _row(seed=1)
    km, ni = q1.shape
    dq = rng.standard_normal(q1.shape)
    q2, q2t = np.zeros((km, 1, ni)), np.zeros((km, 1, ni))
    api.map1_ppm_tl(km, pe1, q1[:, None, :].copy(), dq[:, None, :].copy(), None, km, pe2, q2, q2t, 1, ni, 1, 1, ni,
                    1, 1, iv, kord)
    r2, r2t = O.remap_columns_tl(pe1, q1, dq, pe2, iv=iv, kord=kord)
    assert rel_l2(q2[:, 0], r2) <= TL_TOL and rel_l2(q2t[:, 0], r2t) <= TL_TOL


@pytest.mark.parametrize("kord,iv", [(4, -1), (9, 0)])
def test_map1_ppm_adjoint_dot_product(cuda, kord, iv):
    pe1, pe2, q1, rng = _row(km=64, ni=20, seed=2)
    km, ni = q1.shape
    dq = rng.standard_normal(q1.shape)
    w = rng.standard_normal((km, ni))
    q2t = np.zeros((km, 1, ni))
    api.map1_ppm_tl(km, pe1, q1[:, None, :].copy(), dq[:, None, :].copy(), None, km, pe2, None, q2t, 1, ni, 1, 1, ni,
                    1, 1, iv, kord)
    q1_ad = np.zeros((km, 1, ni))
    q2_ad = w[:, None, :].copy()
    api.map1_ppm_ad(km, pe1, q1[:, None, :].copy(), q1_ad, None, km, pe2, q2_ad, 1, ni, 1, 1, ni, 1, 1, iv, kord)
    lhs, rhs = float((q2t[:, 0] * w).sum()), float((q1_ad[:, 0] * dq).sum())
    assert abs(lhs - rhs) <= DOT_TOL * abs(lhs), (lhs, rhs)
    assert not q2_ad.any()


# ------------------------------------------------------------------ autograd
def test_gradcheck_fv_tp_2d_hord5(cuda):
    torch = pytest.importorskip("torch")
    from ._autograd import FvTp2d
    P = S.make_problem(12, 2, 1, seed=7, cmax=0.6)
    d = _inputs(P, t=3, k=0, iq=0)
    d["q"] = _wave(d["q"].shape)
    args = dict(n=d["n"], hord=5, cx=d["cx"], cy=d["cy"], xfx=d["xfx"], yfx=d["yfx"], grid=api.GridStruct(d["g"]),
                bd=api.bounds_for(d["n"]), rax=d["rax"], ray=d["ray"], mfx=d["mfx"], mfy=d["mfy"])
    q = torch.tensor(d["q"], dtype=torch.float64, requires_grad=True)
    scale = float(np.abs(d["mfx"]).max())  # fluxes carry the mass-flux scale; check them in units of it

    def f(x):
        fx, fy = FvTp2d.apply(x, args)
        return fx / scale, fy / scale

    assert torch.autograd.gradcheck(f, (q,), eps=1e-6, atol=1e-8, rtol=1e-6)


def test_gradcheck_map1_ppm_kord4_slice(cuda):
    """The 12-column x 8-level slice of the kord-4 tangent-linear configuration."""
    torch = pytest.importorskip("torch")
    from ._autograd import Map1Ppm
    pe1, pe2, q1, _ = _row(km=8, ni=12, seed=3)
    args = dict(pe1=pe1, pe2=pe2, iv=-1, kord=4)
    q = torch.tensor(q1, dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(lambda x: Map1Ppm.apply(x, args), (q,), eps=1e-6, atol=1e-8, rtol=1e-6)


# ------------------------------------------- C96 tracer substeps (TL / AD)
def _c96_substeps(nsub=6, hord=5):
    """One C96 tile, one level, nsub tracer_2d substeps with the Courant numbers and
    mass fluxes scaled by 1/nsub; the halo ring is prescribed (no perturbation)."""
    P = S.make_problem(96, 1, 1, ntiles=1, seed=96, cmax=0.8)
    g = P.geoms[0]
    n, ng = P.n, 3
    cx, cy = P.cx[0, 0].numpy() / nsub, P.cy[0, 0].numpy() / nsub
    mfx, mfy = P.mfx[0, 0].numpy() / nsub, P.mfy[0, 0].numpy() / nsub
    xfx, yfx = area_fluxes(cx, cy, g)
    rax, ray = ra_xy(xfx, yfx, g)
    s = slice(ng, ng + n)
    rarea = g.rarea[s, s]
    dps = [P.dp[0, 0].numpy()[s, s]]
    for _ in range(nsub):
        dps.append(dps[-1] + (mfx[:, :-1] - mfx[:, 1:] + mfy[:-1, :] - mfy[1:, :]) * rarea)
    d = dict(n=n, g=g, cx=cx, cy=cy, xfx=xfx, yfx=yfx, rax=rax, ray=ray, mfx=mfx, mfy=mfy)
    return P, d, dps, rarea, s, hord


def _div(fx, fy):
    return fx[:, :-1] - fx[:, 1:] + fy[:-1, :] - fy[1:, :]


def _forward(P, d, dps, rarea, s, hord, q):
    traj = [q]
    n = d["n"]
    for k in range(len(dps) - 1):
        fx, fy = np.zeros((n, n + 1)), np.zeros((n + 1, n))
        api.fv_tp_2d(q.copy(), d["cx"], d["cy"], n + 1, n + 1, hord, fx, fy, d["xfx"], d["yfx"], api.GridStruct(d["g"]),
                     api.bounds_for(n), d["rax"], d["ray"], 1.0, d["mfx"], d["mfy"])
        q = q.copy()
        q[s, s] = (q[s, s] * dps[k] + _div(fx, fy) * rarea) / dps[k + 1]
        traj.append(q)
    return traj


def _tl_substeps(d, dps, rarea, s, hord, traj, dq):
    for k in range(len(dps) - 1):
        d["q"] = traj[k]
        _, fxt, _, fyt = _tl(d, dq, hord)
        out = np.zeros_like(dq)  # the prescribed halo carries no perturbation
        out[s, s] = (dq[s, s] * dps[k] + _div(fxt, fyt) * rarea) / dps[k + 1]
        dq = out
    return dq


def _ad_substeps(d, dps, rarea, s, hord, traj, a):
    n = d["n"]
    for k in reversed(range(len(dps) - 1)):
        ai = a[s, s]
        prev = np.zeros_like(a)
        prev[s, s] = ai * dps[k] / dps[k + 1]
        gq = ai * rarea / dps[k + 1]
        fx_ad, fy_ad = np.zeros((n, n + 1)), np.zeros((n + 1, n))
        fx_ad[:, :-1] += gq
        fx_ad[:, 1:] -= gq
        fy_ad[:-1, :] += gq
        fy_ad[1:, :] -= gq
        d["q"] = traj[k]
        _ad(d, prev, fx_ad, fy_ad, hord)
        halo = np.ones_like(prev, bool)
        halo[s, s] = False
        prev[halo] = 0.0  # adjoints of the prescribed halo are not state
        a = prev
    return a


def test_c96_six_substeps_tl_ad_dot_product_and_finite_differences(cuda):
    P, d, dps, rarea, s, hord = _c96_substeps()
    q = _wave(P.q[0, 0, 0].shape)
    rng = np.random.default_rng(960)
    rms = float(np.sqrt(np.mean(q[s, s] ** 2)))
    x = np.zeros_like(q)
    x[s, s] = 1e-3 * rms * rng.standard_normal(x[s, s].shape)
    y = np.zeros_like(q)
    y[s, s] = 1e-3 * rms * rng.standard_normal(y[s, s].shape)
    traj = _forward(P, d, dps, rarea, s, hord, q)
    tlx = _tl_substeps(d, dps, rarea, s, hord, traj, x)
    ady = _ad_substeps(d, dps, rarea, s, hord, traj, y)
    lhs, rhs = float((tlx * y).sum()), float((x * ady).sum())
    assert abs(lhs - rhs) <= DOT_TOL * abs(lhs), (lhs, rhs)
    # finite differences of the hord-5 substeps at every step 1e-4 .. 1e-8, each against the bound
    # 1e-3 (eps / 1e-4) + 1e-12 / eps (switches of the 2-dx filter crossed along the segment, then
    # round-off of the differenced steps).  The perturbation is relative to the local field (x = 1e-3 q r):
    # hord 5 is piecewise linear, and a perturbation that dwarfs the field's own differences decides the
    # filter's switches by its shape instead
    xr = np.zeros_like(q)
    xr[s, s] = 1e-3 * q[s, s] * rng.standard_normal(q[s, s].shape)
    tlr = _tl_substeps(d, dps, rarea, s, hord, traj, xr)[s, s]
    base = traj[-1][s, s]
    errs = {}
    for eps in (1e-4, 1e-5, 1e-6, 1e-7, 1e-8):
        fd = (_forward(P, d, dps, rarea, s, hord, q + eps * xr)[-1][s, s] - base) / eps
        errs[eps] = rel_l2(fd, tlr)
    print("\nC96 single-tile substeps, finite differences: " + ", ".join(f"{e:.0e}: {v:.3e}" for e, v in errs.items()))
    for eps, err in errs.items():
        assert err <= 1e-3 * (eps / 1e-4) + 1e-12 / eps, (eps, err)


def test_c96_map1_ppm_kord4_adjoint_dot_product(cuda):
    pe1, pe2, q1, rng = _row(km=64, ni=96, seed=96)
    km, ni = q1.shape
    rms = float(np.sqrt(np.mean(q1 ** 2)))
    dq = 1e-3 * rms * rng.standard_normal(q1.shape)
    w = 1e-3 * rms * rng.standard_normal((km, ni))
    q2t = np.zeros((km, 1, ni))
    api.map1_ppm_tl(km, pe1, q1[:, None, :].copy(), dq[:, None, :].copy(), None, km, pe2, None, q2t, 1, ni, 1, 1, ni,
                    1, 1, -1, 4)
    q1_ad = np.zeros((km, 1, ni))
    api.map1_ppm_ad(km, pe1, q1[:, None, :].copy(), q1_ad, None, km, pe2, w[:, None, :].copy(), 1, ni, 1, 1, ni, 1, 1,
                    -1, 4)
    lhs, rhs = float((q2t[:, 0] * w).sum()), float((q1_ad[:, 0] * dq).sum())
    assert abs(lhs - rhs) <= DOT_TOL * abs(lhs), (lhs, rhs)
