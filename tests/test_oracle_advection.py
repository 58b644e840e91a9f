"""Known-answer and property tests of the CPU oracle's advection (no GPU).

No golden vectors exist for this path in the reference (its only test parses a
namelist, tests/test_post_nems_routines.F90), so the oracle is pinned by
properties every correct flux-form PPM transport on the cubed sphere has.
"""
import numpy as np
import pytest

import oracle as O
from fv3atm_gb300 import grid as G
from fv3atm_gb300 import synth as S

from ._helpers import area_fluxes, cube_mass, final_dp, interior, ra_xy


@pytest.fixture(scope="module")
def prob():
    return S.make_problem(16, 4, 3, seed=1, cmax=0.8)


def _cube(P, hord=8, q_split=3, sync=True, q=None):
    return O.tracer_2d_cube(P.q if q is None else q, P.dp, P.mfx, P.mfy, P.cx, P.cy, P.geoms, P.topo, hord=hord,
                            q_split=q_split, sync_edges=sync)


@pytest.mark.parametrize("hord", [5, 8])
def test_global_tracer_mass_conserved(prob, hord):
    P = prob
    q1, dp_last, ns = _cube(P, hord=hord)
    dpf = final_dp(dp_last, P.mfx.numpy(), P.mfy.numpy(), P.geoms, ns, P.n)
    m0 = cube_mass(P.q.numpy(), P.dp.numpy(), P.geoms, P.n)
    m1 = cube_mass(q1, dpf, P.geoms, P.n)
    assert np.all(np.abs(m1 - m0) <= 1e-13 * np.abs(m0)), (m1 - m0) / m0


def test_edge_reconciliation_is_what_conserves_mass(prob):
    P = prob
    q1, dp_last, ns = _cube(P, sync=False)
    dpf = final_dp(dp_last, P.mfx.numpy(), P.mfy.numpy(), P.geoms, ns, P.n)
    m0 = cube_mass(P.q.numpy(), P.dp.numpy(), P.geoms, P.n)
    m1 = cube_mass(q1, dpf, P.geoms, P.n)
    assert np.max(np.abs(m1 - m0) / np.abs(m0)) > 1e-8


@pytest.mark.parametrize("hord", [5, 8])
def test_constant_mixing_ratio_preserved(prob, hord):
    P = prob
    qc = np.full_like(P.q.numpy(), 0.37)
    q1, _, _ = _cube(P, hord=hord, q=qc)
    assert np.abs(interior(q1, P.n) - 0.37).max() <= 1e-14


def test_hord8_creates_no_new_extrema(prob):
    P = prob
    q1, _, _ = _cube(P, hord=8)
    q0 = interior(P.q.numpy(), P.n)
    qq = interior(q1, P.n)
    assert qq.min() >= 0.0 and qq.min() >= q0.min() - 1e-15
    for iq in range(P.nq):
        assert qq[:, iq].max() <= q0[:, iq].max() + 1e-14


def test_zero_courant_leaves_q_unchanged(prob):
    P = prob
    z = [np.zeros_like(a.numpy()) for a in (P.mfx, P.mfy, P.cx, P.cy)]
    q1, _, _ = O.tracer_2d_cube(P.q, P.dp, *z, P.geoms, P.topo, hord=8, q_split=1)
    a, b = interior(q1, P.n), interior(P.q.numpy(), P.n)
    assert np.all(np.abs(a - b) <= 2.3e-16 * np.abs(b))  # (q*dp)/dp: one rounding


def test_nsplt_from_max_courant(prob):
    P = prob
    t = 0
    args = [np.ascontiguousarray(a[t].numpy()) for a in (P.q, P.dp, P.mfx, P.mfy, P.cx, P.cy)]
    cmax = max(np.abs(args[4][:, 3:3 + P.n, :P.n]).max(), np.abs(args[5][:, :P.n, 3:3 + P.n]).max())
    out = O.tracer_2d(*args, P.geoms[t], hord=8, q_split=0)
    assert out[6] == int(1.0 + cmax)
    big = [a * 3.0 if k in (2, 3, 4, 5) else a for k, a in enumerate(args)]
    out2 = O.tracer_2d(*big, P.geoms[t], hord=8, q_split=0)
    assert out2[6] == int(1.0 + 3.0 * cmax) >= 2


def test_cube_step_equals_single_tile_steps_with_neighbour_halos():
    """One substep of the cube (no edge sync) equals six single-tile calls whose halos come from the neighbours."""
    P = S.make_problem(14, 2, 1, seed=4)
    q1, _, _ = O.tracer_2d_cube(P.q, P.dp, P.mfx, P.mfy, P.cx, P.cy, P.geoms, P.topo, hord=8, q_split=1,
                                sync_edges=False)
    qh = O.cube_halo_fill(P.q.numpy(), P.n, P.topo)
    for t in range(6):
        args = [np.ascontiguousarray(a[t]) for a in (qh, P.dp.numpy(), P.mfx.numpy(), P.mfy.numpy(), P.cx.numpy(),
                                                     P.cy.numpy())]
        ref = O.tracer_2d(*args, P.geoms[t], hord=8, q_split=1)[0]
        assert np.array_equal(interior(ref, P.n), interior(q1[t], P.n))


def test_copy_corners_rotations_known_answer():
    """Corner blocks continue the adjacent halo strip by a 90-degree rotation about the cube corner:
    at the south-west corner an x sweep sees q(i, j) = q(j, 1-i), a y sweep q(i, j) = q(1-j, i)."""
    n, ng = 12, 3
    g = G.tile_geometry(n, 0, ng)
    nd = n + 2 * ng
    rng = np.random.default_rng(0)
    q = rng.standard_normal((nd, nd))
    X = lambda a, i, j: a[j - 1 + ng, i - 1 + ng]  # noqa: E731
    for direction in (1, 2):
        qc = O.copy_corners(q, n, direction, g)
        for i in range(1 - ng, 1):
            for j in range(1 - ng, 1):
                want = X(q, j, 1 - i) if direction == 1 else X(q, 1 - j, i)
                assert X(qc, i, j) == want
        # the other corners are the mirror images: NE x sweep continues the east strip
        for i in range(n + 1, n + ng + 1):
            for j in range(n + 1, n + ng + 1):
                if direction == 1:
                    assert X(qc, i, j) == X(q, j, 2 * (n + 1) - 1 - i)
                else:
                    assert X(qc, i, j) == X(q, 2 * (n + 1) - 1 - j, i)
        interior_and_strips = np.ones((nd, nd), bool)
        for cj in (slice(0, ng), slice(n + ng, nd)):
            for ci in (slice(0, ng), slice(n + ng, nd)):
                interior_and_strips[cj, ci] = False
        assert np.array_equal(qc[interior_and_strips], q[interior_and_strips])


def _transpose_geom(g):
    """The same tile with i and j exchanged."""
    t = G.TileGeom(n=g.n, ng=g.ng, tile=g.tile, dx=g.dy.T.copy(), dy=g.dx.T.copy(), dxa=g.dya.T.copy(),
                   dya=g.dxa.T.copy(), area=g.area.T.copy(), rarea=g.rarea.T.copy(),
                   sin_sg=np.stack([g.sin_sg[1].T, g.sin_sg[0].T, g.sin_sg[3].T, g.sin_sg[2].T] +
                                   [s.T for s in g.sin_sg[4:]]).copy(),
                   corners=g.corners.transpose(1, 0, 2).copy(), centers=g.centers.transpose(1, 0, 2).copy())
    return t


@pytest.mark.parametrize("hord", [5, 8])
def test_x_sweep_on_transposed_data_equals_y_sweep(hord):
    P = S.make_problem(16, 1, 1, seed=9, ntiles=1)
    g = P.geoms[0]
    q = np.ascontiguousarray(P.q[0, 0, 0].numpy())
    cx, cy = P.cx[0, 0].numpy(), P.cy[0, 0].numpy()
    xfx, yfx = area_fluxes(cx, cy, g)
    rax, ray = ra_xy(xfx, yfx, g)
    mfx, mfy = P.mfx[0, 0].numpy(), P.mfy[0, 0].numpy()
    fx, fy, _ = O.fv_tp_2d(q, cx, cy, hord, xfx, yfx, g, rax, ray, mfx, mfy)
    gt = _transpose_geom(g)
    c = np.ascontiguousarray
    fxT, fyT, _ = O.fv_tp_2d(c(q.T), c(cy.T), c(cx.T), hord, c(yfx.T), c(xfx.T), gt, c(ray.T), c(rax.T), c(mfy.T),
                             c(mfx.T))
    assert np.allclose(fxT, fy.T, rtol=1e-14, atol=1e-14 * np.abs(fy).max())
    assert np.allclose(fyT, fx.T, rtol=1e-14, atol=1e-14 * np.abs(fx).max())


def test_tangent_linear_hord5_is_the_scheme_itself():
    """hord 5 is linear in q, so its tangent-linear model applied to dq equals fv_tp_2d(dq)."""
    P = S.make_problem(16, 1, 1, seed=2, ntiles=1)
    g = P.geoms[0]
    q = np.ascontiguousarray(P.q[0, 0, 0].numpy())
    dq = np.random.default_rng(3).standard_normal(q.shape)
    cx, cy = P.cx[0, 0].numpy(), P.cy[0, 0].numpy()
    xfx, yfx = area_fluxes(cx, cy, g)
    rax, ray = ra_xy(xfx, yfx, g)
    mfx, mfy = P.mfx[0, 0].numpy(), P.mfy[0, 0].numpy()
    dfx, dfy = O.fv_tp_2d_tl(q, dq, cx, cy, 5, xfx, yfx, g, rax, ray, mfx, mfy)
    fx, fy, _ = O.fv_tp_2d(dq, cx, cy, 5, xfx, yfx, g, rax, ray, mfx, mfy)
    assert np.allclose(dfx, fx, rtol=1e-12, atol=1e-12 * np.abs(fx).max())
    assert np.allclose(dfy, fy, rtol=1e-12, atol=1e-12 * np.abs(fy).max())


def test_tangent_linear_hord8_matches_finite_differences_on_a_monotone_field():
    """hord 8 is not differentiable at flat spots and extrema (its limiter switches branch there), so the
    finite-difference check runs on a strictly monotone trajectory; hord 5 is the FD reference scheme."""
    P = S.make_problem(16, 1, 1, seed=5, ntiles=1, noise=0.0)
    g = P.geoms[0]
    nd = P.nd
    jj, ii = np.meshgrid(np.arange(nd), np.arange(nd), indexing="ij")
    q = np.ascontiguousarray(1.0 + 0.013 * ii + 0.021 * jj + 0.0007 * ii * ii + 0.0004 * jj * jj)
    dq = np.random.default_rng(4).standard_normal(q.shape)
    cx, cy = P.cx[0, 0].numpy(), P.cy[0, 0].numpy()
    xfx, yfx = area_fluxes(cx, cy, g)
    rax, ray = ra_xy(xfx, yfx, g)
    mfx, mfy = P.mfx[0, 0].numpy(), P.mfy[0, 0].numpy()
    dfx, dfy = O.fv_tp_2d_tl(q, dq, cx, cy, 8, xfx, yfx, g, rax, ray, mfx, mfy)
    f0x, f0y, _ = O.fv_tp_2d(q, cx, cy, 8, xfx, yfx, g, rax, ray, mfx, mfy)
    errs = []
    for eps in (1e-4, 1e-5, 1e-6, 1e-7, 1e-8):
        f1x, f1y, _ = O.fv_tp_2d(q + eps * dq, cx, cy, 8, xfx, yfx, g, rax, ray, mfx, mfy)
        errs.append(max(np.linalg.norm((f1x - f0x) / eps - dfx) / np.linalg.norm(dfx),
                        np.linalg.norm((f1y - f0y) / eps - dfy) / np.linalg.norm(dfy)))
    assert min(errs) < 1e-6, errs
