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


def _cube(P, hord=8, q_split=3, sync=False, q=None):
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


def _edge_flux_mismatch(P, geoms):
    """Largest |outflux of tile t + outflux of its neighbour| over every shared tile-edge face after one
    fv_tp_2d of each tile (halo strips of q from the neighbours), relative to the largest edge flux."""
    n = P.n
    qh = O.cube_halo_fill(P.q.numpy(), n, P.topo)[:, 0, 0]
    FX, FY = [], []
    for t in range(6):
        g = geoms[t]
        cx, cy = P.cx.numpy()[t, 0], P.cy.numpy()[t, 0]
        xf, yf = area_fluxes(cx, cy, g)
        rax, ray = ra_xy(xf, yf, g)
        fx, fy, _ = O.fv_tp_2d(qh[t], cx, cy, 8, xf, yf, g, rax, ray, mfx=P.mfx.numpy()[t, 0],
                               mfy=P.mfy.numpy()[t, 0])
        FX.append(fx)
        FY.append(fy)

    def out(t, e, s):
        return (-FX[t][s, 0], FX[t][s, n], -FY[t][0, s], FY[t][n, s])[e]

    worst, scale = 0.0, 0.0
    for t in range(6):
        for e in range(4):
            nt, ne, rev = (int(v) for v in P.topo[t, e])
            for s in range(n):
                a, b = out(t, e, s), out(nt, ne, n - 1 - s if rev else s)
                worst = max(worst, abs(a + b))
                scale = max(scale, abs(a))
    return worst / scale


def test_neighbour_halos_make_every_edge_flux_single_valued():
    """With halos that hold the neighbouring tiles' cells (their q, metrics and Courant numbers, rotated into
    the tile's directions; cube-corner cells by the copy_corners rotation), the two tiles beside a cube edge
    compute the same flux through every shared face, corners included, to round-off."""
    P = S.make_problem(24, 1, 1, seed=1, cmax=0.5)
    assert _edge_flux_mismatch(P, P.geoms) <= 1e-14


def test_extended_grid_halo_metrics_break_the_edge_fluxes():
    """The same problem with each face's halo metrics taken from its own extended gnomonic grid (not the
    neighbours' cells): the tiles' edge fluxes then disagree at the level of the truncation error."""
    P = S.make_problem(24, 1, 1, seed=1, cmax=0.5)
    own = [G.tile_geometry(P.n, t, P.ng) for t in range(6)]
    assert _edge_flux_mismatch(P, own) > 1e-6


def test_edge_reconciliation_changes_only_round_off(prob):
    """The optional tile-edge reconciliation (each shared face takes the upwind tile's flux) moves the result by
    round-off only, and both forms conserve the global tracer mass."""
    P = prob
    q0, dp0, ns = _cube(P, sync=False)
    q1, dp1, _ = _cube(P, sync=True)
    assert np.abs(interior(q1, P.n) - interior(q0, P.n)).max() <= 1e-14 * np.abs(interior(q0, P.n)).max()
    m0 = cube_mass(P.q.numpy(), P.dp.numpy(), P.geoms, P.n)
    for q, dpl in ((q0, dp0), (q1, dp1)):
        m1 = cube_mass(q, final_dp(dpl, P.mfx.numpy(), P.mfy.numpy(), P.geoms, ns, P.n), P.geoms, P.n)
        assert np.all(np.abs(m1 - m0) <= 1e-13 * np.abs(m0))


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
                   corners=g.corners.transpose(1, 0, 2).copy(), centers=g.centers.transpose(1, 0, 2).copy(),
                   del6_u=g.del6_v.T.copy(), del6_v=g.del6_u.T.copy())
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


def _tile_args(P, t=0, k=0):
    g = P.geoms[t]
    cx, cy = P.cx[t, k].numpy(), P.cy[t, k].numpy()
    xfx, yfx = area_fluxes(cx, cy, g)
    rax, ray = ra_xy(xfx, yfx, g)
    return g, cx, cy, xfx, yfx, rax, ray, P.mfx[t, k].numpy(), P.mfy[t, k].numpy()


def test_tangent_linear_hord5_is_linear_in_the_perturbation():
    """hord 5 is piecewise linear in q (its 2-dx filter switches); with the filter frozen at the
    trajectory the tangent-linear model is a linear map of dq."""
    P = S.make_problem(16, 1, 1, seed=2, ntiles=1)
    g, cx, cy, xfx, yfx, rax, ray, mfx, mfy = _tile_args(P)
    q = np.ascontiguousarray(P.q[0, 0, 0].numpy())
    rng = np.random.default_rng(3)
    x, y = rng.standard_normal(q.shape), rng.standard_normal(q.shape)
    tl = [O.fv_tp_2d_tl(q, d, cx, cy, 5, xfx, yfx, g, rax, ray, mfx, mfy) for d in (x, y, 2.0 * x - 3.0 * y)]
    for c in range(2):
        want = 2.0 * tl[0][c] - 3.0 * tl[1][c]
        assert np.allclose(tl[2][c], want, rtol=1e-12, atol=1e-12 * np.abs(want).max())


@pytest.mark.parametrize("hord", [1, 5])
def test_two_dx_filter_gives_first_order_fluxes_on_a_checkerboard(hord):
    """On q = 1 + a (-1)^i (constant in j) every cell is an extremum (bl = br), so hord 5 and hord 1 drop
    the parabola's correction: away from the cube edges the x flux is the upwind value times mfx."""
    P = S.make_problem(16, 1, 1, seed=4, ntiles=1)
    g, cx, cy, xfx, yfx, rax, ray, mfx, mfy = _tile_args(P)
    nd, n, ng = P.nd, P.n, 3
    i = np.arange(nd)[None, :] + np.zeros((nd, 1))
    q = np.ascontiguousarray(1.0 + 0.1 * (-1.0) ** i)
    fx, _, _ = O.fv_tp_2d(q, cx, cy, hord, xfx, yfx, g, rax, ray, mfx, mfy, lim_fac=2.0)
    c = cx[ng:ng + n, :]                                  # (n rows, n+1 faces)
    up = np.where(c > 0, q[ng:ng + n, ng - 1:ng + n], q[ng:ng + n, ng:ng + n + 1])
    sl = slice(3, n - 2)                                  # faces 4 .. n-2
    assert np.allclose(fx[:, sl], (up * mfx)[:, sl], rtol=1e-13, atol=0)
    # hord 8 on the same field: the limiter flattens every cell as well
    fx8, _, _ = O.fv_tp_2d(q, cx, cy, 8, xfx, yfx, g, rax, ray, mfx, mfy)
    assert np.allclose(fx8[:, sl], (up * mfx)[:, sl], rtol=1e-13, atol=0)


def test_hord1_with_lim_fac_1_is_hord5():
    """|b0| < |bl - br| is bl br < 0: hord 1 with lim_fac 1 reproduces hord 5; lim_fac 3 filters more."""
    P = S.make_problem(16, 1, 1, seed=6, ntiles=1)
    g, cx, cy, xfx, yfx, rax, ray, mfx, mfy = _tile_args(P)
    q = np.ascontiguousarray(P.q[0, 0, 0].numpy())
    f5 = O.fv_tp_2d(q, cx, cy, 5, xfx, yfx, g, rax, ray, mfx, mfy)
    f1 = O.fv_tp_2d(q, cx, cy, 1, xfx, yfx, g, rax, ray, mfx, mfy, lim_fac=1.0)
    f3 = O.fv_tp_2d(q, cx, cy, 1, xfx, yfx, g, rax, ray, mfx, mfy, lim_fac=3.0)
    assert np.array_equal(f5[0], f1[0]) and np.array_equal(f5[1], f1[1])
    assert not np.array_equal(f5[0], f3[0])


def _laplacian_fluxes(d2, g, ng=3):
    """x and y fluxes del6 * (d2 upwind-side difference) on the whole data domain (NaN where undefined)."""
    nd = d2.shape[0]
    fx = np.full((nd, nd + 1), np.nan)
    fy = np.full((nd + 1, nd), np.nan)
    fx[:, 1:nd] = g.del6_v[:, 1:nd] * (d2[:, :-1] - d2[:, 1:])
    fy[1:nd, :] = g.del6_u[1:nd, :] * (d2[:-1, :] - d2[1:, :])
    return fx, fy


@pytest.mark.parametrize("nord", [0, 1, 2])
def test_damping_fluxes_are_powers_of_the_discrete_laplacian(nord):
    """Without winds or mass, fv_tp_2d's fluxes are the del-2(nord+1) damping fluxes alone.  Restated here
    with numpy: F0 = del6 * (d(i-1) - d(i)) on d = damp q; each order replaces d by div F * rarea and takes
    the difference the other way.  (nested: no cube-edge or corner treatment.)"""
    P = S.make_problem(16, 1, 1, seed=8, ntiles=1)
    g = P.geoms[0]
    nd, n, ng = P.nd, P.n, 3
    q = np.ascontiguousarray(P.q[0, 0, 0].numpy())
    z = lambda shp: np.zeros(shp)
    cx, cy, xfx, yfx = z((nd, n + 1)), z((n + 1, nd)), z((nd, n + 1)), z((n + 1, nd))
    rax, ray = ra_xy(xfx, yfx, g)
    damp_c = 0.07
    da = float(g.area[ng:ng + n, ng:ng + n].min())
    damp = (damp_c * da) ** (nord + 1)
    fx, fy, _ = O.fv_tp_2d(q, cx, cy, 8, xfx, yfx, g, rax, ray, nord=nord, damp_c=damp_c, nested=1, da_min=da)
    d2 = damp * q
    Fx, Fy = _laplacian_fluxes(d2, g)
    for _ in range(nord):
        d2 = (Fx[:, :-1] - Fx[:, 1:] + Fy[:-1, :] - Fy[1:, :]) * g.rarea
        Fx, Fy = _laplacian_fluxes(d2, g)
        Fx, Fy = -Fx, -Fy
    s = slice(ng, ng + n)
    wx, wy = Fx[s, ng:ng + n + 1], Fy[ng:ng + n + 1, s]
    assert np.allclose(fx, wx, rtol=1e-12, atol=1e-12 * np.abs(wx).max())
    assert np.allclose(fy, wy, rtol=1e-12, atol=1e-12 * np.abs(wy).max())
    if nord == 0:  # a del-2 flux runs down the gradient
        assert np.all(fx * (q[s, ng - 1:ng + n] - q[s, ng:ng + n + 1]) >= 0)


@pytest.mark.parametrize("nord,trdm", [(0, 0.12), (1, 0.1), (2, 0.1)])
def test_damped_transport_conserves_mass_and_smooths(prob, nord, trdm):
    P = prob
    q0, dp_last0, ns = O.tracer_2d_cube(P.q, P.dp, P.mfx, P.mfy, P.cx, P.cy, P.geoms, P.topo, hord=8, q_split=3)
    q1, dp_last, ns1 = O.tracer_2d_cube(P.q, P.dp, P.mfx, P.mfy, P.cx, P.cy, P.geoms, P.topo, hord=8, q_split=3,
                                        nord_tr=nord, trdm=trdm)
    assert ns1 == ns and np.array_equal(dp_last, dp_last0)  # damping moves tracer mass only
    dpf = final_dp(dp_last, P.mfx.numpy(), P.mfy.numpy(), P.geoms, ns, P.n)
    m0 = cube_mass(P.q.numpy(), P.dp.numpy(), P.geoms, P.n)
    m1 = cube_mass(q1, dpf, P.geoms, P.n)
    assert np.all(np.abs(m1 - m0) <= 1e-13 * np.abs(m0)), (m1 - m0) / m0
    # the damped field has less grid-scale variance than the undamped one
    def roughness(q):
        qi = interior(q, P.n)
        return float(np.sum(np.diff(qi, axis=-1) ** 2) + np.sum(np.diff(qi, axis=-2) ** 2))
    assert roughness(q1) < roughness(q0)


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


def _level_scaled(P, factors):
    """The single-tile problem's winds and mass fluxes scaled per level (Courant maxima differ by level)."""
    f = np.asarray(factors, dtype=np.float64)
    args = [np.ascontiguousarray(a[0].numpy()) for a in (P.q, P.dp, P.mfx, P.mfy, P.cx, P.cy)]
    for idx in (2, 3, 4, 5):
        args[idx] = np.ascontiguousarray(args[idx] * f[:, None, None])
    return args


def test_tracer_2d_1L_is_tracer_2d_level_by_level():
    """tracer_2d_1L advances each level with its own substep count: level k equals a one-level tracer_2d call."""
    P = S.make_problem(24, 4, 2, seed=3, cmax=0.9, ntiles=1)
    args = _level_scaled(P, [0.5, 1.5, 2.5, 1.0])
    q, dp, mfx, mfy, cx, cy, ns = O.tracer_2d_1L(*args, P.geoms[0], hord=8)
    assert len(set(ns.tolist())) > 1, ns
    for k in range(P.npz):
        one = [args[0][:, k:k + 1]] + [a[k:k + 1] for a in args[1:]]
        r = O.tracer_2d(*[np.ascontiguousarray(a) for a in one], P.geoms[0], hord=8)
        assert r[6] == ns[k]
        assert np.array_equal(q[:, k], r[0][:, 0]) and np.array_equal(dp[k], r[1][0])
    # a fixed q_split gives tracer_2d itself
    a1 = O.tracer_2d_1L(*args, P.geoms[0], hord=8, q_split=3)
    a2 = O.tracer_2d(*args, P.geoms[0], hord=8, q_split=3)
    assert np.array_equal(a1[0], a2[0]) and np.array_equal(a1[1], a2[1])
