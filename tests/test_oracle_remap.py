"""Known-answer and property tests of the CPU oracle's column remap (no GPU)."""
import numpy as np
import pytest

import oracle as O
from fv3atm_gb300 import grid as G


def _column(km=127, seed=0, ps=101000.0, noise=0.1):
    rng = np.random.default_rng(seed)
    ak, bk = G.hybrid_levels(km)
    dref = np.diff(ak + bk * ps)
    dp = dref * (1 + noise * rng.uniform(-1, 1, km))
    dp *= dref.sum() / dp.sum()
    pe1 = np.concatenate([[ak[0]], ak[0] + np.cumsum(dp)])
    pe2 = ak + bk * pe1[-1]
    return pe1, pe2, rng


@pytest.mark.parametrize("kord", [4, 9])
def test_identity_remap_is_exact(kord):
    pe1, _, rng = _column()
    q = rng.uniform(0, 1, 127)
    assert np.array_equal(O.remap_column(pe1, q, pe1, kord=kord), q)


@pytest.mark.parametrize("kord", [4, 9])
def test_constant_preserved_and_mass_conserved(kord):
    pe1, pe2, rng = _column(seed=1)
    assert np.abs(O.remap_column(pe1, np.full(127, 3.25), pe2, kord=kord) - 3.25).max() <= 1e-14
    q = np.abs(np.sin(np.linspace(0, 7, 127))) + 0.01 * rng.uniform(0, 1, 127)
    q2 = O.remap_column(pe1, q, pe2, kord=kord)
    m1, m2 = (q * np.diff(pe1)).sum(), (q2 * np.diff(pe2)).sum()
    assert abs(m2 - m1) <= 1e-14 * m1


def test_kord9_keeps_monotone_columns_monotone():
    """On a monotone column every interface is clamped into its two means and no layer is an extremum, so the
    kord 9 remap is monotone and stays within the source range."""
    for seed in range(10):
        pe1, pe2, rng = _column(seed=seed)
        q = np.sort(rng.uniform(0, 1, 127)) * (1 if seed % 2 else -1)
        q2 = O.remap_column(pe1, q, pe2, kord=9)
        d = np.diff(q2) * (1 if seed % 2 else -1)
        assert d.min() >= 0.0
        assert q2.min() >= q.min() - 1e-15 and q2.max() <= q.max() + 1e-15


def test_kord9_flattens_two_grid_waves():
    """Interior layers that are extrema next to other extrema (a two-grid-length wave) are flat."""
    pe1, _, rng = _column(seed=2)
    q = 1.0 + 0.3 * (-1.0) ** np.arange(127) + 0.01 * rng.uniform(0, 1, 127)
    a4 = O.column_profile(q, np.diff(pe1), iv=0, kord=9)
    inner = slice(2, 125)
    assert np.array_equal(a4[inner, 1], q[inner]) and np.array_equal(a4[inner, 2], q[inner])
    assert np.all(a4[inner, 3] == 0.0)


def test_kord9_lets_a_smooth_peak_pass_its_mean():
    """Huynh's constraint keeps a resolved smooth extremum: the peak layer's edges may exceed its mean (a clamp
    to the neighbouring means would cut the peak flat), bounded by the upper-limit value q + 2 D."""
    km = 63
    pe1, _, _ = _column(km=km, seed=3, noise=0.0)
    x = (np.arange(km) - 31.3) / 6.0
    q = np.exp(-x * x)
    a4 = O.column_profile(q, np.diff(pe1), iv=0, kord=9)
    k = int(np.argmax(q))
    assert max(a4[k, 1], a4[k, 2]) > q[k]
    assert a4[k, 2] <= q[k] + 2.0 * (q[k] - q[k - 1]) + 1e-15 or a4[k, 2] <= q[k]
    q2 = O.remap_column(pe1, q, pe1, kord=9)
    assert np.array_equal(q2, q)


@pytest.mark.parametrize("kord", [9, 4])
def test_positivity_limiter_is_continuous(kord):
    """The iv >= 0 floor scales a layer's deviations instead of switching the layer to a flat profile, so the
    remap is continuous in q: a perturbation of 1e-10 (relative) moves no value by more than 1e-8 of the range,
    on columns with many local minima next to the floor (a switch there moved single values by O(1))."""
    for seed in range(6):
        pe1, pe2, rng = _column(seed=40 + seed)
        q = np.maximum(rng.uniform(-0.3, 1.0, 127), 0.0) ** 2
        q2 = O.remap_column(pe1, q, pe2, iv=0, kord=kord)
        qp = q * (1.0 + 1e-10 * rng.standard_normal(127))
        q2p = O.remap_column(pe1, qp, pe2, iv=0, kord=kord)
        assert np.abs(q2p - q2).max() <= 1e-8 * q.max()
        assert q2.min() >= -1e-15


def _profile_np(q, dp, iv=0, kord=9, qs=0.0, q_min=0.0):
    """An independent numpy restatement of the column reconstruction (the same published constraints as the
    oracle's column_profile_t, written loop by loop) used to check the C++ oracle."""
    km = len(q)
    floor = q_min if iv == 1 else 0.0
    a = np.zeros(km + 1)
    dm = np.zeros(km)
    D = np.concatenate([[np.nan], np.diff(q)])  # D[u] = q[u] - q[u-1]
    if kord >= 7:
        A = np.zeros((km + 1, km + 1))
        r = np.zeros(km + 1)
        g = dp[1] / dp[0]
        A[0, 0], A[0, 1], r[0] = g, g + 1, (g * (2 * g + 3) * q[0] + q[1]) / (g + 1)
        for k in range(1, km):
            d = dp[k - 1] / dp[k]
            A[k, k - 1], A[k, k], A[k, k + 1], r[k] = 1.0, 2 * (1 + d), d, 3 * (q[k - 1] + d * q[k])
        if iv == -2:
            A[km, km], r[km] = 1.0, qs
        else:
            gb = dp[km - 2] / dp[km - 1]
            A[km, km - 1], A[km, km], r[km] = gb + 1, gb, (gb * (2 * gb + 3) * q[km - 1] + q[km - 2]) / (gb + 1)
        a = np.linalg.solve(A, r)
        a[0] = np.clip(a[0], min(q[0], q[1]), max(q[0], q[1]))
        for u in range(1, km):
            dl, dr = D[max(u - 1, 1) if u > 1 else u], D[u + 1 if u < km - 1 else u]
            lo, hi = min(q[u - 1], q[u]), max(q[u - 1], q[u])
            if dl * dr > 0:
                a[u] = min(max(a[u], lo), hi)
            elif dl > 0:
                a[u] = max(a[u], lo)
            else:
                a[u] = min(a[u], hi)
                if iv >= 0:
                    a[u] = max(a[u], floor)
        if iv != -2:
            a[km] = np.clip(a[km], min(q[km - 2], q[km - 1]), max(q[km - 2], q[km - 1]))
    else:
        for k in range(1, km - 1):
            d0, d1, d2 = dp[k - 1], dp[k], dp[k + 1]
            dq = d1 / (d0 + d1 + d2) * ((2 * d0 + d1) / (d2 + d1) * (q[k + 1] - q[k]) +
                                        (d1 + 2 * d2) / (d0 + d1) * (q[k] - q[k - 1]))
            nb = q[k - 1:k + 2]
            dm[k] = np.copysign(min(0.5 * abs(dq), nb.max() - q[k], q[k] - nb.min()), dq)
        for u in range(2, km - 1):
            j = u - 1
            h = dp[j - 1:j + 3]
            # CW84 eq. 1.6 written with the full increments 2 dm
            t1 = h[1] / (h[1] + h[2]) * (q[j + 1] - q[j])
            t2 = 2 * h[2] * h[1] / (h[1] + h[2]) * ((h[0] + h[1]) / (2 * h[1] + h[2]) -
                                                    (h[3] + h[2]) / (2 * h[2] + h[1])) * (q[j + 1] - q[j])
            t3 = -h[1] * (h[0] + h[1]) / (2 * h[1] + h[2]) * 2 * dm[j + 1]
            t4 = h[2] * (h[2] + h[3]) / (h[1] + 2 * h[2]) * 2 * dm[j]
            a[u] = q[j] + t1 + (t2 + t3 + t4) / h.sum()

        def quad(q0, q1, q2, h0, h1, h2):  # parabola through three layer means, at the end layer's inner edge
            x = np.array([0.0, h0, h0 + h1, h0 + h1 + h2])
            m = np.array([0.0, q0 * h0, q0 * h0 + q1 * h1, q0 * h0 + q1 * h1 + q2 * h2])
            return np.polyval(np.polyder(np.polyfit(x, m, 3)), h0)
        a[1] = np.clip(quad(q[0], q[1], q[2], *dp[:3]), min(q[0], q[1]), max(q[0], q[1]))
        a[km - 1] = np.clip(quad(q[km - 1], q[km - 2], q[km - 3], dp[km - 1], dp[km - 2], dp[km - 3]),
                            min(q[km - 2], q[km - 1]), max(q[km - 2], q[km - 1]))
        a[0] = 2 * q[0] - a[1]
        a[km] = qs if iv == -2 else 2 * q[km - 1] - a[km - 1]
    out = np.zeros((km, 4))
    for k in range(km):
        bl, br = a[k] - q[k], a[k + 1] - q[k]
        if k < 2 or k > km - 3:
            if bl * br >= 0:
                bl = br = 0.0
            else:
                t, d2 = 3 * (br - bl) * (bl + br), (br - bl) ** 2
                if -t > d2:
                    bl = -2 * br
                elif t > d2:
                    br = -2 * bl
        elif kord >= 7:
            extm = [D[i] * D[i + 1] < 0 if 1 <= i <= km - 2 else False for i in (k - 1, k, k + 1)]
            if extm[1] and (extm[0] or extm[2]):
                bl = br = 0.0
            elif 3 * abs(bl + br) > abs(br - bl):
                pr = 2 * D[k]
                lr = pr - 1.5 * D[k - 1]
                pl = -2 * D[k + 1]
                ll = pl + 1.5 * D[k + 2]
                br = min(max(br, min(0.0, pr, lr)), max(0.0, pr, lr))
                bl = min(max(bl, min(0.0, pl, ll)), max(0.0, pl, ll))
        else:
            xt = 2 * dm[k]
            bl = -np.copysign(min(abs(xt), abs(bl)), xt)
            br = np.copysign(min(abs(xt), abs(br)), xt)
        if iv >= 0:  # scale the deviations so that the minimum reaches the floor
            s6, da = -3 * (bl + br), br - bl
            pmin = min(q[k] + bl, q[k] + br)
            if -s6 > abs(da):
                pmin = min(pmin, q[k] + s6 / 12 + da * da / (4 * s6))  # the parabola's interior minimum
            if pmin < floor:
                lam = (q[k] - floor) / (q[k] - pmin) if q[k] > floor else 0.0
                bl, br = lam * bl, lam * br
        out[k] = (q[k], q[k] + bl, q[k] + br, -3 * (bl + br))
    return out


@pytest.mark.parametrize("kord,iv", [(9, 0), (9, 1), (9, -1), (9, -2), (4, 0), (4, 1), (4, -1), (4, -2)])
def test_column_profile_matches_numpy_restatement(kord, iv):
    for seed in range(4):
        km = (63, 127, 32, 7)[seed]
        pe1, _, rng = _column(km=km, seed=10 + seed)
        dp = np.diff(pe1)
        kind = seed % 3
        q = (rng.uniform(0, 1, km) if kind == 0 else np.sin(np.linspace(0, 5, km)) + 0.05 * rng.uniform(0, 1, km)
             if kind == 1 else rng.standard_normal(km).cumsum() * 0.1)
        if iv >= 0:
            q = np.abs(q) + (0.06 if iv == 1 else 0.0)
        got = O.column_profile(q, dp, iv=iv, kord=kord, qs=float(q[-1]) * 1.1, q_min=0.05)
        want = _profile_np(q, dp, iv=iv, kord=kord, qs=float(q[-1]) * 1.1, q_min=0.05)
        scale = np.abs(q).max()
        assert np.abs(got - want).max() <= 1e-12 * scale, (seed, np.abs(got - want).max())


@pytest.mark.parametrize("order", [1, 2])
def test_kord4_exact_for_linear_and_quadratic_profiles(order):
    pe1, pe2, _ = _column(seed=3, noise=0.05)
    x1 = pe1 / pe1[-1]
    x2 = pe2 / pe2[-1]

    def mean(x, p):  # exact layer means of 2 + x + 0.5 x^2 (order 2) or 2 + x (order 1)
        F = 2 * x + x ** 2 / 2 + (x ** 3 / 6 if order == 2 else 0)
        return np.diff(F) / np.diff(x)

    q2 = O.remap_column(pe1, mean(x1, pe1), pe2, kord=4)
    assert np.abs(q2 - mean(x2, pe2)).max() <= 1e-12


def test_kord9_exact_for_linear_away_from_the_boundaries():
    pe1, pe2, _ = _column(seed=4, noise=0.05)
    x1, x2 = pe1 / pe1[-1], pe2 / pe2[-1]
    mean = lambda x: np.diff(2 * x + x ** 2 / 2) / np.diff(x)  # noqa: E731
    q2 = O.remap_column(pe1, mean(x1), pe2, kord=9)
    assert np.abs(q2 - mean(x2))[3:-3].max() <= 1e-12


def test_iv_floor_keeps_reconstruction_above_floor():
    pe1, pe2, rng = _column(seed=5)
    q = 0.01 + np.abs(rng.standard_normal(127)) * 0.05
    for iv, floor in ((1, 0.01), (0, 0.0)):
        a4 = O.column_profile(q, np.diff(pe1), iv=iv, kord=4, q_min=floor)
        assert a4[:, 1:3].min() >= floor - 1e-15
        q2 = O.remap_column(pe1, q, pe2, iv=iv, kord=4, q_min=floor)
        assert q2.min() >= floor - 1e-15


def test_iv_minus2_imposes_the_surface_value():
    pe1, _, _ = _column(seed=6)
    col = np.linspace(0.1, 0.2, 127)
    qs = 0.2 + 0.5 * 0.1 / 126
    a4 = O.column_profile(col, np.diff(pe1), iv=-2, kord=4, qs=qs)
    assert abs(a4[-1, 2] - qs) <= 1e-12


def test_map_scalar_row_matches_columns():
    km, ni, nj = 32, 9, 4
    rng = np.random.default_rng(8)
    ak, bk = G.hybrid_levels(km)
    ps = rng.uniform(95000, 103000, (nj, ni))
    dp = (np.diff(ak)[:, None, None] + np.diff(bk)[:, None, None] * ps[None]) * (1 + 0.1 * rng.uniform(-1, 1, (km, nj, ni)))
    pe1 = np.concatenate([np.full((1, nj, ni), ak[0]), ak[0] + np.cumsum(dp, 0)])
    pe2 = ak[:, None, None] + bk[:, None, None] * pe1[-1][None]
    q1 = np.ascontiguousarray(rng.uniform(0, 1, (km, nj, ni)))
    j = 2
    out = O.map_scalar(km, np.ascontiguousarray(pe1[:, j, 1:8]), q1, None, km, np.ascontiguousarray(pe2[:, j, 1:8]),
                       np.zeros_like(q1), 2, 8, j + 1, 1, ni, 1, nj, 0, 9, 0.0)
    for i in range(1, 8):
        ref = O.remap_column(pe1[:, j, i], q1[:, j, i], pe2[:, j, i], kord=9)
        assert np.array_equal(out[:, j, i], ref)


@pytest.mark.parametrize("kord", [4, 9])
def test_map1_q2_divides_the_overlap_mass_by_dp2(kord):
    """map1_q2 (dp2 given): with dp2 the pe2 differences it is the plain remap; with dp2 doubled, a target
    layer spanning several source layers halves (its overlap mass over dp2) and one inside a single source
    layer keeps its mean."""
    rng = np.random.default_rng(31)
    km, kn, ncol = 40, 25, 12
    pe1 = np.zeros((km + 1, ncol))
    pe1[0] = 100.0
    pe1[1:] = 100.0 + np.cumsum(rng.uniform(200.0, 800.0, (km, ncol)), axis=0)
    pe2 = np.linspace(0.0, 1.0, kn + 1)[:, None] * (pe1[-1] - pe1[0]) + pe1[0]
    pe2[-1] = pe1[-1]
    q1 = rng.uniform(0.5, 1.5, (km, ncol))
    plain = O.remap_columns(pe1, q1, pe2, iv=0, kord=kord)
    assert np.allclose(O.remap_columns(pe1, q1, pe2, iv=0, kord=kord, dp2=np.diff(pe2, axis=0)), plain, rtol=0,
                       atol=1e-15)
    doubled = O.remap_columns(pe1, q1, pe2, iv=0, kord=kord, dp2=2.0 * np.diff(pe2, axis=0))
    for c in range(ncol):
        for k2 in range(kn):
            spans = np.searchsorted(pe1[:, c], pe2[k2, c], side="right") != np.searchsorted(pe1[:, c],
                                                                                           pe2[k2 + 1, c], side="left")
            want = 0.5 * plain[k2, c] if spans else plain[k2, c]
            assert doubled[k2, c] == pytest.approx(want, rel=1e-14), (c, k2)
