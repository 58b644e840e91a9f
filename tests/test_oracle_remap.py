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


def test_kord9_creates_no_new_extrema():
    for seed in range(5):
        pe1, pe2, rng = _column(seed=seed)
        q = rng.standard_normal(127).cumsum() * 0.1 + rng.uniform(0, 1, 127)
        q2 = O.remap_column(pe1, q, pe2, kord=9)
        assert q2.min() >= q.min() - 1e-14 and q2.max() <= q.max() + 1e-14


def test_kord9_monotone_within_the_local_range():
    """Every target value lies within the range of the source layers it overlaps (plus neighbours)."""
    pe1, pe2, rng = _column(seed=7)
    q = rng.uniform(0, 1, 127)
    q2 = O.remap_column(pe1, q, pe2, kord=9)
    for k in range(127):
        lo = np.searchsorted(pe1, pe2[k], side="right") - 2
        hi = np.searchsorted(pe1, pe2[k + 1], side="left") + 1
        seg = q[max(lo, 0):min(hi, 127)]
        assert seg.min() - 1e-14 <= q2[k] <= seg.max() + 1e-14


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
