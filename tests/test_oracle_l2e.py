"""Properties of the oracle's fillz and pressure-variable recompute (no GPU)."""
import numpy as np

import oracle as O


def _columns(seed=0, km=20, im=7, nq=3, neg=0.3):
    rng = np.random.default_rng(seed)
    dp = rng.uniform(50.0, 900.0, (km, im))
    q = rng.uniform(0.0, 1.0, (nq, km, im))
    q[rng.uniform(size=q.shape) < neg] *= -0.4  # scattered negatives
    return q, dp


def test_fillz_conserves_column_mass_and_removes_negatives():
    q, dp = _columns()
    f = O.fillz(q, dp)
    m0, m1 = (q * dp).sum(1), (f * dp).sum(1)
    assert np.all(np.abs(m1 - m0) <= 1e-13 * np.abs(q * dp).sum(1))
    pos_cols = m0 > 0
    assert np.all(f.transpose(0, 2, 1)[pos_cols] >= 0.0)


def test_fillz_leaves_non_negative_columns_unchanged():
    q, dp = _columns(seed=1, neg=0.0)
    assert np.array_equal(O.fillz(q, dp), q)


def test_fillz_borrows_locally_before_the_column_fix():
    dp = np.full((4, 1), 100.0)
    q = np.array([[[0.5], [-0.2], [0.5], [0.5]]])
    f = O.fillz(q, dp)[0, :, 0]
    assert np.allclose(f, [0.3, 0.0, 0.5, 0.5])  # the deficit came from the layer above only


def test_pressure_vars_known_answers():
    dp = np.array([[100.0], [300.0], [600.0]])
    pe, peln, pk, pkz = O.pressure_vars(dp, 200.0, 0.25)
    assert np.allclose(pe[:, 0], [200.0, 300.0, 600.0, 1200.0])
    assert np.allclose(peln, np.log(pe)) and np.allclose(pk, pe ** 0.25)
    # pkz is the mean of p^kappa over ln p across the layer: between the edge values
    assert np.all((pkz > pk[:-1]) & (pkz < pk[1:]))
