"""tracer_2d_nested in the oracle (CPU): the boundary states of a nested grid, interpolated in time, set the
outer-side halo before every substep.  nested_grid_BC_apply_intT's region rules and the substep count that
drives the interpolation are checked directly, and the whole call against tracer_2d with a halo callback that
applies the same states in numpy."""
import numpy as np
import pytest

import oracle as O
from fv3atm_gb300 import synth as S

from ._helpers import interior, sub_domain

NG = 3


@pytest.fixture(scope="module")
def prob():
    return S.make_problem(20, 3, 2, seed=21, cmax=0.9, ntiles=1)


def _args(P):
    return [np.ascontiguousarray(a[0].numpy()) for a in (P.q, P.dp, P.mfx, P.mfy, P.cx, P.cy)]


def _later(f):
    """A boundary state at the parent's t1 that differs from t0 everywhere."""
    return f * 1.25 + 0.05


def _blend(f0, f1, step, split):
    return (f0 * (split - step) + step * f1) * (1.0 / split)


def _ring(nd_j, nd_i, n_j, n_i):
    r = np.ones((nd_j, nd_i), bool)
    r[NG:NG + n_j, NG:NG + n_i] = False
    return r


def test_bc_apply_sets_the_whole_ring_and_interpolates_linearly():
    n = 12
    nd = n + 2 * NG
    rng = np.random.default_rng(3)
    f0, f1 = rng.standard_normal((1, 2, nd, nd)), rng.standard_normal((1, 2, nd, nd))
    bc = S.nest_strips(f0, f1, 1 - NG, 1 - NG, n + 1, n + 1)
    var = np.full((2, nd, nd), 7.0)
    ring = _ring(nd, nd, n, n)
    for step, split in ((0, 4), (4, 4), (1, 4), (5, 6)):
        got = O.nest_bc_apply(var, bc, step, split, O.bounds_for(n), n + 1, n + 1)
        assert np.array_equal(got[:, ~ring], var[:, ~ring])
        assert np.array_equal(got[:, ring], _blend(f0[0], f1[0], step, split)[:, ring])
    assert np.array_equal(O.nest_bc_apply(var, bc, 0, 4, O.bounds_for(n), n + 1, n + 1)[:, ring], f0[0][:, ring])


def test_bc_apply_reads_only_the_outer_sides_of_a_rank():
    """A rank with the nest's west and north sides (is = 1, je = npy-1) but a neighbour to the east and south:
    west over the full height, north over i = is..ied (the corner toward the east neighbour included), nothing
    else."""
    n, is_, ie, js, je = 12, 1, 6, 4, 12
    bd = O.Bounds(is_, ie, js, je, is_ - NG, ie + NG, js - NG, je + NG, NG)
    nid, njd = ie - is_ + 1 + 2 * NG, je - js + 1 + 2 * NG
    rng = np.random.default_rng(5)
    f0, f1 = rng.standard_normal((1, 1, njd, nid)), rng.standard_normal((1, 1, njd, nid))
    bc = S.nest_strips(f0, f1, bd.isd, bd.jsd, n + 1, n + 1)
    var = np.full((1, njd, nid), 7.0)
    got = O.nest_bc_apply(var, bc, 1, 3, bd, n + 1, n + 1)[0]
    want_set = np.zeros((njd, nid), bool)
    want_set[:, :NG] = True                        # west: i = isd..0, all rows
    want_set[njd - NG:, NG:] = True                # north: j = npy..jed, i = 1..ied
    assert np.array_equal(got[want_set], _blend(f0, f1, 1, 3)[0, 0][want_set])
    assert np.all(got[~want_set] == 7.0)


@pytest.mark.parametrize("hord,nord_tr,trdm", [(8, 0, 0.0), (5, 1, 0.1), (1, 0, 0.0)])
def test_nested_equals_tracer_2d_with_a_boundary_callback(prob, hord, nord_tr, trdm):
    """The boundary states applied inside the call equal the same states applied by a halo callback that counts
    substeps itself: bit for bit, with the count advanced by nsplt."""
    P = prob
    args = _args(P)
    f0 = args[0].copy()
    f1 = _later(f0)
    bc = S.nest_strips(f0, f1, 1 - NG, 1 - NG, P.n + 1, P.n + 1)
    k_split, c0, q_split = 2, 1, 3
    kw = dict(hord=hord, q_split=q_split, nord_tr=nord_tr, trdm=trdm, lim_fac=2.0 if hord == 1 else 1.0)
    ref = O.tracer_2d_nested(*args, P.geoms[0], bc, nest_timestep=c0, k_split=k_split, **kw)
    ring = _ring(*f0.shape[-2:], P.n, P.n)
    count = {"c": c0}

    def fill(p, nq, npz, ctx):
        qa = np.ctypeslib.as_array(p, shape=f0.shape)
        qa[..., ring] = _blend(f0, f1, count["c"], q_split * k_split)[..., ring]
        count["c"] += 1

    got = O.tracer_2d_nested(*args, P.geoms[0], None, nest_timestep=c0, k_split=k_split, halo_fn=fill, **kw)
    assert ref[6] == got[6] == q_split
    assert ref[7] == got[7] == c0 + q_split == count["c"]
    for a, b in zip(ref[:6], got[:6]):
        assert np.array_equal(a, b)
    assert not np.array_equal(interior(ref[0], P.n), interior(args[0], P.n))


def test_nested_boundary_time_matters(prob):
    """The same call later in the parent interval sees other boundary values (and, with t1 = t0, does not)."""
    P = prob
    args = _args(P)
    f0 = args[0].copy()
    moving = S.nest_strips(f0, _later(f0), 1 - NG, 1 - NG, P.n + 1, P.n + 1)
    still = S.nest_strips(f0, f0, 1 - NG, 1 - NG, P.n + 1, P.n + 1)
    a = O.tracer_2d_nested(*args, P.geoms[0], moving, nest_timestep=0, k_split=2, q_split=2)
    b = O.tracer_2d_nested(*args, P.geoms[0], moving, nest_timestep=2, k_split=2, q_split=2)
    assert np.abs(interior(a[0], P.n) - interior(b[0], P.n)).max() > 1e-6
    c = O.tracer_2d_nested(*args, P.geoms[0], still, nest_timestep=0, k_split=2, q_split=2)
    d = O.tracer_2d_nested(*args, P.geoms[0], still, nest_timestep=2, k_split=2, q_split=2)
    assert np.array_equal(c[0], d[0])


@pytest.mark.parametrize("nord_tr,trdm", [(0, 0.0), (2, 0.12)])
def test_nested_keeps_a_constant(prob, nord_tr, trdm):
    P = prob
    args = _args(P)
    args[0] = np.full_like(args[0], 2.5)
    bc = S.nest_strips(args[0], args[0], 1 - NG, 1 - NG, P.n + 1, P.n + 1)
    out = O.tracer_2d_nested(*args, P.geoms[0], bc, nest_timestep=0, k_split=1, q_split=3, nord_tr=nord_tr,
                             trdm=trdm)
    assert np.abs(out[0] - 2.5).max() <= 1e-13


def test_not_nested_is_tracer_2d_and_keeps_the_count(prob):
    """On a grid that is not nested (a parent with nests) the call is tracer_2d and the count stays."""
    P = prob
    args = _args(P)
    ref = O.tracer_2d(*args, P.geoms[0], hord=8, q_split=2)
    got = O.tracer_2d_nested(*args, P.geoms[0], None, nest_timestep=4, k_split=3, q_split=2, nested=0)
    assert got[7] == 4 and got[6] == ref[6] == 2
    for a, b in zip(ref[:6], got[:6]):
        assert np.array_equal(a, b)


def test_nested_rank_takes_outer_sides_from_the_boundary_and_inner_sides_from_the_callback(prob):
    """A rank at the nest's south-west corner: after the call its west and south halo hold the states of the
    last substep's start, its east and north halo what the callback wrote."""
    P = prob
    n, ie, je = P.n, 10, 12
    geom, args = sub_domain(P, 0, 1, ie, 1, je)
    bd = O.Bounds(1, ie, 1, je, 1 - NG, ie + NG, 1 - NG, je + NG, NG)
    f0 = args[0].copy()
    f1 = _later(f0)
    bc = S.nest_strips(f0, f1, bd.isd, bd.jsd, n + 1, n + 1)
    halo = f0 * 0.5

    def neighbours(p, nq, npz, ctx):  # the east and north neighbours' cells, fixed
        qa = np.ctypeslib.as_array(p, shape=f0.shape)
        qa[..., :, ie + NG:] = halo[..., :, ie + NG:]
        qa[..., je + NG:, :] = halo[..., je + NG:, :]

    da = float(np.min(P.geoms[0].area[NG:NG + n, NG:NG + n]))
    out = O.tracer_2d_nested(*args, geom, bc, nest_timestep=0, k_split=1, q_split=3, halo_fn=neighbours,
                             bounds=bd, npx=n + 1, npy=n + 1, da_min=da)
    q = out[0]
    last = _blend(f0, f1, 2, 3)
    assert np.array_equal(q[..., :, :NG], last[..., :, :NG])                    # west, full height
    assert np.array_equal(q[..., :NG, NG:], last[..., :NG, NG:])                # south, i = 1..ied
    assert np.array_equal(q[..., NG:, ie + NG:], halo[..., NG:, ie + NG:])      # east above the south rows
    assert np.array_equal(q[..., je + NG:, NG:ie + NG], halo[..., je + NG:, NG:ie + NG])  # north
    assert out[7] == 3
