"""The oracle reproduces its committed golden fixtures (tests/golden/, made by
tests/golden/make_golden.py).  The reference holds no fixtures for this path,
so these pin the oracle against regressions; the GPU tests check the CUDA path
against the same files."""
import os
import types

import numpy as np
import pytest

import oracle as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GEOM_FIELDS = ("dx", "dy", "dxa", "dya", "area", "rarea", "sin_sg", "del6_u", "del6_v")


def load_cube():
    d = dict(np.load(os.path.join(HERE, "cube_c12_l2.npz")))
    geoms = [types.SimpleNamespace(**{f: d["geom_" + f][t] for f in GEOM_FIELDS}, n=int(d["n"]), ng=3)
             for t in range(6)]
    return d, geoms


# name -> oracle keyword arguments (the cases make_golden.py records)
CUBE_CASES = {
    "h8": dict(hord=8, q_split=3),
    "h5": dict(hord=5, q_split=2),
    "h1_lim3": dict(hord=1, q_split=2, lim_fac=3.0),
    "h8_nord0": dict(hord=8, q_split=3, nord_tr=0, trdm=0.12),
    "h8_nord1": dict(hord=8, q_split=2, nord_tr=1, trdm=0.1),
    "h5_nord2": dict(hord=5, q_split=2, nord_tr=2, trdm=0.1),
}


@pytest.mark.parametrize("name", sorted(CUBE_CASES))
def test_oracle_reproduces_cube_fixture(name):
    d, geoms = load_cube()
    q1, dp_last, _ = O.tracer_2d_cube(d["q"], d["dp"], d["mfx"], d["mfy"], d["cx"], d["cy"], geoms, d["topo"],
                                      **CUBE_CASES[name])
    n = int(d["n"])
    assert np.array_equal(q1[..., 3:3 + n, 3:3 + n], d[f"q_{name}"])
    assert np.array_equal(dp_last[..., 3:3 + n, 3:3 + n], d[f"dplast_{name}"])


NESTED_CASES = {
    "h8": dict(hord=8, q_split=2),
    "h5_nord1": dict(hord=5, q_split=2, nord_tr=1, trdm=0.1),
}


def load_nested():
    d = dict(np.load(os.path.join(HERE, "nested_c12_l2.npz")))
    geom = types.SimpleNamespace(**{f: d["geom_" + f] for f in GEOM_FIELDS}, n=int(d["n"]), ng=3)
    strips = {side: (d[f"bc_{side}_t0"], d[f"bc_{side}_t1"]) for side in ("west", "east", "south", "north")}
    return d, geom, strips


@pytest.mark.parametrize("name", sorted(NESTED_CASES))
def test_oracle_reproduces_nested_fixture(name):
    d, geom, strips = load_nested()
    r = O.tracer_2d_nested(d["q"], d["dp"], d["mfx"], d["mfy"], d["cx"], d["cy"], geom, strips, nest_timestep=1,
                           k_split=2, **NESTED_CASES[name])
    n = int(d["n"])
    assert np.array_equal(r[0], d[f"q_{name}"])
    assert np.array_equal(r[1][..., 3:3 + n, 3:3 + n], d[f"dp_{name}"])
    assert r[7] == int(d[f"count_{name}"]) == 3


@pytest.mark.parametrize("kord,iv,qmin", [(9, 0, 0.0), (9, 1, 0.05), (4, 0, 0.0), (4, -1, 0.0), (4, -2, 0.0),
                                          (4, 1, 0.05)])
def test_oracle_reproduces_remap_fixture(kord, iv, qmin):
    d = dict(np.load(os.path.join(HERE, "remap_columns_l63.npz")))
    q2 = O.remap_columns(d["pe1"], d["q1"], d["pe2"], iv=iv, kord=kord, qs=d["qs"], q_min=qmin)
    assert np.array_equal(q2, d[f"q2_k{kord}_iv{iv}"])


def test_oracle_c48_bell_norms_match_golden():
    """The single-tile C48 L63 cosine bell, 10 steps (tests/_c48.py): the oracle's
    error norms against the analytic rotated bell are the recorded golden numbers."""
    import json
    import os
    from . import _c48
    with open(os.path.join(os.path.dirname(__file__), "golden", "c48_bell_norms.json")) as f:
        gold = json.load(f)
    P, exact_halo = _c48.problem()
    q, t = _c48.oracle_run(P, exact_halo)
    assert abs(t - gold["t"]) <= 1e-9 * gold["t"]
    assert np.allclose(_c48.norms(P, q, t), gold["norms_l1_l2_linf"], rtol=1e-9, atol=0)
