"""The oracle's operation counts (its op-counting scalar run through fv_tp_2d and
the column remap) reproduce the committed tests/golden/op_counts.json that
bench.py's flop ceiling reads, and scale as the schemes say."""
import json
import os

import numpy as np

import oracle as O
from fv3atm_gb300 import synth as S

from ._helpers import area_fluxes, ra_xy

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_op_counts_match_the_committed_file():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    assert json.loads(mg.op_counts()) == json.load(open(os.path.join(HERE, "op_counts.json")))


def test_op_counts_follow_the_schemes():
    """hord 8 spends its extra operations in min/max/sign (the limiter); the count of one fv_tp_2d grows with
    the number of cells; the remap count is linear in the column length."""
    P = S.make_problem(24, 1, 1, seed=5, cmax=0.8)
    t = 2
    g = P.geoms[t]
    cx, cy = P.cx[t, 0].numpy(), P.cy[t, 0].numpy()
    xfx, yfx = area_fluxes(cx, cy, g)
    rax, ray = ra_xy(xfx, yfx, g)
    q = np.ascontiguousarray(P.q[t, 0, 0].numpy())
    mfx, mfy = P.mfx[t, 0].numpy(), P.mfy[t, 0].numpy()
    c8 = O.count_fv_tp_2d(q, cx, cy, 8, xfx, yfx, g, rax, ray, mfx, mfy)
    c5 = O.count_fv_tp_2d(q, cx, cy, 5, xfx, yfx, g, rax, ray, mfx, mfy)
    assert c8["cmp"] > 4 * c5["cmp"] and c8["div"] == c5["div"]
    # per cell, within the prior of 150-200 operations for hord 8 on a tile this size (halo overhead grows
    # as the tile shrinks)
    ops = sum(c8.values()) / 24 ** 2
    assert 150 < ops < 260, ops
    pe = np.linspace(100.0, 1e5, 65)
    pe2 = np.linspace(100.0, 1e5, 65) ** 1.0
    r64 = O.count_remap_column(pe, np.linspace(1, 2, 64), pe2)
    r32 = O.count_remap_column(pe[::2].copy(), np.linspace(1, 2, 32), pe2[::2].copy())
    assert abs(sum(r64.values()) / sum(r32.values()) - 2.0) < 0.1
