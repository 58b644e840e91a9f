"""Regenerate the golden fixtures of the tracer path.

The reference tree holds no golden vectors for tracer_2d / fv_tp_2d /
map_scalar (the dycore is an empty submodule and its only test parses a
namelist), so these fixtures are produced by the FP64 CPU oracle (oracle/) on
small seeded problems.  Every input the oracle consumes is stored with the
outputs, so the fixtures do not depend on random-number streams or on the
platform's math library.  Run from the repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from fv3atm_gb300 import synth as S  # noqa: E402

GEOM_FIELDS = ("dx", "dy", "dxa", "dya", "area", "rarea", "sin_sg", "del6_u", "del6_v")


# tracer_2d_cube cases of the cube fixture: name -> oracle keyword arguments
CUBE_CASES = {
    "h8": dict(hord=8, q_split=3),
    "h5": dict(hord=5, q_split=2),
    "h1_lim3": dict(hord=1, q_split=2, lim_fac=3.0),
    "h8_nord0": dict(hord=8, q_split=3, nord_tr=0, trdm=0.12),
    "h8_nord1": dict(hord=8, q_split=2, nord_tr=1, trdm=0.1),
    "h5_nord2": dict(hord=5, q_split=2, nord_tr=2, trdm=0.1),
}


def cube_fixture():
    P = S.make_problem(12, 2, 2, seed=101, cmax=0.8)
    d = {k: getattr(P, k).numpy() for k in ("q", "dp", "cx", "cy", "mfx", "mfy")}
    for f in GEOM_FIELDS:
        d["geom_" + f] = np.stack([getattr(g, f) for g in P.geoms])
    d["ak"], d["bk"], d["topo"] = P.ak, P.bk, P.topo
    out = {}
    for name, kw in CUBE_CASES.items():
        q1, dp_last, ns = O.tracer_2d_cube(d["q"], d["dp"], d["mfx"], d["mfy"], d["cx"], d["cy"], P.geoms, P.topo,
                                           **kw)
        out[f"q_{name}"] = q1[..., 3:15, 3:15]
        out[f"dplast_{name}"] = dp_last[..., 3:15, 3:15]
    return {**d, **out, "n": np.array(12)}


# tracer_2d_nested cases of the nested fixture: name -> oracle keyword arguments
NESTED_CASES = {
    "h8": dict(hord=8, q_split=2),
    "h5_nord1": dict(hord=5, q_split=2, nord_tr=1, trdm=0.1),
}


def nested_fixture():
    """One C12-sized nested domain (no cube edges or corners), 2 levels, 2 tracers: boundary states at t0 (the
    initial halo) and t1, k_split 2, the substep count entering at 1."""
    P = S.make_problem(12, 2, 2, seed=303, cmax=0.8, ntiles=1)
    d = {k: getattr(P, k)[0].numpy() for k in ("q", "dp", "cx", "cy", "mfx", "mfy")}
    g = P.geoms[0]
    for f in GEOM_FIELDS:
        d["geom_" + f] = getattr(g, f)
    strips = S.nest_strips(d["q"], d["q"] * 1.25 + 0.05, -2, -2, 13, 13)
    for side, (t0, t1) in strips.items():
        d[f"bc_{side}_t0"], d[f"bc_{side}_t1"] = t0, t1
    out = {}
    for name, kw in NESTED_CASES.items():
        r = O.tracer_2d_nested(d["q"], d["dp"], d["mfx"], d["mfy"], d["cx"], d["cy"], g, strips, nest_timestep=1,
                               k_split=2, **kw)
        out[f"q_{name}"], out[f"dp_{name}"], out[f"count_{name}"] = r[0], r[1][..., 3:15, 3:15], np.array(r[7])
    return {**d, **out, "n": np.array(12)}


def remap_fixture():
    from fv3atm_gb300 import grid as G
    rng = np.random.default_rng(202)
    km, ncol = 63, 8
    ak, bk = G.hybrid_levels(km)
    ps = rng.uniform(95000, 103000, ncol)
    dref = np.diff(ak)[:, None] + np.diff(bk)[:, None] * ps[None]
    dp = dref * (1 + 0.1 * rng.uniform(-1, 1, dref.shape))
    pe1 = np.concatenate([np.full((1, ncol), ak[0]), ak[0] + np.cumsum(dp, 0)])
    pe2 = ak[:, None] + bk[:, None] * pe1[-1][None]
    q1 = np.abs(rng.standard_normal((km, ncol))).cumsum(0) * 0.01 + rng.uniform(0, 0.1, (km, ncol))
    qs = rng.uniform(0, 1, ncol)
    d = {"pe1": pe1, "pe2": pe2, "q1": q1, "qs": qs}
    for kord, iv, qmin in ((9, 0, 0.0), (9, 1, 0.05), (4, 0, 0.0), (4, -1, 0.0), (4, -2, 0.0), (4, 1, 0.05)):
        d[f"q2_k{kord}_iv{iv}"] = O.remap_columns(pe1, q1, pe2, iv=iv, kord=kord, qs=qs, q_min=qmin)
    return d


def c48_bell_norms():
    """Relative L1 / L2 / Linf errors of the single-tile C48 L63 cosine bell after
    10 steps (tests/_c48.py), as the oracle computes them."""
    import json
    from tests import _c48
    P, exact_halo = _c48.problem()
    q, t = _c48.oracle_run(P, exact_halo)
    return json.dumps({"config": "C48 L63 1 tracer, n_split 1, hord 8, kord 9", "steps": _c48.NSTEPS, "t": t,
                       "norms_l1_l2_linf": list(_c48.norms(P, q, t))}, indent=1)


def op_counts():
    """Operation counts of the oracle's hord-8 fv_tp_2d on a C48 tile level and of its kord-9 remap of one
    127-level column (the counting scalar), normalised per tracer-cell-level; bench.py reads the per-update
    figures for its flop ceiling."""
    import json
    from fv3atm_gb300 import grid as G
    from tests._helpers import area_fluxes, ra_xy
    P = S.make_problem(48, 1, 1, seed=5, cmax=0.8)
    t = 1
    g = P.geoms[t]
    cx, cy = P.cx[t, 0].numpy(), P.cy[t, 0].numpy()
    xfx, yfx = area_fluxes(cx, cy, g)
    rax, ray = ra_xy(xfx, yfx, g)
    q = np.ascontiguousarray(P.q[t, 0, 0].numpy())
    adv = O.count_fv_tp_2d(q, cx, cy, 8, xfx, yfx, g, rax, ray, P.mfx[t, 0].numpy(), P.mfy[t, 0].numpy())
    km = 127
    ak, bk = G.hybrid_levels(km)
    rng = np.random.default_rng(1)
    dp = (np.diff(ak) + np.diff(bk) * 1e5) * (1 + 0.1 * rng.uniform(-1, 1, km))
    pe1 = np.concatenate([[ak[0]], ak[0] + np.cumsum(dp)])
    pe2 = ak + bk * pe1[-1]
    q1 = np.abs(rng.standard_normal(km)).cumsum() * 0.01
    rem = O.count_remap_column(pe1, q1, pe2)
    cells = 48 * 48
    update = {"add": 4, "mul": 2, "div": 1, "cmp": 0}  # q <- (q dp1 + div F rarea) / dp2 per cell
    per_cell = {k: (adv[k] + update[k] * cells) / cells for k in adv}
    per_level = {k: rem[k] / km for k in rem}
    flops = lambda d: d["add"] + d["mul"] + d["div"]
    ops = lambda d: flops(d) + d["cmp"]
    return json.dumps({
        "what": "oracle op counts (add/sub, mul, div on tracer values; cmp = min/max/sign): fv_tp_2d hord 8 + the "
                "flux-form update on one C48 tile level, and the kord-9 remap of one 127-level column",
        "fv_tp_2d_c48": adv, "remap_column_l127": rem,
        "per_tracer_cell_level_substep": per_cell, "per_tracer_column_level_remap": per_level,
        "flops_per_substep_cell": flops(per_cell), "ops_per_substep_cell": ops(per_cell),
        "flops_per_remap_level": flops(per_level), "ops_per_remap_level": ops(per_level)}, indent=1)


if __name__ == "__main__":
    np.savez_compressed(os.path.join(HERE, "cube_c12_l2.npz"), **cube_fixture())
    np.savez_compressed(os.path.join(HERE, "remap_columns_l63.npz"), **remap_fixture())
    np.savez_compressed(os.path.join(HERE, "nested_c12_l2.npz"), **nested_fixture())
    with open(os.path.join(HERE, "c48_bell_norms.json"), "w") as f:
        f.write(c48_bell_norms() + "\n")
    with open(os.path.join(HERE, "op_counts.json"), "w") as f:
        f.write(op_counts() + "\n")
    print("written")
