"""GPU parity of the CUDA path (through the C ABI) against the FP64 CPU oracle.

Tolerances: FP64 path relative L2 <= 1e-12 per field (bit-for-bit agreement is
not expected: the kernels multiply by reciprocals and contract FMAs where the
oracle divides); FP32-mixed path relative L2 <= 1e-5 against the FP64 oracle.
"""
import numpy as np
import pytest

import oracle as O
from fv3atm_gb300 import api
from fv3atm_gb300 import synth as S
from fv3atm_gb300._lib import Fv3gError

from ._helpers import (area_fluxes, cube_mass, final_dp, interior, ra_xy, rel_l2, remap_reference)

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-5


@pytest.fixture(scope="module")
def cube_prob():
    # n = 60: two full 26-cell CTA tiles plus a partial one per direction
    return S.make_problem(60, 5, 3, seed=11, cmax=0.8)


@pytest.fixture(scope="module")
def cube_oracle(cube_prob):
    P = cube_prob
    q1, dp_last, ns = O.tracer_2d_cube(P.q, P.dp, P.mfx, P.mfy, P.cx, P.cy, P.geoms, P.topo, hord=8, q_split=3)
    dpf = final_dp(dp_last, P.mfx.numpy(), P.mfy.numpy(), P.geoms, ns, P.n)
    return q1, dpf


def _run_cube(P, precision, hord=8, q_split=3, kord=9, remap=False, graph=False, warps=0):
    st = api.CubeState(P.n, P.npz, P.nq, precision=precision, hord=hord, kord=kord, warps_per_cta=warps)
    st.load_problem(P)
    if graph:
        st.step(q_split, use_graph=True)
    else:
        st.tracer_2d(q_split)
        if remap:
            st.remap()
    return st


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
def test_cube_tracer_2d_matches_oracle(cuda, cube_prob, cube_oracle, precision, tol):
    P = cube_prob
    q_ref, dp_ref = cube_oracle
    st = _run_cube(P, precision)
    q = st.download("Q")
    dp = st.download("DELP_OUT")
    n = P.n
    for iq in range(P.nq):
        e = rel_l2(interior(q[:, iq], n), interior(q_ref[:, iq], n))
        assert e <= tol, (precision, iq, e)
    assert rel_l2(interior(dp, n), interior(dp_ref, n)) <= tol


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
@pytest.mark.parametrize("hord,nord,trdm", [(8, 0, 0.0), (8, 1, 0.1)])
def test_cube_edge_sync_option_matches_oracle(cuda, cube_prob, precision, tol, hord, nord, trdm):
    """edge_sync = 1 (each shared tile-edge face carries the upwind tile's flux; k_edge_fix) against the oracle
    run the same way; the FP64 global mass is conserved with and without it."""
    P = cube_prob
    q_ref, dp_last, ns = O.tracer_2d_cube(P.q, P.dp, P.mfx, P.mfy, P.cx, P.cy, P.geoms, P.topo, hord=hord,
                                          q_split=3, sync_edges=True, nord_tr=nord, trdm=trdm)
    st = api.CubeState(P.n, P.npz, P.nq, precision=precision, hord=hord, nord_tr=nord, trdm=trdm, edge_sync=True)
    st.load_problem(P)
    st.tracer_2d(3)
    q = st.download("Q")
    for iq in range(P.nq):
        assert rel_l2(interior(q[:, iq], P.n), interior(q_ref[:, iq], P.n)) <= tol
    if precision == "fp64":
        dpf = final_dp(dp_last, P.mfx.numpy(), P.mfy.numpy(), P.geoms, ns, P.n)
        m0 = cube_mass(P.q.numpy(), P.dp.numpy(), P.geoms, P.n)
        m1 = cube_mass(q, dpf, P.geoms, P.n)
        assert np.all(np.abs(m1 - m0) <= 1e-13 * np.abs(m0)), (m1 - m0) / m0
    st.close()


@pytest.mark.parametrize("n,nq,warps,edge_sync", [(60, 3, 0, False), (12, 2, 0, False), (28, 4, 1, False),
                                                  (30, 5, 2, True), (53, 2, 12, False), (29, 25, 4, True)])
def test_tracer_pairs_match_oracle_and_single_tracers(cuda, n, nq, warps, edge_sync):
    """FP32 hord 8 with two tracers per warp (packed pair arithmetic): against the FP64 oracle within the mixed
    tolerance and against the one-tracer-per-warp kernel within FP32 rounding -- odd tracer counts (the last
    pair holds one tracer), windows that hold both cube edges (n <= 28) or an edge at window face 30/31, several
    pairs per warp, and the tile-edge reconciliation (edge fluxes written per tracer of a pair)."""
    P = S.make_problem(n, 3, nq, seed=71, cmax=0.8)
    q_ref, _, _ = O.tracer_2d_cube(P.q, P.dp, P.mfx, P.mfy, P.cx, P.cy, P.geoms, P.topo, hord=8, q_split=2,
                                   sync_edges=edge_sync)
    out = {}
    for pairs in (False, True):
        st = api.CubeState(n, 3, nq, precision="mixed", hord=8, warps_per_cta=warps, edge_sync=edge_sync)
        st.load_problem(P)
        st.set_tracer_pairs(pairs)
        assert st.tracer_pairs() == pairs
        st.tracer_2d(2)
        out[pairs] = st.download("Q")
        st.close()
    for iq in range(nq):
        assert rel_l2(interior(out[True][:, iq], n), interior(q_ref[:, iq], n)) <= MIXED_TOL, iq
        assert rel_l2(interior(out[True][:, iq], n), interior(out[False][:, iq], n)) <= 1e-6, iq


def test_tracer_pairs_only_for_fp32_hord8(cuda):
    P = S.make_problem(14, 2, 2, seed=3)
    for prec, hord in (("fp64", 8), ("mixed", 5)):
        st = api.CubeState(14, 2, 2, precision=prec, hord=hord)
        with pytest.raises(Fv3gError, match="tracer pairs"):
            st.set_tracer_pairs(True)
        assert not st.tracer_pairs()
        st.close()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_independent_tiles_match_single_members(cuda, precision):
    """A state of independent tiles (members of one size, each with its own grid, fields and prescribed halo
    ring; one launch per phase for all of them) gives every member bit for bit what the member's own
    single-tile state gives, over two steps; an ensemble of such batches steps alike."""
    probs = [S.make_problem(32, 12, 3, ntiles=1, seed=700 + k, cmax=0.7) for k in range(3)]
    B = S.stack_tiles(probs)
    batch = api.CubeState(32, 12, 3, precision=precision, ntiles=3, independent_tiles=True, warps_per_cta=3)
    batch.load_problem(B)
    singles = []
    for P in probs:
        st = api.CubeState(32, 12, 3, precision=precision, ntiles=1, warps_per_cta=3)
        st.load_problem(P)
        singles.append(st)
    for step in range(2):
        batch.step(2)
        for st in singles:
            st.step(2)
    out = batch.download("Q_REMAPPED")
    for t, st in enumerate(singles):
        assert np.array_equal(out[t], st.download("Q_REMAPPED")[0]), t
    other = api.CubeState(32, 12, 3, precision=precision, ntiles=3, independent_tiles=True, warps_per_cta=3)
    other.load_problem(B)
    ens = api.Ensemble([other])
    ens.step(2)
    ens.step(2)
    import torch
    torch.cuda.synchronize()
    assert np.array_equal(other.download("Q_REMAPPED"), out)
    ens.close()
    for st in singles + [batch, other]:
        st.close()


@pytest.mark.parametrize("precision,bound", [("mixed", 1e-12), ("fp64", 1e-14)])
def test_mass_fix_restores_global_mass_every_step(cuda, precision, bound):
    """mass_fix = 1: after each step every tracer's global mass sum(q delp area) equals its value at the step's
    start to the bound (the FP32 state's mass summed exactly; the FP32 fixer's floor is ~2^-24 of the largest
    values' share of the mass, then 2^-10 of that in its second pass), over several steps; the fixed state stays
    within 1e-8 of the unfixed one, and the host-array step (tracer groups) fixes bit for bit alike."""
    import torch
    P = S.make_problem(192, 64, 4, seed=83, cmax=0.8)
    st = api.CubeState(P.n, P.npz, P.nq, precision=precision, mass_fix=True)
    st.load_problem(P)
    plain = api.CubeState(P.n, P.npz, P.nq, precision=precision)
    plain.load_problem(P)
    for step in range(4):
        m0 = st.mass("Q")
        st.step(3)
        st.sync()
        m1 = st.mass("Q_REMAPPED")
        assert np.all(np.abs(m1 - m0) <= bound * np.abs(m0)), (step, (m1 - m0) / m0)
        if step == 0:
            plain.step(3)
            a, b = st.download("Q_REMAPPED"), plain.download("Q_REMAPPED")
            for iq in range(P.nq):
                assert rel_l2(interior(a[:, iq], P.n), interior(b[:, iq], P.n)) <= 1e-8
            want = a
        # the next step starts from the remapped (and fixed) field
        st.upload("Q", st.download("Q_REMAPPED"))
    dt = torch.float32 if precision == "mixed" else torch.float64
    src = {"Q": P.q, "DELP": P.dp, "CX": P.cx, "CY": P.cy, "MFX": P.mfx, "MFY": P.mfy}
    host = {k: torch.as_tensor(v).to(dt).contiguous().pin_memory() for k, v in src.items()}
    out = torch.zeros(st.field_shape("Q_REMAPPED"), dtype=dt).pin_memory()
    st.step_host(3, host["Q"].data_ptr(), {k: h.data_ptr() for k, h in host.items()}, out.data_ptr(),
                 precision == "mixed", 2)
    assert np.array_equal(out.numpy().astype(np.float64), want)
    st.close()
    plain.close()


@pytest.mark.parametrize("warps", [1, 3])
def test_cube_warps_per_cta_do_not_change_results(cuda, cube_prob, warps):
    P = cube_prob
    a = _run_cube(P, "fp64", warps=warps).download("Q")
    b = _run_cube(P, "fp64", warps=4).download("Q")
    assert np.array_equal(interior(a, P.n), interior(b, P.n))


def test_cube_hord5_matches_oracle(cuda, cube_prob):
    P = cube_prob
    q_ref, _, _ = O.tracer_2d_cube(P.q, P.dp, P.mfx, P.mfy, P.cx, P.cy, P.geoms, P.topo, hord=5, q_split=2)
    q = _run_cube(P, "fp64", hord=5, q_split=2).download("Q")
    assert rel_l2(interior(q, P.n), interior(q_ref, P.n)) <= FP64_TOL


@pytest.mark.parametrize("n", [12, 27, 28, 29, 30, 53])
@pytest.mark.parametrize("hord", [5, 8])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cube_edge_at_the_window_border(cuda, n, hord, precision):
    """Tile sizes whose east/north cube edge falls at window face 30 or 31 of the last full CTA tile (the next
    tile holds one or two cells), or where windows hold both edges of a direction (n <= 28, the edge CTAs'
    16-slot layout; n >= 29 uses 8 slots): the one-sided edge values still reach the faces next to the edge,
    on the FP64 ring kernel and on the register-capped FP32 one."""
    P = S.make_problem(n, 2, 2, seed=17, cmax=0.8)
    q_ref, _, _ = O.tracer_2d_cube(P.q, P.dp, P.mfx, P.mfy, P.cx, P.cy, P.geoms, P.topo, hord=hord, q_split=2)
    st = api.CubeState(n, 2, 2, precision=precision, hord=hord)
    st.load_problem(P)
    st.tracer_2d(2)
    tol = FP64_TOL if precision == "fp64" else (MIXED_TOL if hord == 8 else FILTER_MIXED_TOL)
    assert rel_l2(interior(st.download("Q"), n), interior(q_ref, n)) <= tol
    st.close()


# (hord, nord_tr, trdm, lim_fac): the hord-1 / hord-5 filters, and del-2 / del-4 / del-6 damping of
# the first substep
SCHEMES = [(1, 0, 0.0, 3.0), (5, 0, 0.0, 1.0), (8, 0, 0.12, 1.0), (8, 1, 0.1, 1.0), (8, 2, 0.1, 1.0),
           (5, 2, 0.1, 1.0)]
# The 2-dx filter of hord 1 / 5 is a switch: where bl br (or |lim_fac b0| - |bl - br|) is within FP32
# rounding of zero the mixed path can take the other branch than the FP64 oracle, and each such face
# moves by the parabola's correction, O(the local variation of q).  On these noisy tracers that leaves
# the mixed path within 2e-4 of the oracle; hord 8's limiter is continuous and keeps 1e-5.
FILTER_MIXED_TOL = 2e-4


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
@pytest.mark.parametrize("hord,nord,trdm,lim_fac", SCHEMES)
def test_cube_schemes_and_damping_match_oracle(cuda, cube_prob, precision, tol, hord, nord, trdm, lim_fac):
    P = cube_prob
    if precision == "mixed" and hord != 8:
        tol = FILTER_MIXED_TOL
    q_ref, dp_last, ns = O.tracer_2d_cube(P.q, P.dp, P.mfx, P.mfy, P.cx, P.cy, P.geoms, P.topo, hord=hord,
                                          q_split=3, nord_tr=nord, trdm=trdm, lim_fac=lim_fac)
    st = api.CubeState(P.n, P.npz, P.nq, precision=precision, hord=hord, nord_tr=nord, trdm=trdm, lim_fac=lim_fac)
    st.load_problem(P)
    st.tracer_2d(3)
    q = st.download("Q")
    for iq in range(P.nq):
        e = rel_l2(interior(q[:, iq], P.n), interior(q_ref[:, iq], P.n))
        assert e <= tol, (iq, e)
    if precision == "fp64":  # damping moves tracer mass between cells only
        dpf = final_dp(dp_last, P.mfx.numpy(), P.mfy.numpy(), P.geoms, ns, P.n)
        m0 = cube_mass(P.q.numpy(), P.dp.numpy(), P.geoms, P.n)
        m1 = cube_mass(q, dpf, P.geoms, P.n)
        assert np.all(np.abs(m1 - m0) <= 1e-13 * np.abs(m0)), (m1 - m0) / m0
    st.close()


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
@pytest.mark.parametrize("kord", [9, 4])
def test_cube_remap_matches_oracle(cuda, cube_prob, cube_oracle, precision, tol, kord):
    P = cube_prob
    q_adv, dpf = cube_oracle
    q_ref, dp2_ref, _, _ = remap_reference(q_adv, dpf, P.ak, P.bk, P.n, kord=kord)
    st = _run_cube(P, precision, remap=True, kord=kord)
    q = st.download("Q_REMAPPED")
    for iq in range(P.nq):
        e = rel_l2(interior(q[:, iq], P.n), interior(q_ref[:, iq], P.n))
        assert e <= tol, (precision, iq, e)


def test_graph_step_equals_eager_step(cuda, cube_prob):
    P = cube_prob
    a = _run_cube(P, "mixed", remap=True).download("Q_REMAPPED")
    st = _run_cube(P, "mixed", graph=True)
    b = st.download("Q_REMAPPED")
    assert np.array_equal(interior(a, P.n), interior(b, P.n))
    st.step(3, use_graph=True)  # replay
    assert np.isfinite(st.download("Q")).all()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("mixed", 1e-6)])
def test_cube_conserves_tracer_mass(cuda, cube_prob, precision, tol):
    P = cube_prob
    st = api.CubeState(P.n, P.npz, P.nq, precision=precision)
    st.load_problem(P)
    m0 = st.mass("Q")
    ref0 = cube_mass(P.q.numpy(), P.dp.numpy(), P.geoms, P.n)
    assert np.allclose(m0, ref0, rtol=1e-13 if precision == "fp64" else 1e-6)
    st.tracer_2d(3)
    m1 = st.mass("Q")
    assert np.all(np.abs(m1 - m0) <= tol * np.abs(m0)), (m0, m1)
    st.remap()
    m2 = st.mass("Q_REMAPPED")
    assert np.all(np.abs(m2 - m0) <= 10 * tol * np.abs(m0)), (m0, m2)


def test_cube_monotone_no_new_extrema(cuda, cube_prob):
    P = cube_prob
    st = _run_cube(P, "fp64", remap=True)
    q0 = interior(P.q.numpy(), P.n)
    q = interior(st.download("Q_REMAPPED"), P.n)
    for iq in range(P.nq):
        assert q[:, iq].min() >= q0[:, iq].min() - 1e-14
        assert q[:, iq].max() <= q0[:, iq].max() + 1e-14


# ------------------------------------------------------------ drop-in entries
def _tile_inputs(P, t=0, k=2, iq=1):
    g = P.geoms[t]
    cx, cy = P.cx[t, k].numpy(), P.cy[t, k].numpy()
    xfx, yfx = area_fluxes(cx, cy, g)
    rax, ray = ra_xy(xfx, yfx, g)
    q = np.ascontiguousarray(P.q[t, iq, k].numpy())
    return g, q, cx, cy, xfx, yfx, rax, ray, P.mfx[t, k].numpy(), P.mfy[t, k].numpy()


@pytest.mark.parametrize("hord,lim_fac", [(1, 2.5), (5, 1.0), (8, 1.0)])
@pytest.mark.parametrize("with_mass", [True, False])
def test_fv_tp_2d_dropin_matches_oracle(cuda, cube_prob, hord, lim_fac, with_mass):
    P = cube_prob
    g, q, cx, cy, xfx, yfx, rax, ray, mfx, mfy = _tile_inputs(P)
    mx, my = (mfx, mfy) if with_mass else (None, None)
    fx_r, fy_r, q_r = O.fv_tp_2d(q, cx, cy, hord, xfx, yfx, g, rax, ray, mx, my, lim_fac=lim_fac)
    n = P.n
    fx = np.zeros((n, n + 1))
    fy = np.zeros((n + 1, n))
    qg = q.copy()
    api.fv_tp_2d(qg, cx, cy, n + 1, n + 1, hord, fx, fy, xfx, yfx, api.GridStruct(g), api.bounds_for(n), rax, ray,
                 lim_fac, mx, my)
    assert rel_l2(fx, fx_r) <= FP64_TOL
    assert rel_l2(fy, fy_r) <= FP64_TOL
    assert np.array_equal(qg, q_r)  # corner blocks rewritten exactly as copy_corners does


@pytest.mark.parametrize("nord,damp_c", [(0, 0.12), (1, 0.1), (2, 0.1)])
@pytest.mark.parametrize("with_mass", [True, False])
def test_fv_tp_2d_dropin_damping_matches_oracle(cuda, cube_prob, nord, damp_c, with_mass):
    """deln_flux added to the fluxes: mass-weighted with mass fluxes, unweighted without them."""
    P = cube_prob
    t, k = 4, 2
    g, q, cx, cy, xfx, yfx, rax, ray, mfx, mfy = _tile_inputs(P, t=t, k=k)
    mass = np.ascontiguousarray(P.dp[t, k].numpy())
    mx, my = (mfx, mfy) if with_mass else (None, None)
    fx_r, fy_r, _ = O.fv_tp_2d(q, cx, cy, 8, xfx, yfx, g, rax, ray, mx, my, mass=mass, nord=nord, damp_c=damp_c)
    fx0, fy0, _ = O.fv_tp_2d(q, cx, cy, 8, xfx, yfx, g, rax, ray, mx, my)
    assert rel_l2(fx_r, fx0) > 1e-6  # the damping is visible at this tolerance
    n = P.n
    fx = np.zeros((n, n + 1))
    fy = np.zeros((n + 1, n))
    api.fv_tp_2d(q.copy(), cx, cy, n + 1, n + 1, 8, fx, fy, xfx, yfx, api.GridStruct(g), api.bounds_for(n), rax,
                 ray, 1.0, mx, my, mass, nord, damp_c)
    assert rel_l2(fx, fx_r) <= FP64_TOL
    assert rel_l2(fy, fy_r) <= FP64_TOL


@pytest.mark.parametrize("nord_tr,trdm", [(0, 0.0), (1, 0.1)])
def test_tracer_2d_dropin_matches_oracle_with_halo_callback(cuda, cube_prob, nord_tr, trdm):
    P = cube_prob
    t = 2
    g = P.geoms[t]
    q0 = np.ascontiguousarray(P.q[t].numpy())          # (nq, npz, nd, nd): halos from the neighbours
    halo = q0.copy()

    def refresh(qarr):  # stand-in for mpp_update_domains: restore the halo ring
        n, ng = P.n, 3
        keep = qarr[..., ng:ng + n, ng:ng + n].copy()
        qarr[...] = halo
        qarr[..., ng:ng + n, ng:ng + n] = keep

    args = [np.ascontiguousarray(a[t].numpy()) for a in (P.dp, P.mfx, P.mfy, P.cx, P.cy)]
    ref = O.tracer_2d(q0, *args, g, hord=8, q_split=3, halo_fn=lambda p, nq, npz, ctx: refresh(
        np.ctypeslib.as_array(p, shape=q0.shape)), nord_tr=nord_tr, trdm=trdm)
    qg = q0.copy()
    dp, mfx, mfy, cx, cy = (a.copy() for a in args)
    ns = api.tracer_2d(qg, dp, mfx, mfy, cx, cy, api.GridStruct(g), api.bounds_for(P.n), P.n + 1, P.n + 1, P.npz,
                       P.nq, 8, 3, P.dt, nord_tr=nord_tr, trdm=trdm, halo_update=refresh)
    assert ns == ref[6] == 3
    assert rel_l2(interior(qg, P.n), interior(ref[0], P.n)) <= FP64_TOL
    assert rel_l2(interior(dp, P.n), interior(ref[1], P.n)) <= FP64_TOL
    for got, want in zip((mfx, mfy, cx, cy), ref[2:6]):
        assert rel_l2(got, want) <= 1e-15


@pytest.mark.parametrize("trdm", [0.0, 0.1])
def test_tracer_2d_1L_dropin_matches_oracle(cuda, trdm):
    """Per-level substep counts (winds scaled by level so the counts differ), a halo callback that restores
    the prescribed ring, and optional damping: the drop-in equals the oracle's tracer_2d_1L."""
    P = S.make_problem(30, 4, 2, seed=13, cmax=0.9, ntiles=1)
    g = P.geoms[0]
    f = np.array([0.5, 1.5, 2.5, 1.0])
    args = [np.ascontiguousarray(a[0].numpy()) for a in (P.q, P.dp, P.mfx, P.mfy, P.cx, P.cy)]
    for idx in (2, 3, 4, 5):
        args[idx] = np.ascontiguousarray(args[idx] * f[:, None, None])
    halo = args[0].copy()

    def refresh(qarr):
        n, ng = P.n, 3
        keep = qarr[..., ng:ng + n, ng:ng + n].copy()
        qarr[...] = halo
        qarr[..., ng:ng + n, ng:ng + n] = keep

    ref = O.tracer_2d_1L(*args, g, hord=8, nord_tr=0, trdm=trdm,
                         halo_fn=lambda p, nq, npz, ctx: refresh(np.ctypeslib.as_array(p, shape=halo.shape)))
    assert len(set(ref[6].tolist())) > 1
    q, dp, mfx, mfy, cx, cy = (a.copy() for a in args)
    ns = api.tracer_2d_1L(q, dp, mfx, mfy, cx, cy, api.GridStruct(g), api.bounds_for(P.n), P.n + 1, P.n + 1, P.npz,
                          P.nq, 8, 0, P.dt, nord_tr=0, trdm=trdm, halo_update=refresh)
    assert ns == int(ref[6].max())
    assert rel_l2(interior(q, P.n), interior(ref[0], P.n)) <= FP64_TOL
    assert rel_l2(interior(dp, P.n), interior(ref[1], P.n)) <= FP64_TOL
    for got, want in zip((mfx, mfy, cx, cy), ref[2:6]):
        assert rel_l2(got, want) <= 1e-15


@pytest.mark.parametrize("hord,nord_tr,trdm,q_split", [(8, 0, 0.0, 3), (5, 1, 0.1, 2), (8, 2, 0.12, 0)])
def test_tracer_2d_nested_dropin_matches_oracle(cuda, hord, nord_tr, trdm, q_split):
    """A nested domain (no cube edges or corners): the parent's boundary states, interpolated to each substep's
    start on the device, set the halo ring; q (ring included), dp1 and the advanced count equal the oracle's."""
    P = S.make_problem(40, 4, 3, seed=17, cmax=0.9, ntiles=1)
    g, n, ng = P.geoms[0], P.n, 3
    args = [np.ascontiguousarray(a[0].numpy()) for a in (P.q, P.dp, P.mfx, P.mfy, P.cx, P.cy)]
    f0 = args[0].copy()
    strips = S.nest_strips(f0, f0 * 1.25 + 0.05, 1 - ng, 1 - ng, n + 1, n + 1)
    ref = O.tracer_2d_nested(*args, g, strips, nest_timestep=1, k_split=2, hord=hord, q_split=q_split,
                             nord_tr=nord_tr, trdm=trdm)
    q, dp, mfx, mfy, cx, cy = (a.copy() for a in args)
    ns, count = api.tracer_2d_nested(q, dp, mfx, mfy, cx, cy, api.GridStruct(g, nested=1), api.bounds_for(n), n + 1,
                                     n + 1, P.npz, P.nq, hord, q_split, P.dt, nord_tr=nord_tr, trdm=trdm, k_split=2,
                                     q_bc=api.NestBoundary(strips), nest_timestep=1)
    assert ns == ref[6] and count == ref[7] == 1 + ns
    assert rel_l2(q, ref[0]) <= FP64_TOL
    ring = np.ones(f0.shape[-2:], bool)
    ring[ng:ng + n, ng:ng + n] = False
    assert np.array_equal(q[..., ring], ref[0][..., ring])  # the boundary fill rounds as the oracle does
    assert rel_l2(interior(dp, n), interior(ref[1], n)) <= FP64_TOL
    for got, want in zip((mfx, mfy, cx, cy), ref[2:6]):
        assert rel_l2(got, want) <= 1e-15


def test_tracer_2d_nested_rank_with_neighbours_matches_oracle(cuda):
    """One rank of a decomposed nest (its south-west part): the west and south halo come from the boundary
    states, the east and north halo from the caller's halo update; damping on."""
    P = S.make_problem(40, 3, 2, seed=19, cmax=0.9, ntiles=1)
    n, ng, ie, je = P.n, 3, 24, 30
    from ._helpers import sub_domain
    geom, args = sub_domain(P, 0, 1, ie, 1, je)
    bd = api.Bounds(1, ie, 1, je, 1 - ng, ie + ng, 1 - ng, je + ng, ng)
    obd = O.Bounds(1, ie, 1, je, 1 - ng, ie + ng, 1 - ng, je + ng, ng)
    f0 = args[0].copy()
    strips = S.nest_strips(f0, f0 * 0.8 + 0.1, bd.isd, bd.jsd, n + 1, n + 1)
    halo = f0.copy()

    def neighbours(qa):
        qa[..., :, ie + ng:] = halo[..., :, ie + ng:]
        qa[..., je + ng:, :] = halo[..., je + ng:, :]

    da = float(np.min(P.geoms[0].area[ng:ng + n, ng:ng + n]))
    ref = O.tracer_2d_nested(*args, geom, strips, nest_timestep=0, k_split=1, q_split=3, nord_tr=1, trdm=0.1,
                             halo_fn=lambda p, nq, npz, ctx: neighbours(np.ctypeslib.as_array(p, shape=f0.shape)),
                             bounds=obd, npx=n + 1, npy=n + 1, da_min=da)
    q, dp, mfx, mfy, cx, cy = (a.copy() for a in args)
    ns, count = api.tracer_2d_nested(q, dp, mfx, mfy, cx, cy, api.GridStruct(geom, nested=1, da_min=da), bd, n + 1,
                                     n + 1, P.npz, P.nq, 8, 3, P.dt, nord_tr=1, trdm=0.1, k_split=1,
                                     q_bc=api.NestBoundary(strips), nest_timestep=0, halo_update=neighbours)
    assert (ns, count) == (ref[6], ref[7]) == (3, 3)
    assert rel_l2(q, ref[0]) <= FP64_TOL
    assert rel_l2(dp[..., ng:ng + je, ng:ng + ie], ref[1][..., ng:ng + je, ng:ng + ie]) <= FP64_TOL


def test_tracer_2d_nested_needs_boundary_states(cuda):
    from fv3atm_gb300._lib import Fv3gError
    P = S.make_problem(20, 2, 1, seed=3, cmax=0.5, ntiles=1)
    args = [np.ascontiguousarray(a[0].numpy()) for a in (P.q, P.dp, P.mfx, P.mfy, P.cx, P.cy)]
    with pytest.raises(Fv3gError, match="q_bc"):
        api.tracer_2d_nested(*args, api.GridStruct(P.geoms[0], nested=1), api.bounds_for(P.n), P.n + 1, P.n + 1,
                             P.npz, P.nq, 8, 1, P.dt)
    # not nested: tracer_2d itself, the count left as it is
    ref = O.tracer_2d(*args, P.geoms[0], hord=8, q_split=1)
    ns, count = api.tracer_2d_nested(*args, api.GridStruct(P.geoms[0]), api.bounds_for(P.n), P.n + 1, P.n + 1,
                                     P.npz, P.nq, 8, 1, P.dt, nest_timestep=5)
    assert (ns, count) == (1, 5)
    assert rel_l2(interior(args[0], P.n), interior(ref[0], P.n)) <= FP64_TOL


def test_tracer_2d_dropin_derives_nsplt(cuda, cube_prob):
    P = cube_prob
    t = 0
    g = P.geoms[t]
    args = [np.ascontiguousarray(a[t].numpy()) for a in (P.q, P.dp, P.mfx, P.mfy, P.cx, P.cy)]
    ref = O.tracer_2d(*args, g, hord=8, q_split=0)
    q, dp, mfx, mfy, cx, cy = (a.copy() for a in args)
    ns = api.tracer_2d(q, dp, mfx, mfy, cx, cy, api.GridStruct(g), api.bounds_for(P.n), P.n + 1, P.n + 1, P.npz,
                       P.nq, 8, 0, P.dt)
    assert ns == ref[6] == 1
    assert rel_l2(interior(q, P.n), interior(ref[0], P.n)) <= FP64_TOL


@pytest.mark.parametrize("kind", ["noise", "smooth"])
@pytest.mark.parametrize("kord,iv", [(9, 0), (9, 1), (9, -1), (9, -2), (4, 0), (4, 1), (4, -1), (4, -2)])
def test_map_scalar_dropin_matches_oracle(cuda, kord, iv, kind):
    """Columns of noise (many two-grid-length waves and single extrema) and smooth columns with resolved
    extrema (kord 9's Huynh bounds act there) through every iv case."""
    rng = np.random.default_rng(5)
    from fv3atm_gb300 import grid as G
    km, ni, nj = 63, 20, 7
    ak, bk = G.hybrid_levels(km)
    ps = rng.uniform(95000, 103000, (nj, ni))
    dref = np.diff(ak)[:, None, None] + np.diff(bk)[:, None, None] * ps[None]
    dp = dref * (1 + 0.1 * rng.uniform(-1, 1, dref.shape))
    dp *= dref.sum(0) / dp.sum(0)
    if kind == "noise":
        q1 = np.ascontiguousarray(np.abs(rng.standard_normal((km, nj, ni))) + 0.1)
    else:
        z = np.linspace(0.0, 1.0, km)[:, None, None]
        q1 = np.ascontiguousarray(1.2 + np.sin(2 * np.pi * (2 + rng.uniform(0, 2, (1, nj, ni))) * z +
                                               rng.uniform(0, 6, (1, nj, ni))))
    pe1 = np.concatenate([np.full((1, nj, ni), ak[0]), ak[0] + np.cumsum(dp, 0)])
    pe2 = ak[:, None, None] + bk[:, None, None] * pe1[-1][None]
    qs = rng.uniform(0, 1, (nj, ni))
    j = 4
    p1 = np.ascontiguousarray(pe1[:, j, 2:18])  # (km+1, i1:i2)
    p2 = np.ascontiguousarray(pe2[:, j, 2:18])
    qsr = np.ascontiguousarray(qs[j, 2:18])
    # Fortran bounds: ibeg=1..ni, jbeg=1..nj, i1=3..i2=18, row j+1
    ref = O.map_scalar(km, p1, q1, qsr, km, p2, np.zeros_like(q1), 3, 18, j + 1, 1, ni, 1, nj, iv, kord, 0.05)
    got = np.zeros_like(q1)
    api.map_scalar(km, p1, q1, qsr, km, p2, got, 3, 18, j + 1, 1, ni, 1, nj, iv, kord, 0.05)
    assert rel_l2(got[:, j, 2:18], ref[:, j, 2:18]) <= FP64_TOL
    assert np.count_nonzero(got[:, j, :2]) == 0 and np.count_nonzero(got[:, :j]) == 0


def test_map_scalar_rows_from_concurrent_threads(cuda):
    """Lagrangian_to_Eulerian calls map_scalar row by row from OpenMP threads: rows remapped from 8 host
    threads at once (each thread has its own stream and device arena) equal the rows remapped one by one."""
    from concurrent.futures import ThreadPoolExecutor
    from fv3atm_gb300 import grid as G
    rng = np.random.default_rng(9)
    km, ni, nj = 127, 48, 16
    ak, bk = G.hybrid_levels(km)
    ps = rng.uniform(95000, 103000, (nj, ni))
    dref = np.diff(ak)[:, None, None] + np.diff(bk)[:, None, None] * ps[None]
    dp = dref * (1 + 0.1 * rng.uniform(-1, 1, dref.shape))
    q1 = np.ascontiguousarray(np.abs(rng.standard_normal((km, nj, ni))) + 0.1)
    pe1 = np.concatenate([np.full((1, nj, ni), ak[0]), ak[0] + np.cumsum(dp, 0)])
    pe2 = ak[:, None, None] + bk[:, None, None] * pe1[-1][None]
    qs = np.zeros(ni)

    def row(j, out):
        p1 = np.ascontiguousarray(pe1[:, j, :])
        p2 = np.ascontiguousarray(pe2[:, j, :])
        api.map_scalar(km, p1, q1, qs, km, p2, out, 1, ni, j + 1, 1, ni, 1, nj, 0, 9, 0.0)

    serial = np.zeros_like(q1)
    for j in range(nj):
        row(j, serial)
    outs = [np.zeros_like(q1) for _ in range(nj)]
    with ThreadPoolExecutor(max_workers=8) as ex:
        list(ex.map(lambda j: row(j, outs[j]), range(nj)))
    for j in range(nj):
        assert np.array_equal(outs[j][:, j, :], serial[:, j, :])


def test_map_scalar_3d_matches_rows(cuda):
    rng = np.random.default_rng(9)
    from fv3atm_gb300 import grid as G
    km, ni, nj, nq = 32, 12, 5, 2
    ak, bk = G.hybrid_levels(km)
    ps = rng.uniform(95000, 103000, (nj, ni))
    dref = np.diff(ak)[:, None, None] + np.diff(bk)[:, None, None] * ps[None]
    dp = dref * (1 + 0.1 * rng.uniform(-1, 1, dref.shape))
    pe1 = np.ascontiguousarray(np.concatenate([np.full((1, nj, ni), ak[0]), ak[0] + np.cumsum(dp, 0)]))
    pe2 = np.ascontiguousarray(ak[:, None, None] + bk[:, None, None] * pe1[-1][None])
    q1 = np.ascontiguousarray(rng.uniform(0, 1, (nq, km, nj, ni)))
    got = np.zeros_like(q1)
    api.map_scalar_3d(km, pe1, q1, None, km, pe2, got, 1, ni, 1, nj, 1, ni, 1, nj, nq, 0, 9, 0.0)
    for iq in range(nq):
        r = O.remap_columns(pe1.reshape(km + 1, -1), q1[iq].reshape(km, -1), pe2.reshape(km + 1, -1), iv=0, kord=9)
        assert rel_l2(got[iq].reshape(km, -1), r) <= FP64_TOL


def test_errors_are_reported_not_fatal(cuda, cube_prob):
    P = cube_prob
    g, q, cx, cy, xfx, yfx, rax, ray, mfx, mfy = _tile_inputs(P)
    n = P.n
    fx = np.zeros((n, n + 1))
    fy = np.zeros((n + 1, n))
    from fv3atm_gb300._lib import Fv3gError
    with pytest.raises(Fv3gError, match="hord 6"):
        api.fv_tp_2d(q, cx, cy, n + 1, n + 1, 6, fx, fy, xfx, yfx, api.GridStruct(g), api.bounds_for(n), rax, ray)
    with pytest.raises(Fv3gError, match="nord"):  # del-8 needs more than the 3-cell halo
        api.fv_tp_2d(q, cx, cy, n + 1, n + 1, 8, fx, fy, xfx, yfx, api.GridStruct(g), api.bounds_for(n), rax, ray,
                     1.0, None, None, None, 3, 0.1)
    with pytest.raises(Fv3gError, match="lim_fac"):
        api.fv_tp_2d(q, cx, cy, n + 1, n + 1, 1, fx, fy, xfx, yfx, api.GridStruct(g), api.bounds_for(n), rax, ray,
                     0.0)
    with pytest.raises(Fv3gError, match="damping"):
        st = api.CubeState(P.n, P.npz, P.nq, trdm=0.1)
        st.upload("Q", P.q.numpy())  # no grid: the damping metrics are missing
        st.tracer_2d(1)
    with pytest.raises(Fv3gError, match="kord 7"):
        api.CubeState(P.n, P.npz, P.nq, kord=7)


@pytest.mark.parametrize("fault,code", [("none", 0), ("nan_cx", -4), ("courant", -3), ("inf_mfx", -4),
                                        ("mass", -5)])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_state_error_word_reports_bad_inputs(cuda, fault, code, precision):
    """The batched step's sticky error word: a non-finite Courant number or mass flux on a compute face, a
    Courant number above q_split, or a mass flux that empties a cell; read once, then cleared."""
    P = S.make_problem(30, 3, 2, seed=23, cmax=0.5)
    cx, mfx = P.cx.numpy().copy(), P.mfx.numpy().copy()
    # tile 2, level 1, the x face between cells i = 5 and 6 of row j = 8
    if fault == "nan_cx":
        cx[2, 1, 10, 5] = np.nan
    elif fault == "courant":
        cx[2, 1, 10, 5] = 2.5  # 1.25 per substep at q_split 2
    elif fault == "inf_mfx":
        mfx[2, 1, 7, 5] = np.inf
    elif fault == "mass":
        mfx[2, 1, 7, 5] = 1e18  # drains cell (5, 8) far beyond its mass (~1e4 Pa x 1e11 m2)
    st = api.CubeState(P.n, P.npz, P.nq, precision=precision)
    st.load_problem(P)
    st.upload("CX", cx)
    st.upload("MFX", mfx)
    st.tracer_2d(2)
    assert st.error_code() == code
    assert st.error_code() == 0  # cleared by the read
    st.close()


def test_step_with_fill_matches_oracle_remap_then_fillz(cuda, cube_prob):
    """desc.fill: the remap of the step is followed by fillz, as Lagrangian_to_Eulerian does with fill on.
    hord 5 (unlimited) leaves undershoots below zero next to the clipped bells, which fillz removes."""
    P = cube_prob
    q1, dp_last, ns = O.tracer_2d_cube(P.q, P.dp, P.mfx, P.mfy, P.cx, P.cy, P.geoms, P.topo, hord=5, q_split=3)
    dpf = final_dp(dp_last, P.mfx.numpy(), P.mfy.numpy(), P.geoms, ns, P.n)
    q2, dp2, _, _ = remap_reference(q1, dpf, P.ak, P.bk, P.n)
    n, s = P.n, slice(3, 3 + P.n)
    assert (q2[..., s, s] < 0).any()  # the case exercises the filler
    # oracle fillz on every interior column: (im, km, nq) with i fastest
    qc = np.ascontiguousarray(q2[..., s, s].transpose(1, 2, 0, 3, 4).reshape(P.nq, P.npz, -1))
    dpc = np.ascontiguousarray(dp2.transpose(1, 0, 2, 3).reshape(P.npz, -1))  # interior columns only
    qf = O.fillz(qc, dpc)
    st = api.CubeState(P.n, P.npz, P.nq, precision="fp64", hord=5, fill=True)
    st.load_problem(P)
    st.step(3)
    got = st.download("Q_REMAPPED")[..., s, s].transpose(1, 2, 0, 3, 4).reshape(P.nq, P.npz, -1)
    assert rel_l2(got, qf) <= FP64_TOL
    st.close()


@pytest.mark.parametrize("precision,groups", [("mixed", 1), ("mixed", 2), ("mixed", 3), ("fp64", 2)])
def test_step_host_pipelined_equals_device_step(cuda, cube_prob, precision, groups):
    """fv3g_step_host (host arrays in and out, tracer groups overlapping their transfers with the compute)
    gives the device-resident step's result bit for bit, also when called again."""
    import torch
    P = cube_prob
    dt = torch.float32 if precision == "mixed" else torch.float64
    st = api.CubeState(P.n, P.npz, P.nq, precision=precision)
    st.load_problem(P)
    st.step(3)
    want = st.download("Q_REMAPPED")
    src = {"Q": P.q, "DELP": P.dp, "CX": P.cx, "CY": P.cy, "MFX": P.mfx, "MFY": P.mfy}
    host = {k: torch.as_tensor(v).to(dt).contiguous().pin_memory() for k, v in src.items()}
    out = torch.zeros(st.field_shape("Q_REMAPPED"), dtype=dt).pin_memory()
    for _ in range(2):
        out.zero_()
        st.step_host(3, host["Q"].data_ptr(), {k: h.data_ptr() for k, h in host.items()}, out.data_ptr(),
                     precision == "mixed", groups)
        assert np.array_equal(out.numpy().astype(np.float64), want)
    st.close()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("groups", [1, 3])
def test_step_host_level_blocks_equal_device_step(cuda, precision, groups):
    """With 16 levels or more the first tracer group streams in level blocks (its per-level inputs and tracers
    upload block by block while the earlier blocks advect): the result is the device step's, bit for bit."""
    import torch
    P = S.make_problem(40, 20, 5, seed=13, cmax=0.8)
    dt = torch.float32 if precision == "mixed" else torch.float64
    st = api.CubeState(P.n, P.npz, P.nq, precision=precision)
    st.load_problem(P)
    st.step(2)
    want = st.download("Q_REMAPPED")
    src = {"Q": P.q, "DELP": P.dp, "CX": P.cx, "CY": P.cy, "MFX": P.mfx, "MFY": P.mfy}
    host = {k: torch.as_tensor(v).to(dt).contiguous().pin_memory() for k, v in src.items()}
    out = torch.zeros(st.field_shape("Q_REMAPPED"), dtype=dt).pin_memory()
    for _ in range(2):
        out.zero_()
        st.step_host(2, host["Q"].data_ptr(), {k: h.data_ptr() for k, h in host.items()}, out.data_ptr(),
                     precision == "mixed", groups)
        assert np.array_equal(out.numpy().astype(np.float64), want)
    st.close()


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
def test_batched_q_split_zero_derives_the_substep_count(cuda, precision, tol):
    """q_split 0 on the batched path (fv_core_nml's default): nsplt = int(1 + max |Courant|) as tracer_2d
    derives it, the same result as passing that count, through tracer_2d, the graph step and the host step."""
    import torch
    P = S.make_problem(24, 3, 2, seed=29, cmax=1.6)
    q_ref, _, ns = O.tracer_2d_cube(P.q, P.dp, P.mfx, P.mfy, P.cx, P.cy, P.geoms, P.topo, hord=8, q_split=0)
    assert ns >= 2
    a = api.CubeState(P.n, P.npz, P.nq, precision=precision)
    b = api.CubeState(P.n, P.npz, P.nq, precision=precision)
    a.load_problem(P)
    b.load_problem(P)
    a.tracer_2d(0)
    b.tracer_2d(ns)
    assert a.nsplt() == ns and b.nsplt() == ns
    assert rel_l2(interior(a.download("Q"), P.n), interior(q_ref, P.n)) <= tol
    assert np.array_equal(a.download("Q"), b.download("Q"))
    for st in (a, b):
        st.load_problem(P)
    a.step(0)
    b.step(ns)
    want = b.download("Q_REMAPPED")
    assert a.nsplt() == ns and np.array_equal(a.download("Q_REMAPPED"), want)
    dt = torch.float32 if precision == "mixed" else torch.float64
    src = {"Q": P.q, "DELP": P.dp, "CX": P.cx, "CY": P.cy, "MFX": P.mfx, "MFY": P.mfy}
    host = {k: torch.as_tensor(v).to(dt).contiguous().pin_memory() for k, v in src.items()}
    out = torch.zeros(a.field_shape("Q_REMAPPED"), dtype=dt).pin_memory()
    a.step_host(0, host["Q"].data_ptr(), {k: h.data_ptr() for k, h in host.items()}, out.data_ptr(),
                precision == "mixed", 2)
    assert a.nsplt() == ns and np.array_equal(out.numpy().astype(np.float64), want)
    from fv3atm_gb300._lib import Fv3gError
    cx = P.cx.numpy().copy()
    cx[1, 0, 9, 4] = np.nan
    a.upload("CX", cx)
    with pytest.raises(Fv3gError, match="non-finite"):
        a.tracer_2d(0)
    a.close()
    b.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_field_copies_roundtrip_many_planes(cuda, precision):
    """6 x 9 x 127 planes through the device, pinned-host and FP64-host copy paths."""
    import torch
    n, npz, nq = 96, 127, 9
    st = api.CubeState(n, npz, nq, precision=precision)
    dt = torch.float64 if precision == "fp64" else torch.float32
    shape = st.field_shape("Q")
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    src = torch.rand(shape, dtype=dt, device="cuda", generator=g)
    cur = torch.cuda.current_stream().cuda_stream
    st.upload_device("Q", src.data_ptr(), stream=cur)
    back = torch.zeros_like(src)
    st.download_device("Q", back.data_ptr(), stream=cur)
    torch.cuda.synchronize()
    assert torch.equal(back, src)
    host = src.cpu().pin_memory()
    st.upload_device("Q", torch.zeros_like(src).data_ptr(), stream=cur)
    torch.cuda.synchronize()
    st.upload_async("Q", host.data_ptr(), precision == "mixed", stream=cur)
    hout = torch.zeros_like(host).pin_memory()
    st.download_async("Q", hout.data_ptr(), precision == "mixed", stream=cur)
    torch.cuda.synchronize()
    assert torch.equal(hout, host)
    h64 = src.double().cpu().numpy()
    st.upload("Q", h64)
    assert np.array_equal(st.download("Q"), h64 if precision == "fp64" else src.cpu().numpy().astype(np.float64))


def test_mixed_matches_fp64_many_tracers(cuda):
    """Every tracer of the multi-tracer CTA loop (nq > warps per CTA) within 1e-5 of FP64."""
    P = S.make_problem(48, 16, 20, seed=21, cmax=0.8)
    a = _run_cube(P, "fp64", remap=True).download("Q_REMAPPED")
    b = _run_cube(P, "mixed", remap=True).download("Q_REMAPPED")
    for iq in range(P.nq):
        assert rel_l2(interior(b[:, iq], P.n), interior(a[:, iq], P.n)) <= MIXED_TOL, iq


def test_device_upload_after_conversion_on_default_stream(cuda):
    """Uploads issued on torch's default (legacy) stream stay ordered after the
    dtype conversion that produced them (127-level fields, FP32 state)."""
    import torch
    P = S.make_problem(96, 127, 4, seed=2000, cmax=0.8, device="cuda")
    out = {}
    for prec, dt in (("fp64", torch.float64), ("mixed", torch.float32)):
        st = api.CubeState(P.n, P.npz, P.nq, precision=prec)
        st.set_grid(P.geoms)
        st.set_levels(P.ak, P.bk)
        for name, val in (("Q", P.q), ("DELP", P.dp), ("CX", P.cx), ("CY", P.cy), ("MFX", P.mfx),
                          ("MFY", P.mfy)):
            v = val.to(dt).contiguous()
            st.upload_device(name, v.data_ptr(), stream=torch.cuda.current_stream().cuda_stream)
            del v
        st.tracer_2d(1)
        q = torch.empty(st.field_shape("Q"), dtype=dt, device="cuda")
        st.download_device("Q", q.data_ptr())
        st.sync()
        out[prec] = q[..., 3:3 + P.n, 3:3 + P.n].double()
    for iq in range(P.nq):
        a, b = out["fp64"][:, iq], out["mixed"][:, iq]
        assert float(torch.linalg.vector_norm(b - a) / torch.linalg.vector_norm(a)) <= MIXED_TOL, iq


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_upload_on_a_delayed_stream_is_ordered_before_the_state_work(cuda, precision):
    """An upload on another stream, held back there by a bounded spin, is still read by the state's next
    step on its own stream: the step runs after the copy.  The transport is homogeneous in q and doubling
    is exact, so uploading 2 q must give exactly twice the step of q (the step of the old q if unordered)."""
    import torch
    P = S.make_problem(30, 5, 2, seed=31, cmax=0.8)
    dt = torch.float64 if precision == "fp64" else torch.float32
    st = api.CubeState(P.n, P.npz, P.nq, precision=precision)
    try:
        st.load_problem(P)
        st.tracer_2d(2)
        ref = st.download("Q")
        st.upload("Q", P.q.numpy())
        q2 = (2 * torch.as_tensor(P.q.numpy())).to(dt).cuda().contiguous()
        side = torch.cuda.Stream()
        torch.cuda.synchronize()
        with torch.cuda.stream(side):
            torch.cuda._sleep(20_000_000)  # a bounded spin of ~10 ms ahead of the copy on that stream
        st.upload_device("Q", q2.data_ptr(), stream=side.cuda_stream)
        st.tracer_2d(2)
        got = st.download("Q")
        torch.cuda.synchronize()
        s = slice(3, 3 + P.n)
        assert np.array_equal(got[..., s, s], 2 * ref[..., s, s])
    finally:
        st.close()


# ------------------------------------------------------- committed fixtures
def test_cube_matches_committed_golden_fixture(cuda):
    from .test_golden import load_cube
    d, geoms = load_cube()
    n = int(d["n"])
    for hord, q_split in ((8, 3), (5, 2)):
        st = api.CubeState(n, d["q"].shape[2], d["q"].shape[1], precision="fp64", hord=hord)
        st.set_grid(geoms)
        st.set_levels(d["ak"], d["bk"])
        for name, key in (("Q", "q"), ("DELP", "dp"), ("CX", "cx"), ("CY", "cy"), ("MFX", "mfx"), ("MFY", "mfy")):
            st.upload(name, d[key])
        st.tracer_2d(q_split)
        q = st.download("Q")[..., 3:3 + n, 3:3 + n]
        assert rel_l2(q, d[f"q_h{hord}"]) <= FP64_TOL, hord


@pytest.mark.parametrize("name", ["h8", "h5_nord1"])
def test_nested_matches_committed_golden_fixture(cuda, name):
    """fv3g_tracer_2d_nested on the committed nested fixture (tests/golden/nested_c12_l2.npz)."""
    from .test_golden import NESTED_CASES, load_nested
    d, geom, strips = load_nested()
    n = int(d["n"])
    kw = NESTED_CASES[name]
    q, dp, mfx, mfy, cx, cy = (np.ascontiguousarray(d[k]).copy() for k in ("q", "dp", "mfx", "mfy", "cx", "cy"))
    da = float(np.min(d["geom_area"][3:3 + n, 3:3 + n]))
    ns, count = api.tracer_2d_nested(q, dp, mfx, mfy, cx, cy, api.GridStruct(geom, nested=1, da_min=da),
                                     api.bounds_for(n), n + 1, n + 1, q.shape[1], q.shape[0], kw["hord"],
                                     kw["q_split"], 0.0, nord_tr=kw.get("nord_tr", 0), trdm=kw.get("trdm", 0.0),
                                     k_split=2, q_bc=api.NestBoundary(strips), nest_timestep=1)
    assert (ns, count) == (2, int(d[f"count_{name}"]))
    assert rel_l2(q, d[f"q_{name}"]) <= FP64_TOL
    assert rel_l2(interior(dp, n), d[f"dp_{name}"]) <= FP64_TOL


def test_remap_matches_committed_golden_fixture(cuda):
    import os
    d = dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "remap_columns_l63.npz")))
    km, ncol = d["q1"].shape
    for kord, iv, qmin in ((9, 0, 0.0), (9, 1, 0.05), (4, 0, 0.0), (4, -1, 0.0), (4, -2, 0.0), (4, 1, 0.05)):
        q1 = np.ascontiguousarray(d["q1"][None, :, None, :])
        out = np.zeros_like(q1)
        api.map_scalar_3d(km, np.ascontiguousarray(d["pe1"]), q1, np.ascontiguousarray(d["qs"]), km,
                          np.ascontiguousarray(d["pe2"]), out, 1, ncol, 1, 1, 1, ncol, 1, 1, 1, iv, kord, qmin)
        assert rel_l2(out[0, :, 0, :], d[f"q2_k{kord}_iv{iv}"]) <= FP64_TOL, (kord, iv)


def test_c48_bell_ten_steps_matches_oracle_and_golden_norms(cuda):
    """C48 L63 cosine bell, n_split 1, hord 8, kord 9, 10 steps through the drop-in
    tracer_2d (halo callback) and map_scalar_3d entries."""
    import json
    import os
    from . import _c48
    P, exact_halo = _c48.problem()
    qg, t = _c48.device_run(P, exact_halo)
    qo, _ = _c48.oracle_run(P, exact_halo)
    assert rel_l2(interior(qg, P.n), interior(qo, P.n)) <= FP64_TOL
    with open(os.path.join(os.path.dirname(__file__), "golden", "c48_bell_norms.json")) as f:
        gold = json.load(f)
    assert np.allclose(_c48.norms(P, qg, t), gold["norms_l1_l2_linf"], rtol=1e-9, atol=0)


def test_autotune_picks_a_width_and_leaves_results_unchanged(cuda, cube_prob):
    P = cube_prob
    st = api.CubeState(P.n, P.npz, P.nq, precision="mixed")
    st.load_problem(P)
    w = st.autotune()
    assert w in (3, 4, 5, 6, 8, 10, 12)
    assert st.widths()[0] == w and st.widths()[1] <= 8  # FP32 edge-ring CTAs are capped at 8 warps
    st.step(3)
    got = st.download("Q_REMAPPED")
    ref = api.CubeState(P.n, P.npz, P.nq, precision="mixed", warps_per_cta=4)
    ref.load_problem(P)
    ref.set_tracer_pairs(st.tracer_pairs())  # the mode the tuner chose, at another width
    ref.step(3)
    want = ref.download("Q_REMAPPED")
    assert np.array_equal(got, want)  # every tracer's arithmetic is independent of the CTA width


# ---------------------------------------------------- Lagrangian_to_Eulerian
def test_fillz_dropin_matches_oracle(cuda):
    rng = np.random.default_rng(9)
    km, im, nq = 32, 50, 3
    dp = rng.uniform(50.0, 900.0, (km, im))
    q = rng.uniform(0.0, 1.0, (nq, km, im))
    q[rng.uniform(size=q.shape) < 0.3] *= -0.4
    want = O.fillz(q, dp)
    got = q.copy()
    api.fillz(im, km, nq, got, dp)
    assert np.allclose(got, want, rtol=1e-13, atol=1e-15)


def test_pressure_vars_dropin_matches_oracle(cuda):
    rng = np.random.default_rng(10)
    km, im = 64, 40
    dp = rng.uniform(50.0, 900.0, (km, im))
    pe, peln, pk = (np.zeros((km + 1, im)) for _ in range(3))
    pkz = np.zeros((km, im))
    api.pressure_vars(im, km, 100.0, 0.2857, dp, pe, peln, pk, pkz)
    # log / exp of the device and host math libraries differ in the last bit; pkz divides a difference of
    # neighbouring pk values by a difference of neighbouring logs, which magnifies that by pk / dpk ~ 1e2
    for got, want, tol in zip((pe, peln, pk, pkz), O.pressure_vars(dp, 100.0, 0.2857), (1e-15, 1e-14, 1e-14, 1e-12)):
        assert np.allclose(got, want, rtol=tol, atol=0)


def test_state_fillz_conserves_column_mass(cuda):
    P = S.make_problem(16, 6, 2, seed=12, cmax=0.7)
    q = P.q.numpy().copy()
    q[:, :, 2] -= 0.3  # a level with negative values everywhere
    st = api.CubeState(P.n, P.npz, P.nq, precision="fp64")
    st.load_problem(P)
    st.upload("Q", q)
    st.step(2)
    before = st.download("Q_REMAPPED")
    st.fillz()
    after = st.download("Q_REMAPPED")
    dpo = st.download("DELP_OUT")
    n = P.n
    ps = P.ak[0] + interior(dpo, n).sum(1)                       # (6, n, n)
    pe2 = P.ak[:, None, None, None] + P.bk[:, None, None, None] * ps[None]
    dpe = np.diff(pe2, axis=0).transpose(1, 0, 2, 3)              # (6, npz, n, n)
    for iq in range(P.nq):
        m0 = (interior(before[:, iq], n) * dpe).sum(1)
        m1 = (interior(after[:, iq], n) * dpe).sum(1)
        assert np.all(np.abs(m1 - m0) <= 1e-12 * np.abs(interior(before[:, iq], n) * dpe).sum(1))
        pos = m0 > 0
        assert np.all(interior(after[:, iq], n).transpose(0, 2, 3, 1)[pos] >= 0.0)


@pytest.mark.parametrize("kord,iv", [(9, 0), (9, -1), (4, 1), (4, -1)])
def test_map1_q2_matches_oracle(cuda, kord, iv):
    """fv3g_map1_q2: row j of q1 onto pe2 with the target thicknesses dp2 given (2-D output row) equals the
    oracle's remap with the same dp2."""
    rng = np.random.default_rng(90 + kord)
    km, kn, ni, nj, j = 48, 40, 9, 3, 2
    pe1 = np.zeros((km + 1, ni))
    pe1[0] = 50.0
    pe1[1:] = 50.0 + np.cumsum(rng.uniform(300.0, 900.0, (km, ni)), axis=0)
    pe2 = np.linspace(0.0, 1.0, kn + 1)[:, None] * (pe1[-1] - pe1[0]) + pe1[0]
    pe2[-1] = pe1[-1]
    dp2 = np.diff(pe2, axis=0) * rng.uniform(0.97, 1.03, (kn, ni))
    q1 = rng.uniform(0.2, 1.4, (km, nj, ni))  # Fortran q1(ibeg:iend, jbeg:jend, km)
    q2 = np.zeros((kn, ni))
    api.map1_q2(km, pe1, q1, kn, pe2, q2, dp2, 1, ni, iv, kord, j, 1, ni, 1, nj, 0.1 if iv == 1 else 0.0)
    want = O.remap_columns(pe1, q1[:, j - 1, :], pe2, iv=iv, kord=kord, q_min=0.1 if iv == 1 else 0.0, dp2=dp2)
    assert rel_l2(q2, want) <= 1e-12


@pytest.mark.parametrize("kind,iv,log_p", [(0, 1, False), (0, 1, True), (1, -1, False), (2, -1, False)])
def test_state_remap_fields_match_oracle(cuda, kind, iv, log_p):
    """fv3g_state_remap_fields after a tracer_2d: cell fields (pt, optionally in ln p) and u / v winds on the
    faces (pressures the mean of the two cells beside a face, across tile edges from the neighbouring tiles)
    equal the oracle's column remap on the same pressures."""
    import torch
    P = S.make_problem(24, 10, 2, seed=47, cmax=0.6)
    st = api.CubeState(24, 10, 2, precision="fp64", kord=9)
    st.load_problem(P)
    st.tracer_2d(2)
    st.sync()
    n, nd, km = 24, 30, 10
    dp = torch.as_tensor(st.download("DELP_OUT"))
    S.fill_cube_halo(dp, n, 3, P.topo)  # the faces' neighbouring columns
    dp = dp.numpy()
    rng = np.random.default_rng(48 + kind)
    f = rng.uniform(250.0, 320.0, (6, 3, km, nd, nd)) if kind == 0 else rng.uniform(-30.0, 30.0, (6, 3, km, nd, nd))
    fin = torch.as_tensor(f, device="cuda")
    fout = torch.zeros_like(fin)
    st.remap_fields(fin.data_ptr(), fout.data_ptr(), 3, kind=kind, iv=iv, kord=9, q_min=1.0, log_p=log_p)
    torch.cuda.synchronize()
    got = fout.cpu().numpy()
    ak, bk = np.asarray(P.ak, np.float64), np.asarray(P.bk, np.float64)
    ni, nj = (n + 1, n) if kind == 2 else (n, n + 1) if kind == 1 else (n, n)
    for t in range(6):
        for (ci, cj) in [(0, 0), (ni - 1, nj - 1), (ni // 2, 3), (1, nj - 2)]:
            i, jj = 1 + ci + 2, 1 + cj + 2  # array indices (halo 3: tile index 1 is array index 3)
            pa = ak[0] + np.concatenate([[0.0], np.cumsum(dp[t, :, jj + 0, i + 0])])
            if kind == 0:
                p = pa
            else:
                ib, jb = (i, jj - 1) if kind == 1 else (i - 1, jj)
                p = 0.5 * (pa + ak[0] + np.concatenate([[0.0], np.cumsum(dp[t, :, jb, ib])]))
            p2 = ak + bk * p[-1]
            if log_p:
                p, p2 = np.log(p), np.log(p2)
            for fi in range(3):
                want = O.remap_columns(p[:, None], f[t, fi, :, jj, i][:, None], p2[:, None], iv=iv, kord=9,
                                       q_min=1.0)[:, 0]
                assert rel_l2(got[t, fi, :, jj, i], want) <= 1e-12, (t, ci, cj, fi)
    st.close()
