"""The single-tile C48 L63 cosine-bell configuration: n_split = 1, hord 8,
kord 9, 10 steps.  Each step refreshes the halo ring from the analytic rotated
bell (on the neighbouring tiles' cell centres), advects with tracer_2d and
remaps onto the hybrid levels of the new surface pressure.  The same driver
runs the oracle and the CUDA path (through the C ABI) on identical inputs."""
import numpy as np

from fv3atm_gb300 import synth as S

from ._helpers import final_dp

NSTEPS = 10


def problem():
    return S.c48_single_tile()


def exact_interior(P, t):
    g = P.geoms[0]
    n, ng = P.n, P.ng
    back = S.rotate(g.centers[ng:ng + n, ng:ng + n], -P.meta["omega"] * t)
    return S.bell(back, P.meta["center"])[None] * P.meta["vert"][:, None, None]


def norms(P, q, t):
    """Relative L1, L2, Linf of the interior tracer against the analytic bell (area weighted)."""
    n, ng = P.n, P.ng
    qe = exact_interior(P, t)
    a = P.geoms[0].area[ng:ng + n, ng:ng + n][None]
    e = q[..., ng:ng + n, ng:ng + n] - qe
    return (float((np.abs(e) * a).sum() / (np.abs(qe) * a).sum()),
            float(np.sqrt((e * e * a).sum() / (qe * qe * a).sum())),
            float(np.abs(e).max() / np.abs(qe).max()))


def run(P, exact_halo, advect, remap, nsteps=NSTEPS):
    """advect(q, dp, mfx, mfy, cx, cy, refresh) -> (q, dp_last, nsplt);
    remap(pe1, q, pe2) -> q (interior columns, kn = km)."""
    n, ng, npz = P.n, P.ng, P.npz
    q = np.ascontiguousarray(P.q[0].numpy())  # (1, npz, nd, nd)
    dp = np.ascontiguousarray(P.dp[0].numpy())
    mfx, mfy, cx, cy = (np.ascontiguousarray(a[0].numpy()) for a in (P.mfx, P.mfy, P.cx, P.cy))
    ring = np.ones((P.nd, P.nd), bool)
    ring[ng:ng + n, ng:ng + n] = False
    for c0 in (slice(0, ng), slice(ng + n, P.nd)):  # cube-corner blocks come from copy_corners
        for c1 in (slice(0, ng), slice(ng + n, P.nd)):
            ring[c0, c1] = False
    t = 0.0
    for _ in range(nsteps):
        halo = exact_halo(t)

        def refresh(qarr, halo=halo):
            qarr[..., ring] = halo[..., ring]

        q, dp_last, ns = advect(q, dp.copy(), mfx, mfy, cx, cy, refresh)
        dpf = final_dp(dp_last[None], mfx[None], mfy[None], P.geoms, ns, n)[0]
        col = dpf[:, ng:ng + n, ng:ng + n].reshape(npz, -1)
        pe1 = np.concatenate([np.full((1, col.shape[1]), P.ak[0]), P.ak[0] + np.cumsum(col, 0)])
        pe2 = P.ak[:, None] + P.bk[:, None] * pe1[-1][None]
        qi = q[0][:, ng:ng + n, ng:ng + n].reshape(npz, -1)
        q2 = remap(np.ascontiguousarray(pe1), np.ascontiguousarray(qi), np.ascontiguousarray(pe2))
        q = q.copy()
        q[0][:, ng:ng + n, ng:ng + n] = q2.reshape(npz, n, n)
        dp = dp.copy()
        dp[:, ng:ng + n, ng:ng + n] = np.diff(pe2, axis=0).reshape(npz, n, n)
        t += P.dt
    return q, t


def oracle_run(P, exact_halo, nsteps=NSTEPS):
    import oracle as O
    g = P.geoms[0]

    def advect(q, dp, mfx, mfy, cx, cy, refresh):
        out = O.tracer_2d(q, dp, mfx, mfy, cx, cy, g, hord=8, q_split=1,
                          halo_fn=lambda p, nq, npz, ctx: refresh(np.ctypeslib.as_array(p, shape=q.shape)))
        return out[0], out[1], out[6]

    def remap(pe1, qi, pe2):
        return O.remap_columns(pe1, qi, pe2, iv=0, kord=9)

    return run(P, exact_halo, advect, remap, nsteps)


def device_run(P, exact_halo, nsteps=NSTEPS):
    from fv3atm_gb300 import api
    g = P.geoms[0]
    n, npz = P.n, P.npz

    def advect(q, dp, mfx, mfy, cx, cy, refresh):
        qg = q.copy()
        ns = api.tracer_2d(qg, dp, mfx.copy(), mfy.copy(), cx.copy(), cy.copy(), api.GridStruct(g), api.bounds_for(n),
                           n + 1, n + 1, npz, 1, 8, 1, P.dt, halo_update=refresh)
        return qg, dp, ns

    def remap(pe1, qi, pe2):
        q2 = np.zeros((1, npz, n, n))
        api.map_scalar_3d(npz, np.ascontiguousarray(pe1.reshape(npz + 1, n, n)),
                          np.ascontiguousarray(qi.reshape(1, npz, n, n)), None, npz,
                          np.ascontiguousarray(pe2.reshape(npz + 1, n, n)), q2, 1, n, 1, n, 1, n, 1, n, 1, 0, 9, 0.0)
        return q2.reshape(npz, n * n)

    return run(P, exact_halo, advect, remap, nsteps)
