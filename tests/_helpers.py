"""Shared helpers of the test-suite (problem builders, norms, oracle glue)."""
from __future__ import annotations

import numpy as np

from fv3atm_gb300 import grid as G
from fv3atm_gb300 import synth as S


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))


def interior(x, n: int, ng: int = 3):
    return x[..., ng:ng + n, ng:ng + n]


def area_fluxes(cx, cy, g: G.TileGeom):
    """xfx (nd, n+1), yfx (n+1, nd) from Courant numbers, as tracer_2d computes them."""
    n, ng = g.n, g.ng
    dxa, dya, dx, dy, sin = g.dxa, g.dya, g.dx, g.dy, g.sin_sg
    xf = np.where(cx > 0, cx * dxa[:, ng - 1:ng + n] * dy[:, ng:ng + n + 1] * sin[2][:, ng - 1:ng + n],
                  cx * dxa[:, ng:ng + n + 1] * dy[:, ng:ng + n + 1] * sin[0][:, ng:ng + n + 1])
    yf = np.where(cy > 0, cy * dya[ng - 1:ng + n, :] * dx[ng:ng + n + 1, :] * sin[3][ng - 1:ng + n, :],
                  cy * dya[ng:ng + n + 1, :] * dx[ng:ng + n + 1, :] * sin[1][ng:ng + n + 1, :])
    return xf, yf


def ra_xy(xfx, yfx, g: G.TileGeom):
    """ra_x (nd, n) over rows jsd..jed, ra_y (n, nd) over columns isd..ied."""
    n, ng = g.n, g.ng
    rax = g.area[:, ng:ng + n] + xfx[:, :-1] - xfx[:, 1:]
    ray = g.area[ng:ng + n, :] + yfx[:-1, :] - yfx[1:, :]
    return rax, ray


def final_dp(dp_last, mfx, mfy, geoms, nsplt: int, n: int, ng: int = 3):
    """Layer thickness after the last substep from the thickness at its start."""
    out = np.array(dp_last, dtype=np.float64, copy=True)
    s = slice(ng, ng + n)
    fr = 1.0 / nsplt
    for t, g in enumerate(geoms):
        mx = mfx[t] * fr if nsplt != 1 else mfx[t]
        my = mfy[t] * fr if nsplt != 1 else mfy[t]
        out[t][..., s, s] = dp_last[t][..., s, s] + (mx[..., :-1] - mx[..., 1:] + my[..., :-1, :] - my[..., 1:, :]) \
            * g.rarea[s, s]
    return out


def remap_reference(q, dp, ak, bk, n: int, kord: int = 9, iv: int = 0, ng: int = 3):
    """Oracle remap of every interior column of q (6, nq, npz, nd, nd) on thickness dp (6, npz, nd, nd)."""
    import oracle as O
    T, nq, npz = q.shape[:3]
    s = slice(ng, ng + n)
    dpi = dp[:, :, s, s].transpose(1, 0, 2, 3).reshape(npz, -1)        # (npz, ncol)
    pe1 = np.concatenate([np.full((1, dpi.shape[1]), ak[0]), ak[0] + np.cumsum(dpi, axis=0)], axis=0)
    pe2 = ak[:, None] + bk[:, None] * pe1[-1][None, :]
    out = np.zeros_like(q)
    for iq in range(nq):
        qi = q[:, iq][:, :, s, s].transpose(1, 0, 2, 3).reshape(npz, -1)
        r = O.remap_columns(pe1, qi, pe2, iv=iv, kord=kord)
        out[:, iq][:, :, s, s] = r.reshape(npz, T, n, n).transpose(1, 0, 2, 3)
    dp2 = np.diff(pe2, axis=0).reshape(npz, T, n, n).transpose(1, 0, 2, 3)
    return out, dp2, pe1, pe2


def cube_mass(q, dp, geoms, n: int, ng: int = 3):
    """Per-tracer compensated global mass with the oracle's summation."""
    import oracle as O
    s = slice(ng, ng + n)
    nq, npz = q.shape[1], q.shape[2]
    tot = np.zeros(nq)
    for iq in range(nq):
        for t in range(6):
            a = geoms[t].area[s, s].ravel()
            tot[iq] += O.mass_sum(q[t, iq][:, s, s].reshape(npz, -1), dp[t][:, s, s].reshape(npz, -1), a)
    return tot


def problem(n=30, npz=5, nq=3, seed=3, **kw) -> S.Problem:
    return S.make_problem(n, npz, nq, seed=seed, **kw)


class _SubGeom:
    """The metric arrays of one rank's part of a tile (attributes as TileGeom's)."""


def sub_domain(P: S.Problem, t: int, is_: int, ie: int, js: int, je: int, ng: int = 3):
    """The arrays of the rank that owns cells [is_, ie] x [js, je] (1-based) of tile t with its own ng-cell halo:
    (geom, [q, dp, mfx, mfy, cx, cy]) shaped as that rank's Fortran arguments, halos from the full tile."""
    g = P.geoms[t]
    ci, cj = slice(is_ - 1, ie + 2 * ng), slice(js - 1, je + 2 * ng)          # data-domain cells
    fi, fj = slice(is_ - 1, ie + 2 * ng + 1), slice(js - 1, je + 2 * ng + 1)  # faces bounding them
    sg = _SubGeom()
    sg.dx, sg.del6_u = g.dx[fj, ci], g.del6_u[fj, ci]
    sg.dy, sg.del6_v = g.dy[cj, fi], g.del6_v[cj, fi]
    for name in ("dxa", "dya", "area", "rarea"):
        setattr(sg, name, getattr(g, name)[cj, ci])
    sg.sin_sg = g.sin_sg[:, cj, ci]
    q = P.q[t].numpy()[..., cj, ci]
    dp = P.dp[t].numpy()[..., cj, ci]
    mfx = P.mfx[t].numpy()[..., js - 1:je, is_ - 1:ie + 1]
    mfy = P.mfy[t].numpy()[..., js - 1:je + 1, is_ - 1:ie]
    cx = P.cx[t].numpy()[..., cj, is_ - 1:ie + 1]
    cy = P.cy[t].numpy()[..., js - 1:je + 1, ci]
    return sg, [np.ascontiguousarray(a, dtype=np.float64) for a in (q, dp, mfx, mfy, cx, cy)]
