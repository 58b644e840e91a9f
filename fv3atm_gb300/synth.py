"""Seeded synthetic inputs for the tracer path (no public dataset exists for it).

Builds, for one tile or the six-tile cube:

* C-grid area fluxes from a stream function sampled at cell corners, so that
  every cell's area-flux divergence telescopes to zero: a solid-body rotation
  tilted 45 degrees, optionally plus a random spherical-harmonic perturbation
  up to degree 20;
* Courant numbers cx/cy inverted from those fluxes through the same upwind
  metric that ``tracer_2d`` uses to rebuild xfx/yfx;
* Lagrangian layer thicknesses on a synthetic hybrid coordinate with seeded
  perturbations that keep column mass, and upwind mass fluxes mfx/mfy;
* tracers: cosine bells of radius R/3 or Gaussian blobs plus 1 % uniform
  noise, clipped at zero.

Shapes follow the Fortran argument shapes of ``tracer_2d`` (i fastest):
q (6, nq, npz, nd, nd), dp (6, npz, nd, nd), cx (6, npz, nd, n+1),
cy (6, npz, n+1, nd), mfx (6, npz, n, n+1), mfy (6, npz, n+1, n) with
nd = n + 2*ng.  The 2-D ingredients are numpy float64; the 3-D/4-D fields are
torch tensors built on the requested device, so full-size problems are
extruded in device memory.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from . import grid as G

TILT = math.radians(45.0)


def _axis(tilt: float = TILT) -> np.ndarray:
    return np.array([-math.sin(tilt), 0.0, math.cos(tilt)])


def solid_body_psi(p: np.ndarray, u0: float, tilt: float = TILT, radius: float = G.RADIUS) -> np.ndarray:
    """Stream function (m^2/s) of a solid-body rotation with equatorial speed u0."""
    return -u0 * radius * (p @ _axis(tilt))


def rotate(p: np.ndarray, angle: float, tilt: float = TILT) -> np.ndarray:
    """Rotate unit vectors about the tilted axis (Rodrigues)."""
    k = _axis(tilt)
    c, s = math.cos(angle), math.sin(angle)
    return p * c + np.cross(k, p) * s + np.outer((p @ k), k).reshape(p.shape) * (1.0 - c)


def sph_harm_psi(p: np.ndarray, lmax: int, rng: np.random.Generator) -> np.ndarray:
    """Random real spherical-harmonic series up to degree lmax (unit-free)."""
    z = np.clip(p[..., 2], -1.0, 1.0)
    lam = np.arctan2(p[..., 1], p[..., 0])
    st = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    out = np.zeros_like(z)
    pmm = np.ones_like(z)
    for m in range(lmax + 1):
        if m > 0:
            pmm = pmm * math.sqrt((2.0 * m + 1.0) / (2.0 * m)) * st
        cm, sm = np.cos(m * lam), np.sin(m * lam)
        p_lm2, p_lm1 = None, pmm
        for l in range(m, lmax + 1):
            if l == m:
                plm = pmm
            elif l == m + 1:
                plm = math.sqrt(2.0 * m + 3.0) * z * pmm
            else:
                a = math.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
                b = math.sqrt(((l - 1.0) ** 2 - m * m) / (4.0 * (l - 1.0) ** 2 - 1.0))
                plm = a * (z * p_lm1 - b * p_lm2)
            if l > m:
                p_lm2, p_lm1 = p_lm1, plm
            if l >= 1:
                w = l ** -1.0
                out += w * plm * (rng.standard_normal() * cm + (rng.standard_normal() * sm if m > 0 else 0.0))
    return out


def area_fluxes_from_psi(psi_c: np.ndarray) -> tuple:
    """Area fluxes (m^2/s) through x faces (nd, nd+1) and y faces (nd+1, nd).

    psi_c holds psi at cell corners, shape (nd+1, nd+1) [J, I].  The flux
    through an x face (toward +i) is psi(south end) - psi(north end); through a
    y face (toward +j) it is psi(east end) - psi(west end).
    """
    ax = psi_c[:-1, :] - psi_c[1:, :]
    ay = psi_c[:, 1:] - psi_c[:, :-1]
    return ax, ay


def courant_from_area_flux(g: G.TileGeom, ax: np.ndarray, ay: np.ndarray) -> tuple:
    """cx on x faces is..ie+1 (rows jsd..jed), cy on y faces js..je+1 (cols isd..ied).

    ax/ay are area fluxes per step (m^2).  Inverts tracer_2d's
    xfx = cx * dxa(upwind) * dy * sin_sg(upwind edge).
    """
    n, ng = g.n, g.ng
    axf = ax[:, ng:ng + n + 1]                  # faces I = 1..n+1
    dy = g.dy[:, ng:ng + n + 1]
    up_pos = g.dxa[:, ng - 1:ng + n] * g.sin_sg[2][:, ng - 1:ng + n]   # cell i-1, east edge
    up_neg = g.dxa[:, ng:ng + n + 1] * g.sin_sg[0][:, ng:ng + n + 1]    # cell i, west edge
    cx = np.where(axf > 0, axf / (up_pos * dy), axf / (up_neg * dy))
    ayf = ay[ng:ng + n + 1, :]
    dx = g.dx[ng:ng + n + 1, :]
    upp = g.dya[ng - 1:ng + n, :] * g.sin_sg[3][ng - 1:ng + n, :]
    upn = g.dya[ng:ng + n + 1, :] * g.sin_sg[1][ng:ng + n + 1, :]
    cy = np.where(ayf > 0, ayf / (upp * dx), ayf / (upn * dx))
    return cx, cy


def bell(p: np.ndarray, center: np.ndarray, r0: float = 1.0 / 3.0) -> np.ndarray:
    """Cosine bell of angular radius r0 (in radians of arc on the unit sphere)."""
    r = np.arccos(np.clip(p @ center, -1.0, 1.0))
    return np.where(r < r0, 0.5 * (1.0 + np.cos(math.pi * r / r0)), 0.0)


def gaussian(p: np.ndarray, center: np.ndarray, width: float = 0.25) -> np.ndarray:
    r2 = np.sum((p - center) ** 2, axis=-1)
    return np.exp(-r2 / (width * width))


def lonlat_vec(lon_deg: float, lat_deg: float) -> np.ndarray:
    lo, la = math.radians(lon_deg), math.radians(lat_deg)
    return np.array([math.cos(la) * math.cos(lo), math.cos(la) * math.sin(lo), math.sin(la)])


def level_weights(npz: int) -> np.ndarray:
    """Vertical profile of the wind speed, 0.5 .. 1."""
    k = np.arange(npz, dtype=np.float64)
    return 0.5 + 0.5 * np.sin(math.pi * (k + 0.5) / npz)


def random_centers(nq: int, rng: np.random.Generator) -> np.ndarray:
    v = rng.standard_normal((nq, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


# ---------------------------------------------------------------- problems ---
@dataclasses.dataclass
class Problem:
    """One tracer_2d + remap problem: six tiles (cube) or one tile."""

    n: int
    ng: int
    npz: int
    nq: int
    ntiles: int
    geoms: list
    topo: np.ndarray
    ak: np.ndarray
    bk: np.ndarray
    dt: float
    # torch tensors (float64) -- see module docstring for shapes
    q: object
    dp: object
    cx: object
    cy: object
    mfx: object
    mfy: object
    meta: dict

    @property
    def nd(self) -> int:
        return self.n + 2 * self.ng


def _halo_index(n: int, ng: int, topo: np.ndarray, ntiles: int = 6) -> tuple:
    """Flat (tile*nd*nd + j*nd + i) destination/source indices of every edge-halo cell."""
    nd = n + 2 * ng
    dst, src = [], []
    for t in range(ntiles):
        for j in range(1 - ng, n + ng + 1):
            for i in range(1 - ng, n + ng + 1):
                inside_i, inside_j = 1 <= i <= n, 1 <= j <= n
                if inside_i == inside_j:  # interior or corner block
                    continue
                st, si, sj = G.halo_source(topo, n, t, i, j)
                dst.append(t * nd * nd + (j - 1 + ng) * nd + (i - 1 + ng))
                src.append(st * nd * nd + (sj - 1 + ng) * nd + (si - 1 + ng))
    return np.asarray(dst, dtype=np.int64), np.asarray(src, dtype=np.int64)


def fill_cube_halo(x, n: int, ng: int, topo: np.ndarray):
    """Edge-halo exchange of a torch tensor shaped (6, ..., nd, nd), in place."""
    import torch
    dst, src = _halo_index(n, ng, topo)
    nd = n + 2 * ng
    v = x.movedim(0, -3).reshape(*x.shape[1:-2], 6 * nd * nd)
    if v.data_ptr() == x.data_ptr():  # the reshape returned a view (one plane per tile): work on a copy
        v = v.clone()
    d = torch.as_tensor(dst, device=x.device)
    s = torch.as_tensor(src, device=x.device)
    v[..., d] = v[..., s]
    x.copy_(v.reshape(*x.shape[1:-2], 6, nd, nd).movedim(-3, 0))
    return x


def stack_tiles(probs: list) -> "Problem":
    """Single-tile problems of one size (n, npz, nq) as one problem of len(probs) independent tiles (the
    layout of a state with independent_tiles): each tile keeps its grid, fields and halo ring."""
    import torch
    p0 = probs[0]
    for p in probs:
        if (p.n, p.npz, p.nq, p.ntiles) != (p0.n, p0.npz, p0.nq, 1):
            raise ValueError("stack_tiles takes single-tile problems of one size")
    cat = lambda name: torch.cat([torch.as_tensor(getattr(p, name)) for p in probs], dim=0)
    return Problem(n=p0.n, ng=p0.ng, npz=p0.npz, nq=p0.nq, ntiles=len(probs), geoms=[p.geoms[0] for p in probs],
                   topo=p0.topo, ak=p0.ak, bk=p0.bk, dt=p0.dt, q=cat("q"), dp=cat("dp"), cx=cat("cx"), cy=cat("cy"),
                   mfx=cat("mfx"), mfy=cat("mfy"), meta=dict(members=[p.meta for p in probs]))


def make_problem(n: int, npz: int, nq: int, *, ntiles: int = 6, seed: int = 0, cmax: float = 0.8,
                 u0: float = 40.0, pert_amp: float = 10.0, lmax: int = 20, dp_noise: float = 0.10,
                 ps_range: tuple = (95000.0, 103000.0), tracer_kind: str = "mixed", noise: float = 0.01,
                 device: str = "cpu", ng: int = 3) -> Problem:
    """Build a seeded problem.  ntiles=6: the cube; ntiles=1: tile 0 alone."""
    import torch
    rng = np.random.default_rng(seed)
    nd = n + 2 * ng
    topo = G.cube_topology()
    geoms = G.cube_geometry(n, ng) if ntiles == 6 else [G.tile_geometry(n, 0, ng)]
    ak, bk = G.hybrid_levels(npz)

    # stream function: solid body + optional random perturbation
    pert_rng = np.random.default_rng(seed + 7919)
    ax_l, ay_l = [], []
    for g in geoms:
        psi = solid_body_psi(g.corners, u0)
        ax, ay = area_fluxes_from_psi(psi)
        ax_l.append(ax)
        ay_l.append(ay)
    if pert_amp > 0.0:
        pax, pay = [], []
        state = pert_rng.bit_generator.state
        for g in geoms:
            pert_rng.bit_generator.state = state  # identical series on every tile
            ps_ = sph_harm_psi(g.corners, lmax, pert_rng)
            a, b = area_fluxes_from_psi(ps_)
            pax.append(a)
            pay.append(b)
        vmax = max(max(np.abs(a[ng:-ng, :]).max() / g.dy[ng:-ng, :].max(), np.abs(b[:, ng:-ng]).max() /
                       g.dx[:, ng:-ng].max()) for a, b, g in zip(pax, pay, geoms))
        scale = pert_amp / vmax
        ax_l = [a + scale * p for a, p in zip(ax_l, pax)]
        ay_l = [a + scale * p for a, p in zip(ay_l, pay)]

    # time step from the target Courant number (interior faces, full wind)
    cfl = 0.0
    for g, ax, ay in zip(geoms, ax_l, ay_l):
        cx, cy = courant_from_area_flux(g, ax, ay)
        cfl = max(cfl, np.abs(cx[ng:ng + n, :]).max(), np.abs(cy[:, ng:ng + n]).max())
    dt = cmax / cfl
    wk = level_weights(npz)

    dev = torch.device(device)
    f64 = torch.float64
    T = len(geoms)
    cx3 = torch.empty((T, npz, nd, n + 1), dtype=f64, device=dev)
    cy3 = torch.empty((T, npz, n + 1, nd), dtype=f64, device=dev)
    for t, (g, ax, ay) in enumerate(zip(geoms, ax_l, ay_l)):
        cx, cy = courant_from_area_flux(g, ax * dt, ay * dt)
        cx3[t] = torch.as_tensor(cx, device=dev)[None] * torch.as_tensor(wk, device=dev)[:, None, None]
        cy3[t] = torch.as_tensor(cy, device=dev)[None] * torch.as_tensor(wk, device=dev)[:, None, None]

    # Lagrangian layer thickness: perturbed hybrid layers, column mass kept
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed * 1000 + 17)
    ps = torch.empty((T, nd, nd), dtype=f64, device=dev).uniform_(ps_range[0], ps_range[1], generator=gen)
    dak = torch.as_tensor(np.diff(ak), device=dev)
    dbk = torch.as_tensor(np.diff(bk), device=dev)
    dref = dak[None, :, None, None] + dbk[None, :, None, None] * ps[:, None]
    r = torch.empty((T, npz, nd, nd), dtype=f64, device=dev).uniform_(-1.0, 1.0, generator=gen)
    dp = dref * (1.0 + dp_noise * r)
    dp = dp * (dref.sum(1, keepdim=True) / dp.sum(1, keepdim=True))
    if T == 6:
        fill_cube_halo(dp, n, ng, topo)

    # upwind mass fluxes on interior faces
    s = slice(ng, ng + n)
    cxi = cx3[:, :, s, :]                        # rows js..je
    cyi = cy3[:, :, :, s]                        # cols is..ie
    xfx = torch.empty_like(cxi)
    yfx = torch.empty_like(cyi)
    for t, g in enumerate(geoms):
        dxa = torch.as_tensor(g.dxa, device=dev)
        dya = torch.as_tensor(g.dya, device=dev)
        sin = torch.as_tensor(g.sin_sg, device=dev)
        dyf = torch.as_tensor(g.dy, device=dev)[s, ng:ng + n + 1]
        dxf = torch.as_tensor(g.dx, device=dev)[ng:ng + n + 1, s]
        upx_p = (dxa * sin[2])[s, ng - 1:ng + n]
        upx_n = (dxa * sin[0])[s, ng:ng + n + 1]
        xfx[t] = torch.where(cxi[t] > 0, cxi[t] * upx_p * dyf, cxi[t] * upx_n * dyf)
        upy_p = (dya * sin[3])[ng - 1:ng + n, s]
        upy_n = (dya * sin[1])[ng:ng + n + 1, s]
        yfx[t] = torch.where(cyi[t] > 0, cyi[t] * upy_p * dxf, cyi[t] * upy_n * dxf)
    dpx_up = torch.where(cxi > 0, dp[:, :, s, ng - 1:ng + n], dp[:, :, s, ng:ng + n + 1])
    dpy_up = torch.where(cyi > 0, dp[:, :, ng - 1:ng + n, s], dp[:, :, ng:ng + n + 1, s])
    mfx = xfx * dpx_up
    mfy = yfx * dpy_up
    if T == 6:
        _sync_edges(mfx, mfy, n, topo, row_off=0)
        _sync_edges(cx3, cy3, n, topo, row_off=ng)
        fill_courant_halo(cx3, cy3, n, ng, topo)

    # tracers
    qrng = np.random.default_rng(seed + 31)
    centers = random_centers(nq, qrng)
    q = torch.zeros((T, nq, npz, nd, nd), dtype=f64, device=dev)
    vert = torch.as_tensor(0.6 + 0.4 * np.cos(np.linspace(0.0, math.pi, npz)), device=dev)
    for iq in range(nq):
        kind = tracer_kind if tracer_kind != "mixed" else ("bell" if iq % 2 == 0 else "gauss")
        for t, g in enumerate(geoms):
            base = bell(g.centers, centers[iq]) if kind == "bell" else gaussian(g.centers, centers[iq])
            q[t, iq] = torch.as_tensor(base, device=dev)[None] * vert[:, None, None]
    if noise > 0.0:  # drawn tracer by tracer: the first tracers do not depend on nq
        for iq in range(nq):
            q[:, iq] += noise * torch.empty_like(q[:, iq]).uniform_(-1.0, 1.0, generator=gen)
        q.clamp_(min=0.0)
    if T == 6:
        fill_cube_halo(q.view(6, nq * npz, nd, nd), n, ng, topo)
    return Problem(n=n, ng=ng, npz=npz, nq=nq, ntiles=T, geoms=geoms, topo=topo, ak=ak, bk=bk, dt=dt, q=q, dp=dp,
                   cx=cx3, cy=cy3, mfx=mfx, mfy=mfy, meta=dict(seed=seed, cmax=cmax, u0=u0, pert_amp=pert_amp,
                                                            centers=centers))


def fill_courant_halo(cx, cy, n: int, ng: int, topo: np.ndarray) -> None:
    """Courant numbers of the halo faces of six tiles from the faces they stand for (grid.face_source), as a
    halo update of the winds gives them: cx (6, npz, nd, n+1) on the halo rows, cy (6, npz, n+1, nd) on the
    halo columns.  The sources are interior or tile-edge faces, which this does not change."""
    import torch
    o = ng - 1
    halo = list(range(1 - ng, 1)) + list(range(n + 1, n + ng + 1))
    # (destination array, t, row, col) <- (source array, t, row, col, sign), grouped by the pair of arrays
    groups = {}
    for t in range(6):
        for j in halo:
            for i in range(1, n + 2):
                tt, fk, fi, fj, sign = G.face_source(topo, n, t, "x", i, j)
                src = (fj + o, fi - 1) if fk == "x" else (fj - 1, fi + o)
                groups.setdefault(("x", fk), []).append((t, j + o, i - 1, tt, *src, sign))
        for i in halo:
            for j in range(1, n + 2):
                tt, fk, fi, fj, sign = G.face_source(topo, n, t, "y", i, j)
                src = (fj + o, fi - 1) if fk == "x" else (fj - 1, fi + o)
                groups.setdefault(("y", fk), []).append((t, j - 1, i + o, tt, *src, sign))
    arrays = {"x": cx, "y": cy}
    for (dk, sk), rows in groups.items():
        idx = torch.as_tensor(np.array(rows, dtype=np.int64), device=cx.device)
        src = arrays[sk][idx[:, 3], :, idx[:, 4], idx[:, 5]] * idx[:, 6:7].to(cx.dtype)
        arrays[dk][idx[:, 0], :, idx[:, 1], idx[:, 2]] = src


def _sync_edges(xf, yf, n: int, topo: np.ndarray, row_off: int) -> None:
    """Make face fields on shared tile edges single-valued (owner = lower tile).

    xf: (6, npz, rows, n+1) with interior rows starting at row_off;
    yf: (6, npz, n+1, cols) with interior cols starting at row_off.
    """
    r = slice(row_off, row_off + n)

    def outward(t, e):
        if e == G.W:
            return -xf[t, :, r, 0]
        if e == G.E:
            return xf[t, :, r, n]
        if e == G.S:
            return -yf[t, :, 0, r]
        return yf[t, :, n, r]

    for t in range(6):
        for e in range(4):
            nt, ne, rev = (int(v) for v in topo[t, e])
            if nt > t:
                continue
            inflow = outward(nt, ne)
            if rev:
                inflow = inflow.flip(-1)
            if e == G.W:
                xf[t, :, r, 0] = inflow
            elif e == G.E:
                xf[t, :, r, n] = -inflow
            elif e == G.S:
                yf[t, :, 0, r] = inflow
            else:
                yf[t, :, n, r] = -inflow


def pressure_edges(dp, ak: np.ndarray, bk: np.ndarray):
    """pe1 (Lagrangian, from dp) and pe2 (hybrid, ps = column total), float64.

    dp: torch (..., npz, ...) with the level axis at -3 (levels, j, i).
    Returns tensors with npz+1 interfaces on that axis.
    """
    import torch
    ptop = float(ak[0])
    pe1 = torch.cat([torch.full_like(dp[..., :1, :, :], ptop), ptop + torch.cumsum(dp, dim=-3)], dim=-3)
    ps = pe1[..., -1:, :, :]
    a = torch.as_tensor(ak, device=dp.device, dtype=torch.float64).view(-1, 1, 1)
    b = torch.as_tensor(bk, device=dp.device, dtype=torch.float64).view(-1, 1, 1)
    pe2 = a + b * ps
    return pe1, pe2


# ------------------------------------------------- single-tile C48 problem ---
def c48_single_tile(n: int = 48, npz: int = 63, seed: int = 0, cmax: float = 0.4, u0: float = 40.0,
                    ps_noise: float = 0.05, noise: float = 0.01):
    """One C48 tile, one cosine-bell tracer, solid-body rotation tilted 45 deg,
    hybrid delp with ps = 1e5 +- 5 % (the target thickness is unperturbed).

    Returns (Problem, exact) where exact(t_seconds) gives the halo-ring values
    of the analytic rotated bell on the neighbouring tiles' cell centres,
    shape (npz, nd, nd) (interior and corner blocks left at zero)."""
    import torch
    P = make_problem(n, npz, 1, ntiles=1, seed=seed, cmax=cmax, u0=u0, pert_amp=0.0, dp_noise=0.0,
                     ps_range=(1.0e5 * (1 - ps_noise), 1.0e5 * (1 + ps_noise)), tracer_kind="bell", noise=0.0)
    ng = P.ng
    nd = n + 2 * ng
    g0 = P.geoms[0]
    center = lonlat_vec(-35.0, 8.0)
    vert = 0.6 + 0.4 * np.cos(np.linspace(0.0, math.pi, npz))
    rng = np.random.default_rng(seed + 99)
    base = bell(g0.centers, center)
    q = base[None] * vert[:, None, None] + noise * rng.uniform(-1.0, 1.0, (npz, nd, nd))
    P.q = torch.as_tensor(np.clip(q, 0.0, None)[None, None])  # (1, 1, npz, nd, nd)
    P.meta["center"] = center
    P.meta["omega"] = u0 / G.RADIUS
    P.meta["vert"] = vert
    topo = G.cube_topology()
    geoms = {t: G.tile_geometry(n, t, ng) for t in range(6)}
    omega = u0 / G.RADIUS
    halo_pts, halo_idx = [], []
    for j in range(1 - ng, n + ng + 1):
        for i in range(1 - ng, n + ng + 1):
            if (1 <= i <= n) == (1 <= j <= n):
                continue
            t, si, sj = G.halo_source(topo, n, 0, i, j)
            halo_pts.append(geoms[t].centers[sj - 1 + ng, si - 1 + ng])
            halo_idx.append((j - 1 + ng, i - 1 + ng))
    halo_pts = np.asarray(halo_pts)
    jj, ii = np.asarray(halo_idx).T

    def exact(t_seconds: float) -> np.ndarray:
        # the stream function above turns the field by -omega*t about the
        # tilted axis; sample the initial bell at the back-rotated positions
        back = rotate(halo_pts, -omega * t_seconds)
        out = np.zeros((npz, nd, nd))
        out[:, jj, ii] = bell(back, center)[None] * vert[:, None]
        return out

    return P, exact


def nest_strips(field_t0, field_t1, isd: int, jsd: int, npx: int, npy: int) -> dict:
    """Boundary states of a nested domain cut from two full fields (nq, npz, njd, nid) at the parent times t0
    and t1: {side: (t0, t1)} with the strips laid out as a nest's q_BC holds them, west (isd:0, jsd:jed),
    east (npx:ied, jsd:jed), south (isd:ied, jsd:0), north (isd:ied, npy:jed), each (nq, npz, rows, cols)."""
    out = {}
    for name, cut in (("west", np.s_[..., :, :1 - isd]), ("east", np.s_[..., :, npx - isd:]),
                      ("south", np.s_[..., :1 - jsd, :]), ("north", np.s_[..., npy - jsd:, :])):
        out[name] = tuple(np.ascontiguousarray(np.asarray(f)[cut], dtype=np.float64) for f in (field_t0, field_t1))
    return out
