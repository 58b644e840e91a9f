"""Cubed-sphere geometry and topology (no GPU)."""
import numpy as np

import oracle as O
from fv3atm_gb300 import grid as G
from fv3atm_gb300 import synth as S


def test_topology_is_a_consistent_involution():
    topo = G.cube_topology()
    for t in range(6):
        for e in range(4):
            nt, ne, rev = topo[t, e]
            assert nt != t
            assert tuple(topo[nt, ne]) == (t, e, rev)


def test_halo_cells_share_the_cube_edge_with_their_source_cells():
    """A depth-1 halo cell is filled from the neighbour's cell that touches the same cube-edge segment
    (both segment end points coincide), and deeper halo cells come from deeper neighbour cells."""
    n, ng = 24, 3
    topo = G.cube_topology()
    geoms = [G.tile_geometry(n, t, ng) for t in range(6)]

    def corner(t, I, J):
        return geoms[t].corners[J - 1 + ng, I - 1 + ng]

    def cell_corners(t, i, j):
        return [corner(t, i, j), corner(t, i + 1, j), corner(t, i, j + 1), corner(t, i + 1, j + 1)]

    for t in range(6):
        for s in range(1, n + 1):
            for (i, j, seg) in ((0, s, ((1, s), (1, s + 1))), (n + 1, s, ((n + 1, s), (n + 1, s + 1))),
                                (s, 0, ((s, 1), (s + 1, 1))), (s, n + 1, ((s, n + 1), (s + 1, n + 1)))):
                st, si, sj = G.halo_source(topo, n, t, i, j)
                cc = cell_corners(st, si, sj)
                for (I, J) in seg:
                    p = corner(t, I, J)
                    assert min(np.linalg.norm(p - c) for c in cc) < 1e-12, (t, i, j)
                for d in (2, 3):  # deeper halo cells: one cell further from the edge on the neighbour
                    ii = i if 1 <= i <= n else (i - (d - 1) if i < 1 else i + d - 1)
                    jj = j if 1 <= j <= n else (j - (d - 1) if j < 1 else j + d - 1)
                    st2, si2, sj2 = G.halo_source(topo, n, t, ii, jj)
                    assert st2 == st and abs(si2 - si) + abs(sj2 - sj) == d - 1


def test_face_metrics_close_the_sphere():
    geoms = G.cube_geometry(20)
    s = slice(3, 23)
    total = sum(g.area[s, s].sum() for g in geoms)
    assert abs(total - 4 * np.pi * G.RADIUS ** 2) <= 1e-9 * total
    for g in geoms:
        assert np.all(g.sin_sg[:4] > 0.5) and np.all(g.sin_sg[:4] <= 1.0)
        assert np.allclose(g.rarea * g.area, 1.0)


def test_area_fluxes_from_stream_function_are_nondivergent():
    g = G.tile_geometry(16, 2)
    psi = S.solid_body_psi(g.corners, 40.0) + 1e6 * S.sph_harm_psi(g.corners, 6, np.random.default_rng(1))
    ax, ay = S.area_fluxes_from_psi(psi)
    div = ax[:, 1:] - ax[:, :-1] + ay[1:, :] - ay[:-1, :]
    assert np.abs(div).max() <= 1e-9 * np.abs(ax).max()


def test_shared_edge_mass_fluxes_are_single_valued():
    P = S.make_problem(14, 3, 1, seed=3)
    topo = P.topo
    mfx, mfy, n = P.mfx.numpy(), P.mfy.numpy(), P.n

    def outward(t, e):
        return {0: -mfx[t, :, :, 0], 1: mfx[t, :, :, n], 2: -mfy[t, :, 0, :], 3: mfy[t, :, n, :]}[e]

    for t in range(6):
        for e in range(4):
            nt, ne, rev = topo[t, e]
            a = outward(t, e)
            b = outward(nt, ne)
            b = b[:, ::-1] if rev else b
            assert np.array_equal(a, -b)


def test_hybrid_levels_are_monotone_for_surface_pressures():
    for km in (32, 63, 64, 127):
        ak, bk = G.hybrid_levels(km)
        assert bk[0] == 0 and bk[-1] == 1 and ak[-1] == 0
        for ps in (90000.0, 101325.0, 110000.0):
            assert np.all(np.diff(ak + bk * ps) > 0)


def test_oracle_halo_fill_matches_python_exchange():
    P = S.make_problem(13, 2, 2, seed=2)
    q = P.q.numpy().copy()
    q[..., :3, :] = -1.0
    q[..., -3:, :] = -1.0
    q[..., :, :3] = -1.0
    q[..., :, -3:] = -1.0
    a = O.cube_halo_fill(q, P.n, P.topo)
    import torch
    b = S.fill_cube_halo(torch.as_tensor(q).reshape(6, -1, P.nd, P.nd).clone(), P.n, 3, P.topo).numpy()
    assert np.array_equal(a.reshape(b.shape), b)
