"""Single-tile states (one cube face, halo ring prescribed by the caller and held
over the step) against the oracle, and ensembles of independent states advanced
by one graph against the same members stepped one by one."""
import numpy as np
import pytest

import oracle as O
from fv3atm_gb300 import api
from fv3atm_gb300 import synth as S

from ._helpers import final_dp, interior, rel_l2, remap_reference

pytestmark = pytest.mark.gpu


def _oracle_single_tile(P, q_split):
    g = P.geoms[0]
    q0 = np.ascontiguousarray(P.q[0].numpy())
    n, ng = P.n, 3

    def restore(qarr):  # the prescribed ring, as the state holds it over the step
        keep = qarr[..., ng:ng + n, ng:ng + n].copy()
        qarr[...] = q0
        qarr[..., ng:ng + n, ng:ng + n] = keep

    args = [np.ascontiguousarray(a[0].numpy()) for a in (P.dp, P.mfx, P.mfy, P.cx, P.cy)]
    out = O.tracer_2d(q0, *args, g, hord=8, q_split=q_split,
                      halo_fn=lambda p, nq, npz, ctx: restore(np.ctypeslib.as_array(p, shape=q0.shape)))
    dpf = final_dp(out[1][None], P.mfx.numpy(), P.mfy.numpy(), P.geoms, out[6], n)
    q2, _, _, _ = remap_reference(out[0][None], dpf, P.ak, P.bk, n)
    return q2


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-5)])
def test_single_tile_state_matches_oracle_with_prescribed_halo(cuda, precision, tol):
    P = S.make_problem(30, 5, 2, ntiles=1, seed=31, cmax=0.7)
    st = api.CubeState(P.n, P.npz, P.nq, precision=precision, ntiles=1)
    st.load_problem(P)
    st.step(2)
    got = st.download("Q_REMAPPED")
    want = _oracle_single_tile(P, 2)
    for iq in range(P.nq):
        assert rel_l2(interior(got[:, iq], P.n), interior(want[:, iq], P.n)) <= tol


def test_ensemble_step_equals_members_stepped_alone(cuda):
    import torch
    specs = [(12, 4, 2, 1), (20, 6, 3, 1), (30, 3, 2, 1), (14, 3, 2, 6)]  # (n, npz, nq, ntiles)
    probs = [S.make_problem(n, npz, nq, ntiles=nt, seed=40 + k, cmax=0.7) for k, (n, npz, nq, nt) in
             enumerate(specs)]

    def states():
        out = []
        for (n, npz, nq, nt), P in zip(specs, probs):
            st = api.CubeState(n, npz, nq, precision="mixed", ntiles=nt)
            st.load_problem(P)
            out.append(st)
        return out

    alone = states()
    for st in alone:
        st.step(2)
    together = states()
    ens = api.Ensemble(together)
    ens.step(2)
    torch.cuda.synchronize()  # the graph ran on the ensemble's stream
    for a, b in zip(alone, together):
        assert np.array_equal(a.download("Q_REMAPPED"), b.download("Q_REMAPPED"))
    # a second ensemble step reuses the captured graph
    for st, P in zip(together, probs):
        st.upload("Q", P.q.numpy())
    ens.step(2)
    torch.cuda.synchronize()
    for a, b in zip(alone, together):
        assert np.array_equal(a.download("Q_REMAPPED"), b.download("Q_REMAPPED"))
    ens.close()
