"""torch.autograd.Function wrappers of the fv3g tangent-linear / adjoint entries
(test harness only: gradcheck drives the adjoint through them).

The forward passes call the exact-shape forward entries (fv3g_fv_tp_2d,
fv3g_map1_ppm); the backward passes call the adjoint entries at the same
trajectory.  Courant numbers, mass fluxes and pressures are constants.
"""
import numpy as np
import torch

from fv3atm_gb300 import api


class FvTp2d(torch.autograd.Function):
    """q (isd:ied, jsd:jed) -> (fx, fy) of fv_tp_2d for fixed winds."""

    @staticmethod
    def forward(ctx, q, args):
        qn = np.ascontiguousarray(q.detach().cpu().numpy(), dtype=np.float64)
        n = args["n"]
        fx, fy = np.zeros((n, n + 1)), np.zeros((n + 1, n))
        api.fv_tp_2d(qn.copy(), args["cx"], args["cy"], n + 1, n + 1, args["hord"], fx, fy, args["xfx"], args["yfx"],
                     args["grid"], args["bd"], args["rax"], args["ray"], 1.0, args["mfx"], args["mfy"])
        ctx.args, ctx.q = args, qn
        return torch.from_numpy(fx), torch.from_numpy(fy)

    @staticmethod
    def backward(ctx, gfx, gfy):
        a, n = ctx.args, ctx.args["n"]
        q_ad = np.zeros_like(ctx.q)
        fx_ad = np.ascontiguousarray(gfx.cpu().numpy(), dtype=np.float64).copy()
        fy_ad = np.ascontiguousarray(gfy.cpu().numpy(), dtype=np.float64).copy()
        api.fv_tp_2d_ad(ctx.q, q_ad, a["cx"], a["cy"], n + 1, n + 1, a["hord"], fx_ad, fy_ad, a["xfx"], a["yfx"],
                        a["grid"], a["bd"], a["rax"], a["ray"], 1.0, a["mfx"], a["mfy"])
        return torch.from_numpy(q_ad), None


class Map1Ppm(torch.autograd.Function):
    """q1 (km, ni) of one row -> q2 (kn, ni) of map1_ppm for fixed pressures."""

    @staticmethod
    def forward(ctx, q1, args):
        q1n = np.ascontiguousarray(q1.detach().cpu().numpy(), dtype=np.float64)
        km, ni = q1n.shape
        kn = args["pe2"].shape[0] - 1
        src = np.ascontiguousarray(q1n[:, None, :])
        q2 = np.zeros((kn, 1, ni))
        api.map1_ppm(km, args["pe1"], src, None, kn, args["pe2"], q2, 1, ni, 1, 1, ni, 1, 1, args["iv"], args["kord"])
        ctx.args, ctx.q1 = args, src
        return torch.from_numpy(q2[:, 0, :].copy())

    @staticmethod
    def backward(ctx, g2):
        a = ctx.args
        km, _, ni = ctx.q1.shape
        kn = a["pe2"].shape[0] - 1
        q1_ad = np.zeros_like(ctx.q1)
        q2_ad = np.ascontiguousarray(g2.cpu().numpy(), dtype=np.float64)[:, None, :].copy()
        api.map1_ppm_ad(km, a["pe1"], ctx.q1, q1_ad, None, kn, a["pe2"], q2_ad, 1, ni, 1, 1, ni, 1, 1, a["iv"],
                        a["kord"])
        return torch.from_numpy(q1_ad[:, 0, :].copy()), None
