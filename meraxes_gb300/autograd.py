"""Gradients of a 21 cm power-spectrum loss through the reionization step.

`DeltaT21` is the brightness-temperature box of one snapshot (ComputeTs ->
find_HII_bubbles -> 21cm box, src/core/ComputeTs.c, find_HII_bubbles.c,
BrightnessTemperature.c) as a function of the SFR grid, the stars grid as
find_HII_bubbles reads it (escape-fraction weighted), LXrayGal and E0
(NuXrayGalThreshold).  Its backward is the library's hand-written adjoint
(mx_adjoint_device): the 40 ComputeTs shells are recomputed, the ionisation
flags are held fixed, and xH enters through the partial ionisation of the last
filter step.  `PSLoss21` is the binned power-spectrum loss (mx_ps_loss_device).

Both run on CUDA tensors through the library's C ABI; there is no CPU path.
"""
from __future__ import annotations

import math
from typing import Dict, Sequence

import torch

# state grids the forward reads and updates (copied, so the caller's state is
# not changed)
STATE = ["deltax", "weighted_sfr", "x_e_box", "x_e_box_prev", "Tk_box", "N_rec", "z_at_ionization",
         "J_21_at_ionization", "Gamma12", "sfr_histories", "xH", "r_bubble", "J_21", "TS_box", "delta_T"]


class DeltaT21(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sfr, stars, lx, e0, step, snapshot: int, state: Dict[str, torch.Tensor]):
        step.set_xray(float(lx), float(e0))
        grids = {k: v.clone() for k, v in state.items() if v is not None}
        grids["sfr"] = sfr.detach().clone()
        grids["stars"] = stars.detach().clone()
        x_e_prev0 = grids["x_e_box_prev"].clone()
        tk0 = grids["Tk_box"].clone()
        step.step(snapshot, grids)
        saved = {"deltax": grids["deltax"], "stars": stars.detach(), "sfr": sfr.detach(),
                 "x_e_box_prev": x_e_prev0, "Tk_box": tk0, "x_e_box": grids["x_e_box"], "xH": grids["xH"],
                 "TS_box": grids["TS_box"]}
        if "sfr_histories" in grids:
            saved["sfr_histories"] = grids["sfr_histories"]
        ctx.step, ctx.snapshot, ctx.saved_grids = step, snapshot, saved
        ctx.lx, ctx.e0 = float(lx), float(e0)
        return grids["delta_T"]

    @staticmethod
    def backward(ctx, g_dT):
        step = ctx.step
        step.set_xray(ctx.lx, ctx.e0)
        gs, gst, dlx, de0 = step.adjoint(ctx.snapshot, ctx.saved_grids, g_dT.contiguous())
        dev = g_dT.device
        return (gs, gst, torch.tensor(dlx, dtype=torch.float64, device=dev),
                torch.tensor(de0, dtype=torch.float64, device=dev), None, None, None)


class PSLoss21(torch.autograd.Function):
    @staticmethod
    def forward(ctx, delta_T, step, edges: Sequence[float], target: Sequence[float]):
        loss, _, grad = step.ps_loss(delta_T.detach().contiguous(), edges, target, grad=True)
        ctx.save_for_backward(grad)
        return torch.tensor(loss, dtype=torch.float64, device=delta_T.device)

    @staticmethod
    def backward(ctx, g):
        (grad,) = ctx.saved_tensors
        return grad * g.to(grad.dtype), None, None, None


def log_bins(step, nbins: int = 20):
    """nbins log-spaced bin edges from the fundamental mode 2 pi / (BoxSize/h)
    to the Nyquist mode D/2 times it (1/Mpc)."""
    p = step.params
    dk = 2.0 * math.pi / (p.box_size / p.hubble_h)
    kmax = dk * p.grid_dim / 2
    return [dk * (kmax / dk) ** (i / nbins) for i in range(nbins + 1)]


__all__ = ["DeltaT21", "PSLoss21", "log_bins", "STATE"]
