"""torch.autograd bridge for gradient checks: the recorder misfit as a
differentiable function of the source series and the PML face scales.

The forward calls ard_adjoint, which computes the misfit and every gradient
in one pass (forward run + hand-written adjoint on the GPU); backward returns
the stored gradients scaled by the incoming gradient.  Inputs live on the
host (the C ABI takes host buffers); the work runs on the context's GPU.
"""
from __future__ import annotations

import numpy as np
import torch


class RecorderMisfit(torch.autograd.Function):
    """J = 0.5 sum_{t<T} sum_r (rec[t][r] - target[t][r])^2 of a one-scene
    Simulation created with adjoint=True.

        J = RecorderMisfit.apply(series, scale6, sim, T, target)

    series: [n_sources][T] tensor, scale6: [6] tensor (float32 values are
    what the library takes); gradients flow to both."""

    @staticmethod
    def forward(ctx, series, scale6, sim, T, target):
        s = series.detach().cpu().to(torch.float32).numpy()
        sc = scale6.detach().cpu().to(torch.float32).numpy()
        sim.reset()
        for i in range(s.shape[0]):
            sim.set_source_series(i, s[i])
        sim.set_pml_scale(sc)
        g = sim.adjoint(T, np.asarray(target, np.float32), want_scale=True)
        ctx.save_for_backward(torch.from_numpy(np.ascontiguousarray(g["grad_source"])).to(series.dtype),
                              torch.from_numpy(np.ascontiguousarray(g["grad_scale"][0])).to(scale6.dtype))
        return torch.tensor(float(g["loss"][0]), dtype=series.dtype)

    @staticmethod
    def backward(ctx, gout):
        gs, gz = ctx.saved_tensors
        return gout * gs, gout * gz, None, None, None
