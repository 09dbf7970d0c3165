"""torch.autograd wrapper of the adjoint (hc_adj_gradient), for checking the
gradient with torch's machinery.

`OutletLossProblem` fixes a hydro-only catchment, a warm-up of `warm`
iterations, a window of `n` iterations and a target discharge series.  The
loss is the mean over the window's samples (the first iteration of every
simulated minute) of (Q - target)^2, Q being water_flux_out's outflow.  Its
parameters are the Manning's n of every cell and the elevation of every
cell, both as they are during the window (the warm-up runs on the case's own
fields), and the rain table (rows x zones, mm/h), which the run reads from
its start: only rows the window reads should be varied.

`OutletLoss.apply(manning, elev, rain, problem)` is a torch.autograd.Function:
its forward runs the adjoint on the device (libhc_gpu, through the C ABI)
and keeps the three gradients; its backward scales them.  Time steps, wet
mask and input points are those of the run at the given parameters, held
fixed (they are piecewise constant in them); `problem.loss(...)` evaluates
the loss with the time steps of a recorded run imposed, which is what a
central finite difference of this gradient has to use.
"""
import numpy as np
import torch

import hc


class OutletLossProblem:
    def __init__(self, case, warm, n, target, max_states=64):
        self.case = case
        self.warm = int(warm)
        self.n = int(n)
        self.target = np.ascontiguousarray(target, dtype=np.float64)
        self.max_states = int(max_states)
        self.record = None

    def _model(self, manning, elev, rain):
        import copy
        c = copy.copy(self.case)
        if rain is not None:
            c.rain = np.ascontiguousarray(rain, dtype=np.float32)
        m = hc.Model(c)
        m.run(self.warm, records=False)
        p = self.case.params
        if manning is not None:
            full = np.zeros((p.imax + 2, p.jmax + 2))
            full[1:-1, 1:-1] = manning
            m.upload("spat_var_mannings", full)
        if elev is not None:
            full = m.field("elev")
            full[1:-1, 1:-1] = elev
            m.upload("elev", full)
        return m

    def gradient(self, manning, elev, rain):
        """(loss, dL/dn, dL/delev (both imax x jmax), dL/drain, info); also
        records the run's time steps for `loss`."""
        m = self._model(manning, elev, rain)
        rec, _ = m.adj_forward(self.n)
        self.record = rec
        m.close()
        m = self._model(manning, elev, rain)
        loss, gn, gr, info, ge = m.adj_gradient(self.n, self.max_states, self.target, elev=True)
        m.close()
        return loss, gn[1:-1, 1:-1], ge[1:-1, 1:-1], gr, info

    def loss(self, manning=None, elev=None, rain=None, record=None):
        """The loss with the time steps of `record` (default: the run of the
        last `gradient` call) imposed."""
        rec = self.record if record is None else record
        m = self._model(manning, elev, rain)
        _, q = m.adj_forward(self.n, fixed=rec)
        m.close()
        k = min(len(q), len(self.target))
        return float(np.mean((q[:k] - self.target[:k]) ** 2))


class OutletLoss(torch.autograd.Function):
    """loss(manning, elev, rain) of an OutletLossProblem, differentiable in
    all three (float64 tensors: imax x jmax, imax x jmax, rain rows x
    zones)."""

    @staticmethod
    def forward(ctx, manning, elev, rain, problem):
        as_np = lambda t: t.detach().cpu().numpy().astype(np.float64)
        loss, gn, ge, gr, info = problem.gradient(as_np(manning), as_np(elev), as_np(rain))
        ctx.save_for_backward(torch.from_numpy(gn).to(manning.device),
                              torch.from_numpy(ge).to(elev.device),
                              torch.from_numpy(gr).to(rain.device))
        ctx.info = info
        return torch.tensor(loss, dtype=torch.float64, device=manning.device)

    @staticmethod
    def backward(ctx, grad_out):
        gn, ge, gr = ctx.saved_tensors
        return grad_out * gn, grad_out * ge, grad_out * gr, None
