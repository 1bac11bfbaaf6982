"""torch.autograd entry: wave speed C -> least-squares misfit, gradient by the adjoint state.

``FWIMisfit(solver, shots, observed, ts_observed)`` is callable on a velocity
tensor ``C`` (unpadded grid, any device, requires_grad optional) and returns
the objective of TemporalLeastSquares.evaluate (0.5*dt*sum||r||^2,
pysit/objective_functions/temporal_least_squares.py:67-82).  Its backward
returns the partial derivatives dJ/dC_i = dJ/dm_i * dm_i/dC_i (m = C**-2,
model_parameter.py:80-92).  The reference's compute_gradient g is the gradient
for the cell-volume inner product of model space (mesh.inner_product; the
adjoint test of temporal_modeling.py:982-984 pairs it with prod(deltas)), so
dJ/dm_i = g_i * dV and dJ/dC_i = g_i * dV * (-2 C_i**-3), dV = prod(mesh.deltas).

Per call: C goes to the device, is edge-padded there (solver_base.py:111),
dt/nsteps follow from max|C| (constant_density_acoustic_time_base.py:54-70),
the observed data (on the host or the device) are copied to the device and
resampled there onto the solver's time axis (linear, zero fill), and one plan
call computes misfit and gradient of every shot (FP64 reductions on the GPU).
"""
from __future__ import annotations

import weakref

import math

import numpy as np

from . import _native
from .engine import plan_for

__all__ = ["FWIMisfit", "resample_linear"]


def resample_linear(data, ts_src, ts_new):
    """Device linear interpolation along axis 1 of [nshots, nt, nrec] with zero fill
    outside [ts_src[0], ts_src[-1]] (interp1d semantics of ReceiverBase.interpolate_data)."""
    torch = _native.require_cuda()
    ts_src = np.asarray(ts_src, dtype=float)
    ts_new = np.asarray(ts_new, dtype=float)
    n = len(ts_src)
    if n < 2:
        # no interval to interpolate on: a single sample is kept at its own time only, as in
        # core.acquisition.linear_interpolate
        out = data.new_zeros((data.shape[0], len(ts_new)) + tuple(data.shape[2:]))
        hit = np.nonzero(ts_new == ts_src[0])[0] if n == 1 else np.zeros(0, dtype=np.int64)
        if len(hit):
            idx_t = torch.as_tensor(hit, device=data.device)
            out.index_copy_(1, idx_t, data[:, :1].expand(-1, len(hit), *data.shape[2:]).contiguous())
        return out
    idx = np.clip(np.searchsorted(ts_src, ts_new, side="left"), 1, n - 1)
    lo = idx - 1
    frac = (ts_new - ts_src[lo]) / (ts_src[idx] - ts_src[lo])
    inside = (ts_new >= ts_src[0]) & (ts_new <= ts_src[-1])
    dev = data.device
    lo_t = torch.as_tensor(lo, device=dev)
    hi_t = torch.as_tensor(idx, device=dev)
    f = torch.as_tensor(frac, dtype=data.dtype, device=dev).view(1, -1, 1)
    m = torch.as_tensor(inside, dtype=data.dtype, device=dev).view(1, -1, 1)
    y0 = data.index_select(1, lo_t)
    y1 = data.index_select(1, hi_t)
    return ((y1 - y0) * f + y0) * m


def _edge_pad(C, mesh):
    """Edge padding of a grid tensor on its device (numpy.pad mode='edge')."""
    torch = _native.require_cuda()
    out = C
    for a in range(mesh.dim):
        lo, hi = mesh.parameters[a].lbc.n, mesh.parameters[a].rbc.n
        n = out.shape[a]
        idx = torch.clamp(torch.arange(-lo, n + hi, device=C.device), 0, n - 1)
        out = out.index_select(a, idx)
    return out


def _make_function():
    torch = _native.require_cuda()

    class MisfitFunction(torch.autograd.Function):
        @staticmethod
        def forward(ctx, C, obj):
            J, grad_m = obj._run(C, want_grad=C.requires_grad)
            if grad_m is not None:
                ctx.save_for_backward(C.detach(), grad_m)
                ctx.dV = float(np.prod(obj.solver.mesh.deltas))
            return J

        @staticmethod
        def backward(ctx, gJ):
            C, grad_m = ctx.saved_tensors
            Cd = C.to(device=grad_m.device, dtype=torch.float64)
            dC = grad_m * (-2.0 * ctx.dV) * Cd ** -3
            return (gJ.to(dC.device) * dC).to(dtype=C.dtype, device=C.device), None

    return MisfitFunction


class FWIMisfit:
    """Differentiable misfit of a shot batch for one solver configuration."""

    def __init__(self, solver, shots, observed, ts_observed, imaging_period=1, **plan_kw):
        self.solver = solver
        self.shots = list(shots)
        self.observed = observed  # [nshots, nt_obs, nrec] torch tensor (host pinned or device)
        self.ts_observed = np.asarray(ts_observed, dtype=float)
        shape = tuple(observed.shape)
        nrec = max(s.receivers.receiver_count for s in self.shots)
        if len(shape) != 3 or shape != (len(self.shots), len(self.ts_observed), nrec):
            raise ValueError(f"observed data of shape {shape} do not fit {len(self.shots)} shots, "
                             f"{len(self.ts_observed)} samples and {nrec} receivers (the most of any shot)")
        self.imaging_period = imaging_period
        self.plan_kw = plan_kw
        self._fn = None
        self._last_plan = None  # weak: a cached plan may hold most of the device memory

    @property
    def last_plan(self):
        """The plan of the last call while the plan cache still holds it, else None."""
        return self._last_plan() if self._last_plan is not None else None

    def _set_model(self, C_dev):
        torch = _native.require_cuda()
        s = self.solver
        mesh = s.mesh
        Cg = C_dev.reshape(mesh.shape(as_grid=True)).to(torch.float64)
        Cpad = _edge_pad(Cg, mesh).contiguous()
        maxc = float(Cg.abs().max().item())
        dt = s.cfl_safety * min(mesh.deltas) / maxc
        nsteps = int(math.ceil((s.tf - s.t0) / dt))
        changed = (s.dt != dt) or (s.nsteps != nsteps) or s._C_dev is None
        s.dt, s.nsteps = dt, nsteps
        s._C_dev = Cpad.reshape(-1)
        s._model_change_count += 1
        if s._mp is None or changed:
            s._mp = s.ModelParameters(mesh, inputs=Cpad.reshape(-1, 1).cpu().numpy(), padded=True)
        return dt, nsteps

    def _run(self, C, want_grad):
        torch = _native.require_cuda()
        C_dev = C.detach().to("cuda", non_blocking=True)
        dt, nsteps = self._set_model(C_dev)
        plan = plan_for(self.solver, self.shots, self.imaging_period, **self.plan_kw)
        self._last_plan = weakref.ref(plan)
        # observed traces to the device and onto the plan's time axis, a few shots at a time
        # (bounded temporaries beside a plan that may hold most of the device memory)
        ts = self.solver.ts()
        for i in range(0, plan.nshots, 16):
            obs = self.observed[i:i + 16].to("cuda", non_blocking=True).to(plan.tdtype)
            plan.dobs[i:i + 16].copy_(resample_linear(obs, self.ts_observed, ts))
        if want_grad:
            g, rn = plan.gradient()
            # flat, x-major like PySIT's model vectors: takes the caller's shape of C
            grad_m = g.reshape(C.shape).clone()
        else:
            rn = plan.misfit()
            grad_m = None
        plan.check_status()
        J = (0.5 * dt) * rn.reshape(())
        return J.to(C.dtype if C.dtype.is_floating_point else torch.float64), grad_m

    def __call__(self, C):
        if self._fn is None:
            self._fn = _make_function()
        return self._fn.apply(C, self)
