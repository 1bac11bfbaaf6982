"""Least-squares time-domain objective (mirror of pysit.objective_functions.temporal_least_squares).

Semantics (pysit/objective_functions/temporal_least_squares.py):
  * residual r = interpolate(d_obs, solver.ts()) - d_sim            (:27-65)
  * evaluate = 0.5 * dt * sum_shots ||r||^2                          (:67-82)
  * compute_gradient = -sum_shots F*_s r_s (m = C**-2 space), with
    aux_info 'objective_value' = 0.5*dt*sum||r||^2 and 'residual_norm' =
    sqrt(dt*sum||r||^2)                                              (:141-198)
With ``batched=True`` (default) all shots go through one plan call (the FP64
misfit and the FP64 cross-shot gradient sum stay on the GPU); ``batched=False``
runs the reference's per-shot loop on the plain per-step device path, which
also provides the pseudo-Hessian diagonal (:121-139).
"""
from __future__ import annotations

import weakref

import numpy as np

from ..engine import plan_for
from ..modeling.temporal_modeling import TemporalModeling

__all__ = ["TemporalLeastSquares", "ObjectiveFunctionBase"]


class ObjectiveFunctionBase:
    def __init__(self, solver, parallel_wrap_shot=None):
        self.solver = solver
        self.modeling_tools = None
        self.parallel_wrap_shot = parallel_wrap_shot

    def use_parallel(self):
        return bool(getattr(self.parallel_wrap_shot, "use_parallel", False))

    def evaluate(self, *args, **kwargs):
        raise NotImplementedError("Must be implemented by subclass.")

    def compute_gradient(self, *args, **kwargs):
        raise NotImplementedError("Must be implemented by subclass.")

    def apply_hessian(self, *args, **kwargs):
        raise NotImplementedError("Must be implemented by subclass.")


class TemporalLeastSquares(ObjectiveFunctionBase):
    """How to compute the parts of the objective needed for optimisation."""

    def __init__(self, solver, parallel_wrap_shot=None, imaging_period=1, batched=True, **plan_kwargs):
        super().__init__(solver, parallel_wrap_shot)
        self.modeling_tools = TemporalModeling(solver, batched=batched)
        self.imaging_period = int(imaging_period)
        self.batched = batched
        self.plan_kwargs = plan_kwargs
        self._last_plan = None  # weak: a cached plan may hold most of the device memory

    @property
    def last_plan(self):
        """The plan of the last batched call while the plan cache still holds it, else None."""
        return self._last_plan() if self._last_plan is not None else None

    # ---- reference per-shot path ---------------------------------------------------
    def _residual(self, shot, m0, dWaveOp=None, wavefield=None):
        rp = ["simdata"]
        if dWaveOp is not None:
            rp.append("dWaveOp")
        if wavefield is not None:
            rp.append("wavefield")
        mt = self.modeling_tools
        if set(rp) <= {"simdata"}:
            retval = mt.forward_model(shot, m0, self.imaging_period, return_parameters=rp)
        else:
            self.solver.model_parameters = m0
            retval = mt._forward_plain(shot, self.imaging_period, set(rp), device_outputs=True)
            retval["simdata"] = retval["simdata"].double().cpu().numpy()
        resid = shot.receivers.interpolate_data(self.solver.ts()) - retval["simdata"]
        if dWaveOp is not None:
            dWaveOp[:] = retval["dWaveOp"][:]
        if wavefield is not None:
            wavefield[:] = retval["wavefield"][:]
        return resid

    def _gradient_helper(self, shot, m0, ignore_minus=False, ret_pseudo_hess_diag_comp=False, **kwargs):
        dWaveOp = []
        r = self._residual(shot, m0, dWaveOp=dWaveOp)
        g = self.modeling_tools.migrate_shot(shot, m0, r, self.imaging_period, dWaveOp=dWaveOp)
        if not ignore_minus:
            g = -1 * g
        if ret_pseudo_hess_diag_comp:
            return g, r, self._pseudo_hessian_diagonal_component_shot(dWaveOp)
        return g, r

    def _pseudo_hessian_diagonal_component_shot(self, dWaveOp):
        mesh = self.solver.mesh
        acc = None
        for d in dWaveOp:
            a = d.double().cpu().numpy() if hasattr(d, "cpu") else np.asarray(d)
            v = mesh.unpad_array(a.reshape(-1, 1))
            acc = v * v if acc is None else acc + v * v
        return acc * self.imaging_period

    # ---- public API ------------------------------------------------------------------
    def _plan(self, shots, m0):
        self.solver.model_parameters = m0
        plan = plan_for(self.solver, list(shots), self.imaging_period, **self.plan_kwargs)
        plan.load_observed()
        self._last_plan = weakref.ref(plan)
        return plan

    def evaluate(self, shots, m0, **kwargs):
        if self.batched:
            plan = self._plan(shots, m0)
            r_norm2 = float(plan.misfit().item())
            plan.check_status()
        else:
            r_norm2 = 0.0
            for shot in shots:
                r = self._residual(shot, m0)
                r_norm2 += np.linalg.norm(r) ** 2
        return 0.5 * r_norm2 * self.solver.dt

    def compute_gradient(self, shots, m0, aux_info={}, **kwargs):
        want_phd = ("pseudo_hess_diag" in aux_info) and aux_info["pseudo_hess_diag"][0]
        if self.batched and not want_phd:
            plan = self._plan(shots, m0)
            g, rn = plan.gradient()
            plan.check_status()
            grad = m0.perturbation(data=g.cpu().numpy().reshape(-1, 1))
            r_norm2 = float(rn.item())
            pseudo_h_diag = None
        else:
            grad = m0.perturbation()
            r_norm2 = 0.0
            pseudo_h_diag = np.zeros(m0.asarray().shape)
            for shot in shots:
                if want_phd:
                    g, r, h = self._gradient_helper(shot, m0, ignore_minus=True, ret_pseudo_hess_diag_comp=True)
                    pseudo_h_diag += h
                else:
                    g, r = self._gradient_helper(shot, m0, ignore_minus=True)
                grad -= g
                r_norm2 += np.linalg.norm(r) ** 2
        r_norm2 *= self.solver.dt
        if ("residual_norm" in aux_info) and aux_info["residual_norm"][0]:
            aux_info["residual_norm"] = (True, np.sqrt(r_norm2))
        if ("objective_value" in aux_info) and aux_info["objective_value"][0]:
            aux_info["objective_value"] = (True, 0.5 * r_norm2)
        if want_phd:
            aux_info["pseudo_hess_diag"] = (True, pseudo_h_diag * self.solver.dt)
        return grad

    def apply_hessian(self, shots, m0, m1, hessian_mode="approximate", levenberg_mu=0.0, *args, **kwargs):
        """Hessian application at m0 (temporal_least_squares.py:200-249).

        'approximate' (Gauss-Newton, sum_s F_s* F_s m1) and 'levenberg' (+ mu m1) run as one
        batched plan call over all shots when ``batched``; 'full' adds the second-order terms
        driven by the residual and runs the reference's per-shot loop on the plain device path.
        Every migration images at every step (imaging period 1, the period of the dWaveOp0
        lists; the reference's call of migrate_shot omits that positional argument).  `m1` is
        a model perturbation or a plain array of the unpadded grid."""
        modes = ["approximate", "full", "levenberg"]
        if hessian_mode not in modes:
            raise ValueError("Invalid Hessian mode.  Valid options for applying hessian are {0}".format(modes))
        if not hasattr(m1, "with_padding"):
            m1 = m0.perturbation(data=np.asarray(m1, dtype=float).reshape(-1, 1))
        mt = self.modeling_tools
        if self.batched and hessian_mode in ("approximate", "levenberg"):
            self.solver.model_parameters = m0
            plan = plan_for(self.solver, list(shots), 1, **self.plan_kwargs)
            self._last_plan = weakref.ref(plan)
            h, _ = plan.hessian(m1)
            plan.check_status()
            result = m0.perturbation(data=h.cpu().numpy().reshape(-1, 1))
        else:
            result = m0.perturbation()
            for shot in shots:
                if hessian_mode in ("approximate", "levenberg"):
                    self.solver.model_parameters = m0
                    dWaveOp0 = mt._forward_plain(shot, 1, {"dWaveOp"}, device_outputs=True)["dWaveOp"]
                    d1 = mt._linear_plain(shot, m1, {"simdata"}, dWaveOp0=dWaveOp0, device_outputs=True)["simdata"]
                    result += mt.migrate_shot(shot, m0, d1, 1, dWaveOp=dWaveOp0)
                else:
                    dWaveOp0 = []
                    r0 = self._residual(shot, m0, dWaveOp=dWaveOp0)
                    lin = mt._linear_plain(shot, m1, {"simdata", "dWaveOp1"}, dWaveOp0=dWaveOp0, device_outputs=True)
                    dWaveOpAdj1 = []
                    result += mt.migrate_shot(shot, m0, r0, 1, dWaveOp=lin["dWaveOp1"], dWaveOpAdj=dWaveOpAdj1)
                    result += mt.migrate_shot(shot, m0, lin["simdata"], 1, operand_dWaveOpAdj=dWaveOpAdj1,
                                              operand_model=m1, dWaveOp=dWaveOp0)
        if hessian_mode == "levenberg":
            result += levenberg_mu * m1
        return result
