"""Time-domain modelling tools (mirror of pysit.modeling.temporal_modeling).

``TemporalModeling(solver)`` keeps the reference signatures:
  forward_model(shot, m0, imaging_period=1, return_parameters=[])      (:60-169)
  migrate_shot(shot, m0, operand_simdata, imaging_period, ..., dWaveOp=None) (:171-214)
  adjoint_model(shot, m0, operand_simdata, imaging_period=1, operand_dWaveOpAdj=None,
                operand_model=None, return_parameters=[], dWaveOp=None, wavefield=None) (:228-387)
  linear_forward_model(shot, m0, m1, return_parameters=[], dWaveOp0=None)   (:389-546)

Two device paths implement them:
  * the batched plan (engine.WavePlan) when only traces or an image are asked
    for: forward_model(..., ['simdata']), linear_forward_model(..., ['simdata'])
    and migrate_shot without dWaveOp;
  * the plain per-step loop of the reference, every step on the GPU
    (solver.time_step on device-resident solver data, dWaveOp stored per step
    on the device), for 'wavefield' / 'dWaveOp' / 'adjointfield' outputs and for
    adjoint_model with a given dWaveOp.  This is also the "plain per-shot"
    baseline of the benchmarks.
"""
from __future__ import annotations

import numpy as np

from .. import _native
from ..engine import padded_cells, plan_for
from ..solvers.model_parameter import fold_padding

__all__ = ["TemporalModeling"]


class _DeviceOps:
    """Receiver sampling / injection operators of one shot on the device."""

    def __init__(self, solver, shot):
        torch = _native.require_cuda()
        mesh = solver.mesh
        tdt = torch.float64 if solver.dtype == np.double else torch.float32
        self.tdt = tdt
        self.dof = mesh.dof(include_bc=True)
        cells, pts, w = shot.sources.taps()
        self.s_cells = torch.as_tensor(padded_cells(mesh, cells), device="cuda")
        self.s_pts = torch.as_tensor(np.asarray(pts, np.int64), device="cuda")
        self.s_w = torch.as_tensor(w, dtype=tdt, device="cuda")
        ts = solver.ts()
        amps = shot.sources.amplitudes(np.concatenate([ts, [solver.nsteps * solver.dt]]))
        self.s_amp = torch.as_tensor(amps, dtype=tdt, device="cuda")
        rc, rr, rws, rwi = shot.receivers.taps()
        self.nrec = shot.receivers.receiver_count
        self.r_cells = torch.as_tensor(padded_cells(mesh, rc), device="cuda")
        self.r_recs = torch.as_tensor(np.asarray(rr, np.int64), device="cuda")
        self.r_ws = torch.as_tensor(rws, dtype=tdt, device="cuda")
        self.r_wi = torch.as_tensor(rwi, dtype=tdt, device="cuda")

    def source_rhs(self, k, out):
        """Padded rhs = S*(intensity w(k dt)) (sources.py:106-129 then pad_array)."""
        out.zero_()
        out.index_add_(0, self.s_cells, self.s_w * self.s_amp[k, self.s_pts])
        return out

    def sample(self, u, out_row):
        """Traces S u (receivers.py:462-510)."""
        out_row.zero_()
        out_row.index_add_(0, self.r_recs, self.r_ws * u.reshape(-1)[self.r_cells])

    def inject(self, values, out):
        """Padded rhs = S* values (receivers.py:512-564 then pad_array)."""
        out.zero_()
        out.index_add_(0, self.r_cells, self.r_wi * values[self.r_recs])
        return out


class TemporalModeling:
    """Forward, adjoint and migration operators of the time-domain solver."""

    solver_type = "time"
    modeling_type = "time"

    def __init__(self, solver, batched=True):
        if solver.supports["equation_dynamics"] != self.solver_type:
            raise TypeError(f"Argument 'solver' type {solver.supports['equation_dynamics']} does not match "
                            f"modeling solver type {self.solver_type}.")
        self.solver = solver
        self.batched = batched

    # ------------------------------------------------------------------------------
    def forward_model(self, shot, m0, imaging_period=1, return_parameters=[]):
        solver = self.solver
        solver.model_parameters = m0
        rp = set(return_parameters)
        if self.batched and rp <= {"simdata"}:
            retval = {}
            if "simdata" in rp:
                plan = plan_for(solver, [shot], imaging_period, forward_only=True)
                tr = plan.forward()
                retval["simdata"] = tr[0, :, :shot.receivers.receiver_count].to(dtype=__import__("torch").float64) \
                    .cpu().numpy()
                plan.check_status()
            return retval
        return self._forward_plain(shot, imaging_period, rp)

    def _forward_plain(self, shot, imaging_period, rp, device_outputs=False):
        torch = _native.require_cuda()
        solver = self.solver
        mesh = solver.mesh
        nsteps = solver.nsteps
        ops = _DeviceOps(solver, shot)
        sd = solver.DeviceSolverData()
        rhs = torch.zeros(ops.dof, dtype=ops.tdt, device="cuda")
        us, dwo = [], []
        simdata = torch.zeros((nsteps, ops.nrec), dtype=ops.tdt, device="cuda") if "simdata" in rp else None
        for k in range(nsteps):
            uk = sd.k.u
            if "wavefield" in rp:
                us.append(mesh.unpad_array(uk.reshape(-1, 1)).cpu().numpy().copy())
            if simdata is not None:
                ops.sample(uk, simdata[k])
            ops.source_rhs(k, rhs)
            solver.time_step(sd, rhs, None)
            if "dWaveOp" in rp and k % imaging_period == 0:
                dwo.append(solver.compute_dWaveOp("time", sd))
            if k == nsteps - 1:
                break
            sd.advance()
        retval = {}
        if "wavefield" in rp:
            retval["wavefield"] = us
        if "dWaveOp" in rp:
            retval["dWaveOp"] = dwo if device_outputs else [d.cpu().numpy() for d in dwo]
        if simdata is not None:
            retval["simdata"] = simdata if device_outputs else simdata.double().cpu().numpy()
        return retval

    # ------------------------------------------------------------------------------
    def linear_forward_model(self, shot, m0, m1, return_parameters=[], dWaveOp0=None):
        """Born modelling about m0: u1 driven by rhs_k = -m1_edge * dWaveOp0_k, traces of u1_k
        recorded before step k.  'simdata' alone (dWaveOp0 not given) runs the batched plan;
        'wavefield1', 'dWaveOp0', 'dWaveOp1' or a given dWaveOp0 run the reference's loop
        step by step on the device."""
        solver = self.solver
        solver.model_parameters = m0
        rp = set(return_parameters)
        if self.batched and rp <= {"simdata"} and dWaveOp0 is None:
            retval = {}
            if "simdata" in rp:
                plan = plan_for(solver, [shot])
                tr = plan.born(m1)
                retval["simdata"] = tr[0, :, :shot.receivers.receiver_count].to(
                    dtype=__import__("torch").float64).cpu().numpy()
                plan.check_status()
            return retval
        return self._linear_plain(shot, m1, rp, dWaveOp0)

    def _linear_plain(self, shot, m1, rp, dWaveOp0=None, device_outputs=False):
        torch = _native.require_cuda()
        solver = self.solver
        mesh = solver.mesh
        nsteps = solver.nsteps
        ops = _DeviceOps(solver, shot)
        dev = lambda a: a.reshape(-1) if isinstance(a, torch.Tensor) else torch.as_tensor(  # noqa: E731
            np.asarray(a).reshape(-1), dtype=ops.tdt, device="cuda")
        m1p = torch.as_tensor(np.asarray(m1.with_padding(padding_mode="edge").data).reshape(-1), dtype=ops.tdt,
                              device="cuda")
        sd = solver.DeviceSolverData()
        rhs = torch.zeros(ops.dof, dtype=ops.tdt, device="cuda")
        if dWaveOp0 is None:
            # background field one step ahead: dWaveOp0_k needs u0_{k+1}
            sd0 = solver.DeviceSolverData()
            rhs0 = torch.zeros(ops.dof, dtype=ops.tdt, device="cuda")
            solver.time_step(sd0, ops.source_rhs(0, rhs0), None)
            dw0_k = solver.compute_dWaveOp("time", sd0)
            sd0.advance()
        us, dw0s, dw1s = [], [], []
        simdata = torch.zeros((nsteps, ops.nrec), dtype=ops.tdt, device="cuda") if "simdata" in rp else None
        for k in range(nsteps):
            uk = sd.k.u
            if "wavefield1" in rp:
                us.append(mesh.unpad_array(uk.reshape(-1, 1)).cpu().numpy().copy())
            if simdata is not None:
                ops.sample(uk, simdata[k])
            if dWaveOp0 is None:
                solver.time_step(sd0, ops.source_rhs(k + 1, rhs0), None)
                dw0_kp1 = solver.compute_dWaveOp("time", sd0)
                sd0.advance()
            else:
                dw0_k = dev(dWaveOp0[k])
            if "dWaveOp0" in rp:
                dw0s.append(dw0_k)
            torch.mul(m1p, dw0_k.reshape(-1), out=rhs)
            rhs.neg_()
            solver.time_step(sd, rhs, None)
            if "dWaveOp1" in rp:
                dw1s.append(solver.compute_dWaveOp("time", sd))
            if k == nsteps - 1:
                break
            sd.advance()
            if dWaveOp0 is None:
                dw0_k = dw0_kp1
        host = (lambda L: L) if device_outputs else (lambda L: [d.cpu().numpy() for d in L])  # noqa: E731
        retval = {}
        if "wavefield1" in rp:
            retval["wavefield1"] = us
        if "dWaveOp0" in rp:
            retval["dWaveOp0"] = host(dw0s)
        if "dWaveOp1" in rp:
            retval["dWaveOp1"] = host(dw1s)
        if simdata is not None:
            retval["simdata"] = simdata if device_outputs else simdata.double().cpu().numpy()
        return retval

    # ------------------------------------------------------------------------------
    def migrate_shot(self, shot, m0, operand_simdata, imaging_period=1, operand_dWaveOpAdj=None,
                     operand_model=None, dWaveOp=None, adjointfield=None, dWaveOpAdj=None, wavefield=None):
        solver = self.solver
        solver.model_parameters = m0
        if (self.batched and dWaveOp is None and adjointfield is None and dWaveOpAdj is None
                and operand_dWaveOpAdj is None and operand_model is None):
            torch = _native.require_cuda()
            plan = plan_for(solver, [shot], imaging_period)
            op = np.zeros((1, solver.nsteps, plan.nrec))
            op[0, :, :shot.receivers.receiver_count] = np.asarray(operand_simdata)
            img = plan.migrate(torch.as_tensor(op, dtype=plan.tdtype, device="cuda"))
            out = m0.perturbation(data=img.cpu().numpy().reshape(-1, 1))
            plan.check_status()
            return out
        if dWaveOp is None:
            dWaveOp = self._forward_plain(shot, imaging_period, {"dWaveOp"}, device_outputs=True)["dWaveOp"]
        rp = ["imaging_condition"]
        if adjointfield is not None:
            rp.append("adjointfield")
        if dWaveOpAdj is not None:
            rp.append("dWaveOpAdj")
        rv = self.adjoint_model(shot, m0, operand_simdata, imaging_period, operand_dWaveOpAdj, operand_model,
                                return_parameters=rp, dWaveOp=dWaveOp, wavefield=wavefield)
        if adjointfield is not None:
            adjointfield[:] = rv["adjointfield"][:]
        if dWaveOpAdj is not None:
            dWaveOpAdj[:] = rv["dWaveOpAdj"][:]
        return rv["imaging_condition"]

    def adjoint_model(self, shot, m0, operand_simdata, imaging_period=1, operand_dWaveOpAdj=None,
                      operand_model=None, return_parameters=[], dWaveOp=None, wavefield=None):
        """Time-reversed adjoint with the forward operator, zero-lag imaging
        ic += q_k * dWaveOp[k // p] (temporal_modeling.py:312-371)."""
        torch = _native.require_cuda()
        solver = self.solver
        solver.model_parameters = m0
        mesh = solver.mesh
        nsteps = solver.nsteps
        dt = solver.dt
        rp = set(return_parameters)
        ops = _DeviceOps(solver, shot)
        if dWaveOp is not None:
            do_ic = True
        elif "imaging_condition" in rp:
            raise ValueError("To compute imaging condition, forward component must be specified.")
        else:
            do_ic = False
        dev = lambda a: a.reshape(-1) if isinstance(a, torch.Tensor) else torch.as_tensor(  # noqa: E731
            np.asarray(a).reshape(-1), dtype=ops.tdt, device="cuda")
        operand = torch.as_tensor(np.asarray(operand_simdata), dtype=ops.tdt, device="cuda") \
            if not isinstance(operand_simdata, torch.Tensor) else operand_simdata.to(ops.tdt)
        m1 = None
        if operand_model is not None:
            m1 = torch.as_tensor(operand_model.with_padding().data.reshape(-1), dtype=ops.tdt, device="cuda")
        sd = solver.DeviceSolverData()
        rhs = torch.zeros(ops.dof, dtype=ops.tdt, device="cuda")
        ic = torch.zeros(ops.dof, dtype=torch.float64, device="cuda") if do_ic else None
        vs, dwa = [], []
        for k in range(nsteps - 1, -1, -1):
            vk = sd.k.u.reshape(-1)
            if "adjointfield" in rp:
                vs.append(mesh.unpad_array(vk.reshape(-1, 1)).cpu().numpy().copy())
            if do_ic and k % imaging_period == 0:
                ic += (vk * dev(dWaveOp[k // imaging_period])).double()
            ops.inject(operand[k], rhs)
            if operand_dWaveOpAdj is not None and m1 is not None:
                rhs += m1 * dev(operand_dWaveOpAdj[k])
            solver.time_step(sd, rhs, None)
            if "dWaveOpAdj" in rp and k % imaging_period == 0:
                dwa.append(solver.compute_dWaveOp("time", sd).cpu().numpy())
            if k == 0:
                break
            sd.advance()
        retval = {}
        if do_ic:
            ic *= -1 * dt
            ic *= imaging_period
            retval["imaging_condition"] = m0.perturbation(data=fold_padding(mesh, ic.cpu().numpy()))
        if "adjointfield" in rp:
            vs.reverse()
            retval["adjointfield"] = vs
        if "dWaveOpAdj" in rp:
            dwa.reverse()
            retval["dWaveOpAdj"] = dwa
        return retval
