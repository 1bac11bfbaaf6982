"""Batched checkpointed pipeline over the C ABI (pysit_plan_*).

A ``WavePlan`` binds one solver configuration (grid, order, precision, dt,
nsteps) and one list of shots to a device workspace owned by torch.  It runs
the forward modelling of all shots (``forward``), their misfit (``misfit``) or
misfit plus gradient (``gradient``) with one library call each, the time loops
captured in CUDA graphs.  It replaces, for the batch, the per-shot loops of
TemporalModeling.forward_model / adjoint_model and TemporalLeastSquares
(pysit/modeling/temporal_modeling.py:60-387,
pysit/objective_functions/temporal_least_squares.py:27-198).
"""
from __future__ import annotations

import ast
import ctypes as C
import json
import math
import os
import weakref

import numpy as np

from . import _native
from .solvers.cda_time import axis_sigma_map

__all__ = ["WavePlan", "PlanGroup", "padded_cells", "default_checkpoint_every"]

_DESC_AXIS = {1: [2], 2: [0, 2], 3: [0, 1, 2]}  # mesh axis -> (x, y, z) slot of the descriptor

# tunings chosen by WavePlan.autotune (task length along x, 2D shell block shares per step
# mode, z extent of the interior tasks), per (dim, order, padded grid, dtype, psi form, shots per launch, schedule, forward
# only, lanes); later plans of the same configuration start from them.  With the environment
# variable PYSIT_CUDA_TUNE_CACHE naming a JSON file, the table is read from that file on first
# use and written back after every new tuning, so later processes on the machine start from it.
_TUNED = {}
_TUNE_FILES_READ = set()
TILE_CANDIDATES = {2: (8, 16, 32, 64), 3: (8, 16, 32, 64)}
# z extents of the interior tasks tried, as fractions of the kernels' full width (32 lanes x
# the 16-byte lane vector: 128 cells in FP32, 64 in FP64); 0 stands for the full width
TILE_Z_FRACTIONS = (1.0, 0.75, 0.5)


def tile_z_candidates(dtype_bytes):
    full = 32 * (16 // dtype_bytes)
    return [0] + [max(16, int(full * f) // 4 * 4) for f in TILE_Z_FRACTIONS[1:]]


def _tune_cache_file():
    return os.environ.get("PYSIT_CUDA_TUNE_CACHE") or None


def _read_tunings(path):
    """Tunings stored in `path` ({} for a missing or unreadable file; bad rows are skipped)."""
    try:
        with open(path) as f:
            rows = json.load(f)
    except (OSError, ValueError):
        return {}
    out = {}
    for row in rows if isinstance(rows, list) else []:
        try:
            key, tile, share = row[:3]
            tile_z = int(row[3]) if len(row) > 3 else 0
            out[ast.literal_eval(key)] = (int(tile), tuple(float(v) for v in share), tile_z)
        except (ValueError, SyntaxError, TypeError):
            continue
    return out


def _write_tunings(path, table):
    rows = [[repr(k), v[0], list(v[1]), v[2] if len(v) > 2 else 0] for k, v in table.items()]
    tmp = f"{path}.{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(rows, f)
    os.replace(tmp, path)  # readers see the old file or the new one, never a partial one


def _plain_key(key):
    """The tuning key with numpy scalars as Python numbers (so that its repr reads back)."""
    if isinstance(key, tuple):
        return tuple(_plain_key(v) for v in key)
    return key.item() if isinstance(key, np.generic) else key


def _tuning_get(key):
    key = _plain_key(key)
    path = _tune_cache_file()
    if path and path not in _TUNE_FILES_READ:
        _TUNE_FILES_READ.add(path)
        for k, v in _read_tunings(path).items():
            _TUNED.setdefault(k, v)
    return _TUNED.get(key)


def _tuning_put(key, value):
    key = _plain_key(key)
    _TUNED[key] = value
    path = _tune_cache_file()
    if path:
        _write_tunings(path, {**_read_tunings(path), **_TUNED})


def padded_cells(mesh, cells):
    """Map flat indices of the unpadded grid to flat indices of the padded grid."""
    cells = np.asarray(cells, dtype=np.int64)
    idx = np.unravel_index(cells, tuple(mesh.shape(include_bc=False, as_grid=True)))
    idx = [i + mesh.parameters[a].lbc.n for a, i in enumerate(idx)]
    return np.ravel_multi_index(idx, tuple(mesh.shape(include_bc=True, as_grid=True))).astype(np.int64)


def default_checkpoint_every(nsteps, dim):
    """Segment length minimising replay + checkpoint storage: sqrt(fields_per_checkpoint * nsteps)."""
    fields = {1: 3, 2: 4, 3: 6}[dim]
    return int(max(1, min(nsteps, round(math.sqrt(fields * nsteps)))))


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class WavePlan:
    """Device plan of one (solver configuration, shot list)."""

    def __init__(self, solver, shots, imaging_period=1, checkpoint_every=None, shots_per_launch=None,
                 use_graph=None, record_steps=None, gradient_schedule=None, forward_only=False, lanes=None,
                 wait_polls=0, wait_fault=False):
        """``record_steps``: optional record length of each shot in time steps (<= solver.nsteps);
        a shorter shot's residual is zero from its length on, so its misfit and gradient are those
        of a run of that length (the shots of one plan still step together).

        ``gradient_schedule`` ('checkpoint' | 'store' | 'auto', default the solver's): how a
        gradient recovers dWaveOp of the forward field - recomputed from checkpoints, or kept
        from the forward sweep in HBM (no recompute sweep; about ceil(nsteps / imaging_period)
        fields per shot of a launch).  'auto' keeps them when the launch fits in free device
        memory, taking as many shots per launch as fit unless shots_per_launch is fixed.
        ``forward_only`` plans model data only (no adjoint, imaging or checkpoint storage).
        ``lanes`` (default 1): the shots split into that many ranges whose launch sequences run
        side by side on their own streams, shots_per_launch being per lane.
        ``wait_polls`` (default 0, the library's limit): tries of a step kernel's wait for a
        bulk copy before it counts as expired (``check_status`` then raises).  ``wait_fault``
        (test aid): the 2D step kernels' tasks first wait on a barrier nothing arrives on, so
        that the wait runs out and the expiry path runs."""
        torch = _native.require_cuda()
        lib = _native.load()
        self.solver = solver
        self.shots = list(shots)
        mesh = solver.mesh
        self.mesh = mesh
        self.dim = mesh.dim
        self.nsteps = solver.nsteps
        self.dt = solver.dt
        self.imaging_period = int(imaging_period)
        self.nshots = len(self.shots)
        self.tdtype = torch.float64 if solver.dtype == np.double else torch.float32
        if checkpoint_every is None:
            checkpoint_every = solver.checkpoint_every or default_checkpoint_every(self.nsteps, self.dim)
        self.checkpoint_every = int(min(max(1, checkpoint_every), self.nsteps))
        fixed_launch = shots_per_launch is not None or bool(solver.shots_per_launch)
        if shots_per_launch is None:
            shots_per_launch = solver.shots_per_launch or self.nshots
        self.shots_per_launch = int(max(1, min(shots_per_launch, self.nshots)))
        self.forward_only = bool(forward_only)
        self.lanes = int(max(1, min(lanes or 1, self.nshots)))
        if gradient_schedule is None:
            gradient_schedule = getattr(solver, "gradient_schedule", "checkpoint")
        if gradient_schedule not in ("checkpoint", "store", "auto"):
            raise ValueError("gradient_schedule must be 'checkpoint', 'store' or 'auto'")
        if self.forward_only:
            gradient_schedule = "checkpoint"
        use_graph = solver.use_graph if use_graph is None else use_graph

        d = _native.PlanDesc()
        d.dim = self.dim
        d.order = solver.spatial_accuracy_order
        d.dtype = _native.PYSIT_F64 if solver.dtype == np.double else _native.PYSIT_F32
        full = mesh.shape(include_bc=True, as_grid=True)
        keep = []  # numpy buffers referenced by the descriptor during plan creation
        for slot in range(3):
            d.n[slot] = 1
            d.delta[slot] = 1.0
        for a, slot in enumerate(_DESC_AXIS[self.dim]):
            p = mesh.parameters[a]
            d.n[slot] = full[a]
            d.delta[slot] = p.delta
            d.pad_lo[slot] = p.lbc.n
            d.pad_hi[slot] = p.rbc.n
            lp, rp = solver._profiles(a)
            lp, rp = np.ascontiguousarray(lp), np.ascontiguousarray(rp)
            mp = np.ascontiguousarray(axis_sigma_map(mesh, a))
            keep += [lp, rp, mp]
            d.sig_l[slot] = _dptr(lp)
            d.nsig_l[slot] = len(lp)
            d.sig_r[slot] = _dptr(rp)
            d.nsig_r[slot] = len(rp)
            d.sigmap[slot] = _dptr(mp)
        d.dt = self.dt
        d.nsteps = self.nsteps
        d.imaging_period = self.imaging_period
        d.checkpoint_every = self.checkpoint_every
        d.shots_per_launch = self.shots_per_launch
        d.nshots = self.nshots
        d.use_graph = 1 if use_graph else 0
        d.psi_consistent = 1 if getattr(solver, "pml_psi", "reference") == "consistent" else 0
        d.wait_polls = int(wait_polls)
        d.wait_fault = 1 if wait_fault else 0
        self._tune_key = (self.dim, solver.spatial_accuracy_order, tuple(full), str(solver.dtype),
                          d.psi_consistent)
        self.record_steps = None
        if record_steps is not None:
            rs = np.ascontiguousarray(np.asarray(record_steps, dtype=np.int32).reshape(-1))
            if rs.size != self.nshots:
                raise ValueError("record_steps needs one entry per shot")
            keep.append(rs)
            d.shot_nsteps = rs.ctypes.data_as(C.POINTER(C.c_int32))
            self.record_steps = rs.copy()

        ts = np.arange(self.nsteps) * self.dt
        # sources
        s_ptr, s_cell, s_pt, s_w, amps = [0], [], [], [], []
        nsrc = max(getattr(s.sources, "source_count", 1) for s in self.shots)
        for s in self.shots:
            cells, pts, w = s.sources.taps()
            s_cell.append(padded_cells(mesh, cells)); s_pt.append(np.asarray(pts, np.int32))
            s_w.append(np.asarray(w, float)); s_ptr.append(s_ptr[-1] + len(cells))
            a = np.zeros((self.nsteps, nsrc))
            aa = s.sources.amplitudes(ts)
            a[:, :aa.shape[1]] = aa
            amps.append(a)
        # receivers
        r_ptr, r_cell, r_pt, r_ws, r_wi = [0], [], [], [], []
        self.nrec_shot = [s.receivers.receiver_count for s in self.shots]
        nrec = max(self.nrec_shot)
        for s in self.shots:
            cells, recs, ws, wi = s.receivers.taps()
            r_cell.append(padded_cells(mesh, cells)); r_pt.append(np.asarray(recs, np.int32))
            r_ws.append(np.asarray(ws, float)); r_wi.append(np.asarray(wi, float))
            r_ptr.append(r_ptr[-1] + len(cells))
        self.nrec = nrec
        self.nsrc = nsrc
        arrs = dict(
            src_tap_ptr=np.asarray(s_ptr, np.int64), src_tap_cell=np.concatenate(s_cell),
            src_tap_point=np.concatenate(s_pt), src_tap_w=np.concatenate(s_w),
            src_amp=np.ascontiguousarray(np.stack(amps)),
            rec_tap_ptr=np.asarray(r_ptr, np.int64), rec_tap_cell=np.concatenate(r_cell),
            rec_tap_point=np.concatenate(r_pt), rec_tap_wsample=np.concatenate(r_ws),
            rec_tap_winject=np.concatenate(r_wi))
        ctype = {np.int64: C.c_int64, np.int32: C.c_int32, np.float64: C.c_double}
        for k, v in arrs.items():
            v = np.ascontiguousarray(v)
            keep.append(v)
            setattr(d, k, v.ctypes.data_as(C.POINTER(ctype[v.dtype.type])))
        d.nsrc = nsrc
        d.nrec = nrec
        d.forward_only = 1 if self.forward_only else 0
        d.lanes = self.lanes
        if gradient_schedule == "auto":
            gradient_schedule = self._choose_schedule(lib, d, fixed_launch, nrec)
        d.lanes = self.lanes
        d.store_dwaveop = 1 if gradient_schedule == "store" else 0
        d.shots_per_launch = self.shots_per_launch
        self.gradient_schedule = gradient_schedule
        # the tuning key knows the launch size and schedule only now
        self._tune_key = self._tune_key + (self.shots_per_launch, gradient_schedule, self.forward_only, self.lanes)
        tuned = _tuning_get(self._tune_key)
        d.tile_x = tuned[0] if tuned else 0
        for k in range(3):
            d.shell_share[k] = tuned[1][k] if tuned else 0.0
        d.tile_z = tuned[2] if tuned and len(tuned) > 2 else 0
        self.tile_x = d.tile_x
        self.tile_z = d.tile_z

        h = C.c_void_p()
        _native.check(lib.pysit_plan_create(C.byref(d), C.byref(h)))
        self._h = h
        nbytes = C.c_uint64()
        _native.check(lib.pysit_plan_workspace_bytes(h, C.byref(nbytes)))
        self.workspace_bytes = int(nbytes.value)
        self.workspace = torch.empty(self.workspace_bytes + 256, dtype=torch.uint8, device="cuda")
        base = self.workspace.data_ptr()
        self._ws_ptr = (base + 255) // 256 * 256
        _native.check(lib.pysit_plan_bind_workspace(h, C.c_void_p(self._ws_ptr), C.c_uint64(self.workspace_bytes),
                                                    C.c_void_p(_native.stream_handle())))
        self._model_version = None
        # reusable outputs (stable pointers keep the captured graphs valid)
        self.traces = torch.zeros((self.nshots, self.nsteps, nrec), dtype=self.tdtype, device="cuda")
        self.dobs = torch.zeros_like(self.traces)
        dof_phys = mesh.dof(include_bc=False)
        self.grad = torch.zeros(dof_phys, dtype=torch.float64, device="cuda")
        self.rnorm2 = torch.zeros(1, dtype=torch.float64, device="cuda")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _native.load().pysit_plan_destroy(h)
            except Exception:
                pass
            self._h = None

    @staticmethod
    def _workspace_for(lib, d, shots_per_launch, store, lanes=1):
        d.shots_per_launch = int(shots_per_launch)
        d.store_dwaveop = 1 if store else 0
        d.lanes = int(lanes)
        h = C.c_void_p()
        _native.check(lib.pysit_plan_create(C.byref(d), C.byref(h)))
        n = C.c_uint64()
        try:
            _native.check(lib.pysit_plan_workspace_bytes(h, C.byref(n)))
        finally:
            lib.pysit_plan_destroy(h)
        return int(n.value)

    def _choose_schedule(self, lib, d, fixed_launch, nrec):
        """'store' with the largest balanced launch that fits in free device memory (at least
        8 shots or all of them), else 'checkpoint' with the largest balanced launch that fits."""
        torch = _native.require_cuda()
        free = torch.cuda.mem_get_info()[0]
        elem = 8 if self.tdtype == torch.float64 else 4
        outputs = 3 * self.nshots * self.nsteps * nrec * elem  # traces, observed data, recorded traces
        budget = free - outputs - max(2 << 30, int(0.03 * free))
        G = self.shots_per_launch
        if fixed_launch:
            return "store" if self._workspace_for(lib, d, G, True, self.lanes) <= budget else "checkpoint"
        lanes = self.lanes  # lanes are not split further: two half-size lanes measured slower in 2D
        per_lane = -(-self.nshots // lanes)           # shots of the largest lane

        def fit(store):
            """Largest balanced launch of this schedule within the budget (0: none fits)."""
            b1 = self._workspace_for(lib, d, 1, store)
            per = self._workspace_for(lib, d, 2, store) - b1
            gmax = self.nshots if per <= 0 else int((budget - (b1 - per)) // per)
            gmax = min(gmax, self.nshots)
            if gmax < 1:
                return 0
            glane = max(1, min(gmax // lanes, per_lane))
            g = -(-per_lane // -(-per_lane // glane))
            while g > 1 and self._workspace_for(lib, d, g, store, lanes) > budget:
                g -= 1
            return g

        g = fit(True)
        if g >= min(8, self.nshots):
            self.shots_per_launch = g
            return "store"
        # checkpointed: the largest launch that fits (one shot at least; the plan reports a
        # workspace the device lacks when even that does not fit)
        self.shots_per_launch = max(1, fit(False))
        return "checkpoint"

    # ---------------------------------------------------------------------------
    def set_model(self):
        """Upload the solver's current padded model (once per model change)."""
        ver = (self.solver._model_change_count, id(self.solver._mp))
        if ver != self._model_version:
            C_dev = self.solver.device_model()
            _native.check(_native.load().pysit_plan_set_model(self._h, C.c_void_p(C_dev.data_ptr()),
                                                              C.c_void_p(_native.stream_handle())))
            self._model_version = ver

    def launches(self):
        n = C.c_int64()
        _native.check(_native.load().pysit_plan_last_launch_count(self._h, C.byref(n)))
        return int(n.value)

    def forward(self):
        """Simulated traces of all shots, [nshots, nsteps, nrec] (device)."""
        self.set_model()
        _native.check(_native.load().pysit_plan_forward(self._h, C.c_void_p(self.traces.data_ptr()),
                                                        C.c_void_p(_native.stream_handle())))
        return self.traces

    def load_observed(self, dobs=None):
        """Copy observed data (resampled to this plan's time axis) into the device buffer.

        ``dobs`` is a [nshots, nsteps, nrec] array/tensor; by default the shots'
        recorded data are interpolated onto ``solver.ts()`` (ReceiverSet.interpolate_data)."""
        torch = _native.require_cuda()
        if dobs is None:
            ts = self.solver.ts()
            dev = _observed_on_device(self.shots, self.tdtype, self.nrec)
            if dev is not None:  # resampled on the device from a cached upload of the recorded traces
                raw, ts_obs = dev
                step = 16
                for i in range(0, self.nshots, step):
                    self.dobs[i:i + step].copy_(_resample(raw[i:i + step], ts_obs, ts))
                return self.dobs
            host = np.zeros((self.nshots, self.nsteps, self.nrec))
            for i, s in enumerate(self.shots):
                host[i, :, :self.nrec_shot[i]] = s.receivers.interpolate_data(ts)
            dobs = host
        if isinstance(dobs, np.ndarray):
            src = torch.from_numpy(np.ascontiguousarray(dobs, dtype=np.float64 if self.tdtype == torch.float64
                                                        else np.float32))
            self.dobs.copy_(src.pin_memory() if src.numel() > (1 << 20) else src, non_blocking=True)
        else:
            self.dobs.copy_(dobs)
        return self.dobs

    def gradient(self, with_traces=False):
        """Run misfit + gradient on the loaded observed data.

        Returns (grad [dof_phys] FP64 device, rnorm2 [1] FP64 device); grad is with
        respect to m = C**-2 with the PML strips folded (compute_gradient semantics)."""
        self.set_model()
        _native.check(_native.load().pysit_plan_gradient(
            self._h, C.c_void_p(self.dobs.data_ptr()), C.c_void_p(self.grad.data_ptr()),
            C.c_void_p(self.rnorm2.data_ptr()), C.c_void_p(self.traces.data_ptr() if with_traces else None),
            C.c_void_p(_native.stream_handle())))
        return self.grad, self.rnorm2

    def migrate(self, operand):
        """F* of a data-space operand [nshots, nsteps, nrec] summed over shots (unpadded, FP64)."""
        self.set_model()
        self.dobs.copy_(operand)
        _native.check(_native.load().pysit_plan_migrate(
            self._h, C.c_void_p(self.dobs.data_ptr()), C.c_void_p(self.grad.data_ptr()),
            C.c_void_p(self.rnorm2.data_ptr()), C.c_void_p(_native.stream_handle())))
        return self.grad

    def _perturbation(self, m1):
        """Copy a model perturbation (unpadded, m-space) into the plan's FP64 device buffer."""
        torch = _native.require_cuda()
        if not hasattr(self, "m1"):
            self.m1 = torch.zeros(self.mesh.dof(include_bc=False), dtype=torch.float64, device="cuda")
            self.hess = torch.zeros_like(self.m1)
        data = m1.data if hasattr(m1, "with_padding") else m1  # a model perturbation or an array
        if isinstance(data, torch.Tensor):
            self.m1.copy_(data.reshape(-1).to(torch.float64))
        else:
            self.m1.copy_(torch.from_numpy(np.ascontiguousarray(np.asarray(data, dtype=np.float64).reshape(-1))))
        return self.m1

    def born(self, m1):
        """Linearised traces F m1 of all shots [nshots, nsteps, nrec] (device): the u1 field of
        TemporalModeling.linear_forward_model driven by -m1 dWaveOp0 (m1 edge-padded)."""
        self.set_model()
        m = self._perturbation(m1)
        _native.check(_native.load().pysit_plan_born(self._h, C.c_void_p(m.data_ptr()),
                                                     C.c_void_p(self.traces.data_ptr()),
                                                     C.c_void_p(_native.stream_handle())))
        return self.traces

    def hessian(self, m1):
        """Gauss-Newton Hessian application sum_s F_s* F_s m1 (FP64 device, unpadded, m-space),
        apply_hessian 'approximate'; returns (H m1, ||F m1||^2)."""
        self.set_model()
        m = self._perturbation(m1)
        _native.check(_native.load().pysit_plan_hessian(self._h, C.c_void_p(m.data_ptr()),
                                                        C.c_void_p(self.hess.data_ptr()),
                                                        C.c_void_p(self.rnorm2.data_ptr()),
                                                        C.c_void_p(_native.stream_handle())))
        return self.hess, self.rnorm2

    def autotune(self, candidates=None, nsteps=48, z_candidates=None):
        """Time every pair of a task length along x in `candidates` and a z extent of the
        interior tasks in `z_candidates` (0: the full width; forward + adjoint steps on this
        plan's buffers), keep the fastest for this plan and for later plans of the same
        configuration.  Returns {"chosen": rows, "chosen_z": cells, "ms": {(x, z): milliseconds}}.
        1D plans have no tiles."""
        if self.dim == 1:
            return {"chosen": 0, "chosen_z": 0, "ms": {}}
        torch = _native.require_cuda()
        cand = list(candidates or TILE_CANDIDATES[self.dim])
        zc = list(z_candidates if z_candidates is not None
                  else tile_z_candidates(8 if self.tdtype == torch.float64 else 4))
        self.set_model()
        ax = (C.c_int * len(cand))(*cand)
        az = (C.c_int * len(zc))(*zc)
        ms = (C.c_double * (len(cand) * len(zc)))()
        cx, cz = C.c_int(), C.c_int()
        _native.check(_native.load().pysit_plan_autotune_tiles(
            self._h, ax, len(cand), az, len(zc), int(nsteps), C.byref(cx), C.byref(cz), ms,
            C.c_void_p(_native.stream_handle())))
        self.tile_x, self.tile_z = int(cx.value), int(cz.value)
        tile, share = C.c_int(), (C.c_double * 3)()
        _native.check(_native.load().pysit_plan_get_tuning(self._h, C.byref(tile), share))
        self.shell_share = [float(v) for v in share]
        _tuning_put(self._tune_key, (self.tile_x, tuple(self.shell_share), self.tile_z))
        times = {(x, z): ms[i * len(zc) + j] for i, x in enumerate(cand) for j, z in enumerate(zc)}
        return {"chosen": self.tile_x, "chosen_z": self.tile_z, "ms": times, "shell_share": self.shell_share}

    def step_loop(self, mode, nsteps):
        """Enqueue `nsteps` launches of one step kernel (0 forward, 1 recompute, 2 adjoint) on the
        plan's own buffers, for timing one kernel; returns nothing useful (benchmarking aid)."""
        _native.check(_native.load().pysit_plan_step_loop(self._h, int(mode), int(nsteps),
                                                           C.c_void_p(_native.stream_handle())))

    def status(self):
        """Device status flags (1: bulk-copy wait expired, 2: non-finite wavefield); clears them."""
        f = C.c_int()
        _native.check(_native.load().pysit_plan_status(self._h, C.byref(f), C.c_void_p(_native.stream_handle())))
        return int(f.value)

    def check_status(self):
        """Read and clear the status flags of the runs since the last read.  An expired
        bulk-copy wait (flag 1) makes those runs' results invalid: PysitCudaError with
        PYSIT_ETIMEOUT.  A non-finite wavefield (flag 2: the time step is unstable) is left to
        the caller, as the reference leaves it: the flags are returned."""
        f = self.status()
        if f & 1:
            raise _native.PysitCudaError(
                _native.PYSIT_ETIMEOUT, "a step kernel's wait for a bulk copy expired: the results of the "
                "plan's last runs are invalid")
        return f

    def misfit(self, with_traces=False):
        self.set_model()
        _native.check(_native.load().pysit_plan_misfit(
            self._h, C.c_void_p(self.dobs.data_ptr()), C.c_void_p(self.rnorm2.data_ptr()),
            C.c_void_p(self.traces.data_ptr() if with_traces else None), C.c_void_p(_native.stream_handle())))
        return self.rnorm2


class PlanGroup:
    """Plans (e.g. of different grids) whose gradients run concurrently in one CUDA graph:
    each plan on a stream of its own, forked from the current stream and joined back."""

    def __init__(self, plans):
        self.plans = list(plans)
        arr = (C.c_void_p * len(self.plans))(*[p._h.value for p in self.plans])
        h = C.c_void_p()
        _native.check(_native.load().pysit_group_create(arr, len(self.plans), C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _native.load().pysit_group_destroy(h)
            except Exception:
                pass
            self._h = None

    def gradient(self):
        """Misfit and gradient of every plan on its loaded observed data: [(grad, rnorm2), ...]."""
        for p in self.plans:
            p.set_model()
        n = len(self.plans)
        dobs = (C.c_void_p * n)(*[p.dobs.data_ptr() for p in self.plans])
        grad = (C.c_void_p * n)(*[p.grad.data_ptr() for p in self.plans])
        rn = (C.c_void_p * n)(*[p.rnorm2.data_ptr() for p in self.plans])
        _native.check(_native.load().pysit_group_gradient(self._h, dobs, grad, rn,
                                                          C.c_void_p(_native.stream_handle())))
        return [(p.grad, p.rnorm2) for p in self.plans]


class _ObservedCache:
    """The recorded traces of the last shot list on the device: one entry, keyed by the
    receivers' data arrays, the dtype and nrec.  The entry is reused while every shot still
    holds the same array with the same fingerprint (a sample of its values): assign a new
    array to receivers.data, or pass the data to load_observed, after editing recorded traces
    in place.  The arrays are held weakly: when one of them is freed, the device copy goes
    with it."""

    def __init__(self):
        self._entry = None  # (key, value, [weakref of array], [fingerprint])

    def get(self, key, arrays):
        e = self._entry
        if e is None or e[0] != key:
            return None
        if all(w() is a and fp == _fingerprint(a) for w, fp, a in zip(e[2], e[3], arrays)):
            return e[1]
        return None

    def put(self, key, value, arrays):
        self.clear()
        try:
            refs = [weakref.ref(a) for a in arrays]
        except TypeError:  # data that cannot be held weakly is not cached
            return
        for a in {id(a): a for a in arrays}.values():
            weakref.finalize(a, self._drop, refs)
        self._entry = (key, value, refs, [_fingerprint(a) for a in arrays])

    def _drop(self, refs):
        if self._entry is not None and self._entry[2] is refs:
            self._entry = None

    def clear(self):
        self._entry = None


_OBSERVED = _ObservedCache()


def _fingerprint(a):
    a = np.asarray(a)
    flat = a.reshape(-1)
    return (a.shape, float(np.sum(flat[::4099], dtype=np.float64)), float(np.sum(a[:1], dtype=np.float64)),
            float(np.sum(a[-1:], dtype=np.float64)))


def _resample(data, ts_src, ts_new):
    from .autograd import resample_linear
    return resample_linear(data, ts_src, ts_new)


def _observed_on_device(shots, tdtype, nrec):
    """The shots' recorded traces as one device tensor (uploaded once per data arrays), or None
    when the shots have different time axes or the device lacks room for it."""
    torch = _native.require_cuda()
    recv = [s.receivers for s in shots]
    ts0 = getattr(recv[0], "ts", None)
    if ts0 is None or any(getattr(r, "data", None) is None for r in recv):
        return None
    if any(r.ts is not ts0 and not np.array_equal(r.ts, ts0) for r in recv[1:]):
        return None
    key = (tuple(id(r.data) for r in recv), str(tdtype), nrec, len(ts0))
    arrays = [r.data for r in recv]
    hit = _OBSERVED.get(key, arrays)
    if hit is not None:
        return hit
    _OBSERVED.clear()
    elem = 8 if tdtype == torch.float64 else 4
    need = len(recv) * len(ts0) * nrec * elem
    if torch.cuda.mem_get_info()[0] < need + (4 << 30):
        return None
    host = np.zeros((len(recv), len(ts0), nrec), dtype=np.float64 if elem == 8 else np.float32)
    for i, r in enumerate(recv):
        host[i, :, :r.data.shape[1]] = r.data
    raw = torch.from_numpy(host).pin_memory().to("cuda", non_blocking=True)
    ts_obs = np.asarray(ts0, dtype=float).copy()
    _OBSERVED.put(key, (raw, ts_obs), arrays)
    return raw, ts_obs


def plan_for(solver, shots, imaging_period=1, **kw):
    """Cached WavePlan of a solver for a shot list (rebuilt when dt/nsteps change)."""
    # a source-encoded supershot carries an encoding counter: a new encoding needs a new plan
    key = (tuple((id(s), getattr(s, "encoding", 0)) for s in shots), solver.dt, solver.nsteps, solver.precision,
           solver.spatial_accuracy_order, getattr(solver, "pml_psi", "reference"),
           getattr(solver, "gradient_schedule", "checkpoint"), int(imaging_period), tuple(sorted(kw.items())))
    cache = solver._plans
    p = cache.get(key)
    if p is None:
        # keep at most a few plans alive (each owns a workspace)
        while len(cache) >= 2:
            cache.pop(next(iter(cache)))
        if getattr(solver, "gradient_schedule", "checkpoint") != "checkpoint":
            # a plan that keeps dWaveOp sizes itself to the free memory: release the others first
            cache.clear()
            _native.require_cuda().cuda.empty_cache()
        p = WavePlan(solver, shots, imaging_period=imaging_period, **kw)
        if getattr(solver, "autotune", False) and _tuning_get(p._tune_key) is None:
            p.autotune()
        cache[key] = p
    return p
