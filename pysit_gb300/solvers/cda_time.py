"""Time-domain constant-density acoustic solvers, ``kernel_implementation='cuda'``.

Mirrors the reference solver classes ConstantDensityAcousticTimeScalar_{1,2,3}D_cpp
(pysit/solvers/constant_density_acoustic/time/scalar/
constant_density_acoustic_time_scalar_{1D.py:126-158,2D.py:154-190,3D.py:182-227}):
same ``supports`` keys, constructor arguments, ``dt``/``nsteps``/``ts()``
(constant_density_acoustic_time_base.py:30-70: ``dt = cfl_safety * min(deltas) / max|C|``,
``nsteps = ceil((tf - t0)/dt)``), model assignment with 'edge' padding
(solver_base.py:107-117), the 3-slot ``SolverData`` ring (scalar_base.py:11-51),
``time_step(solver_data, rhs_k, rhs_kp1)`` and ``compute_dWaveOp('time', solver_data)``.

``time_step`` runs the sm_103a step kernel (pysit_cda_step_{1,2,3}d).  It accepts
the reference's host (numpy) solver data, copying through the device, and the
device-resident solver data of ``DeviceSolverData()`` (torch tensors), which is
what the plain per-shot path of TemporalModeling uses.
"""
from __future__ import annotations

import math

import numpy as np

from .. import _native
from .model_parameter import ConstantDensityAcousticParameters

__all__ = ["ConstantDensityAcousticTimeScalar_1D_cuda", "ConstantDensityAcousticTimeScalar_2D_cuda",
           "ConstantDensityAcousticTimeScalar_3D_cuda", "build_sigma"]


def build_sigma(mesh, dim_param):
    """Full-grid sigma of one axis as a flat array (pysit/util/matrix_helpers.py:6-13)."""
    s = np.zeros(mesh.shape(include_bc=True))
    if dim_param.lbc.type == "pml":
        s += dim_param.lbc.eval_on_mesh()
    if dim_param.rbc.type == "pml":
        s += dim_param.rbc.eval_on_mesh()
    return s.reshape(-1)


def axis_sigma_map(mesh, axis):
    """1-D sigma map along ``axis`` (length = padded nodes on that axis): the mesh
    convention used by the imaging operand."""
    p = mesh.parameters[axis]
    n = p.n + p.lbc.n + p.rbc.n
    out = np.zeros(n)
    if p.lbc.type == "pml":
        out[:p.lbc.n] += p.lbc.sigma
    if p.rbc.type == "pml":
        out[n - p.rbc.n:] += p.rbc.sigma
    return out


class _HostWavefieldVector:
    """Stacked [u; aux...] column on the host (wavefield_vector.py:7-145)."""

    aux_names: list = []

    def __init__(self, mesh, dtype=np.double, data=None):
        self.mesh = mesh
        self.dof = mesh.dof(include_bc=True)
        self.n_aux = len(self.aux_names)
        self.n_fields = 1 + self.n_aux
        if data is None:
            self._data = np.zeros((self.dof * self.n_fields, 1), dtype=dtype)
        else:
            if data.size != self.n_fields * self.dof:
                raise ValueError("Size mismatch between mesh and proposed data.")
            self._data = data.reshape(-1, 1)
        self.dtype = self._data.dtype

    def _field(self, i):
        return self._data[i * self.dof:(i + 1) * self.dof]

    @property
    def data(self):
        return self._data

    @data.setter
    def data(self, v):
        self._data[:] = v

    @property
    def u(self):
        return self._field(0)

    @u.setter
    def u(self, v):
        self._field(0)[:] = v

    primary_wavefield = u

    def __getattr__(self, name):
        aux = type(self).aux_names
        if name in aux:
            return self._field(1 + aux.index(name))
        raise AttributeError(name)

    def __imul__(self, s):
        self._data *= s
        return self

    def __iadd__(self, other):
        self._data += other.data if isinstance(other, _HostWavefieldVector) else other
        return self

    def copy(self):
        return type(self)(self.mesh, data=self._data.copy())


class _DeviceWavefieldVector(_HostWavefieldVector):
    """Same stacked layout held in a torch CUDA tensor."""

    def __init__(self, mesh, dtype=np.double, data=None):
        torch = _native.require_cuda()
        self.mesh = mesh
        self.dof = mesh.dof(include_bc=True)
        self.n_aux = len(self.aux_names)
        self.n_fields = 1 + self.n_aux
        tdt = torch.float64 if np.dtype(dtype) == np.float64 else torch.float32
        self._data = torch.zeros((self.dof * self.n_fields, 1), dtype=tdt, device="cuda") if data is None \
            else data.reshape(-1, 1)
        self.dtype = dtype

    def __imul__(self, s):
        self._data.mul_(s)
        return self

    def zero_(self):
        self._data.zero_()

    def copy(self):
        return type(self)(self.mesh, dtype=self.dtype, data=self._data.clone())


class _SolverData:
    """Three wavefield vectors: us[0] = k+1, us[1] = k, us[2] = k-1."""

    def __init__(self, solver, vec_cls, **kwargs):
        self.solver = solver
        self.temporal_accuracy_order = 2
        self.us = [vec_cls(solver.mesh, dtype=solver.dtype) for _ in range(3)]

    def advance(self):
        self.us[-1] *= 0
        self.us.insert(0, self.us.pop(-1))

    kp1 = property(lambda s: s.us[0], lambda s, v: s.us.__setitem__(0, v))
    k = property(lambda s: s.us[1], lambda s, v: s.us.__setitem__(1, v))
    km1 = property(lambda s: s.us[2], lambda s, v: s.us.__setitem__(2, v))


class _CDATimeScalarCuda:
    """Common part of the 1D/2D/3D solvers."""

    _dim = None
    _aux_names: list = []
    supports = {
        "equation_physics": "constant-density-acoustic",
        "equation_dynamics": "time",
        "equation_formulation": "scalar",
        "temporal_integrator": "leap-frog",
        "temporal_accuracy_order": 2,
        "spatial_discretization": "finite-difference",
        "spatial_accuracy_order": [2, 4, 6, 8],
        "kernel_implementation": "cuda",
        "boundary_conditions": ["pml", "pml-sim", "dirichlet"],
        "precision": ["single", "double"],
    }
    ModelParameters = ConstantDensityAcousticParameters

    def __init__(self, mesh, spatial_accuracy_order=4, trange=(0.0, 1.0), cfl_safety=1 / 6,
                 precision="double", checkpoint_every=None, shots_per_launch=None, use_graph=True,
                 pml_psi="reference", autotune=False, gradient_schedule="checkpoint", **kwargs):
        if mesh.dim != self._dim:
            raise ValueError(f"{type(self).__name__} needs a {self._dim}D mesh")
        if spatial_accuracy_order not in (2, 4, 6, 8):
            raise ValueError("spatial_accuracy_order must be one of 2, 4, 6, 8")
        if precision not in ("single", "double"):
            raise ValueError("precision must be 'single' or 'double'")
        if pml_psi not in ("reference", "consistent"):
            raise ValueError("pml_psi must be 'reference' or 'consistent'")
        if gradient_schedule not in ("checkpoint", "store", "auto"):
            raise ValueError("gradient_schedule must be 'checkpoint', 'store' or 'auto'")
        for i in range(mesh.dim):
            for bc in (mesh.parameters[i].lbc, mesh.parameters[i].rbc):
                if bc.type == "pml" and getattr(bc.domain_bc, "compact", False):
                    raise NotImplementedError("Compact option is not available for time solvers")
        self.mesh = mesh
        self.domain = mesh.domain
        self.spatial_accuracy_order = spatial_accuracy_order
        self.precision = precision
        self.dtype = np.double if precision == "double" else np.single
        self.trange = trange
        self.t0, self.tf = trange
        self.cfl_safety = cfl_safety
        self.dt = 0.0
        self.nsteps = 0
        self.checkpoint_every = checkpoint_every
        self.shots_per_launch = shots_per_launch
        self.use_graph = use_graph
        # 3D batched path: 'reference' reproduces the reference's step, whose C^2 on
        # sigma_x sigma_y sigma_z psi (_3D.h:219) makes the PML unstable at realistic
        # amplitudes; 'consistent' drops that C^2 (the matrix operator's form)
        self.pml_psi = pml_psi
        # choose the 2D/3D task length along x by timing when a batched plan is first built
        self.autotune = autotune
        # batched gradients: 'checkpoint' (forward, recompute and adjoint sweeps over
        # checkpoints), 'store' (the forward sweep keeps dWaveOp of every imaged step in
        # HBM, no recompute), 'auto' (store when the shots of a launch fit in free device
        # memory, with as many shots per launch as fit, else checkpoint)
        self.gradient_schedule = gradient_schedule
        self._mp = None
        self._model_change_count = 0
        self._C_dev = None
        self._sig_dev = None
        self._plans = {}
        self.operator_components = {}
        self._build_sigma_components()

        class WavefieldVector(_HostWavefieldVector):
            aux_names = list(self._aux_names)

        class DeviceWavefieldVector(_DeviceWavefieldVector):
            aux_names = list(self._aux_names)

        self.WavefieldVector = WavefieldVector
        self.DeviceWavefieldVector = DeviceWavefieldVector

    # ---- sigma -------------------------------------------------------------
    def _build_sigma_components(self):
        m = self.mesh
        oc = self.operator_components
        axes = {1: ["z"], 2: ["x", "z"], 3: ["x", "y", "z"]}[m.dim]
        for a in axes:
            oc["s" + a] = build_sigma(m, m.parameters[a])
        if m.dim == 2:
            oc["sxPsz"] = oc["sx"] + oc["sz"]
            oc["sxsz"] = oc["sx"] * oc["sz"]
        if m.dim == 3:
            oc["sxPsyPsz"] = oc["sx"] + oc["sy"] + oc["sz"]
            oc["sxsyPsxszPsysz"] = oc["sx"] * oc["sy"] + oc["sx"] * oc["sz"] + oc["sy"] * oc["sz"]
            oc["sxsysz"] = oc["sx"] * oc["sy"] * oc["sz"]

    def _profiles(self, axis):
        """(left, right) profiles passed to the step kernel (time_step of the reference)."""
        p = self.mesh.parameters[axis]
        lp = p.lbc.sigma if p.lbc.type == "pml" else np.array([])
        rp = p.rbc.sigma if p.rbc.type == "pml" else np.array([])
        return np.ascontiguousarray(lp, dtype=float), np.ascontiguousarray(rp, dtype=float)

    # ---- time axis -----------------------------------------------------------
    def ts(self):
        return np.arange(self.nsteps) * self.dt

    def _process_mp_reset(self):
        C = self._mp.C
        max_C = max(abs(C.min()), C.max())
        self.dt = self.cfl_safety * min(self.mesh.deltas) / max_C
        self.nsteps = int(math.ceil((self.tf - self.t0) / self.dt))
        self._C_dev = None

    @property
    def model_parameters(self):
        return self._mp

    @model_parameters.setter
    def model_parameters(self, mp):
        if not isinstance(mp, self.ModelParameters):
            raise TypeError(f"{type(mp)} is not of type {self.ModelParameters}")
        if self._mp is None or np.linalg.norm(self._mp.without_padding().data - mp.data) != 0.0:
            self._mp = mp.with_padding(padding_mode="edge")
            self._process_mp_reset()
            self._model_change_count += 1

    def device_model(self):
        """Padded C on the device (FP64), uploaded once per model."""
        torch = _native.require_cuda()
        if self._C_dev is None:
            self._C_dev = torch.as_tensor(np.ascontiguousarray(self._mp.C.reshape(-1)), dtype=torch.float64,
                                          device="cuda")
        return self._C_dev

    def release_plans(self):
        """Drop this solver's cached batched plans.  Their device workspaces (with the kept
        dWaveOp schedule, most of the device memory) go back to the device; the next batched
        call builds a new plan."""
        self._plans.clear()
        import torch
        if torch.cuda.is_available() and torch.cuda.is_initialized():
            torch.cuda.empty_cache()

    # ---- solver data -----------------------------------------------------------
    def SolverData(self, *args, **kwargs):
        """Host (numpy) ring, the reference-compatible solver state."""
        return _SolverData(self, self.WavefieldVector)

    def DeviceSolverData(self, *args, **kwargs):
        """Device-resident ring (torch CUDA tensors)."""
        return _SolverData(self, self.DeviceWavefieldVector)

    # ---- one step ------------------------------------------------------------------
    def _device_sigmas(self):
        torch = _native.require_cuda()
        key = self.precision
        if self._sig_dev is None or self._sig_dev[0] != key:
            tdt = torch.float64 if self.dtype == np.double else torch.float32
            sig = []
            for ax in range(self.mesh.dim):
                lp, rp = self._profiles(ax)
                sig.append((torch.as_tensor(lp, dtype=tdt, device="cuda"), len(lp),
                            torch.as_tensor(rp, dtype=tdt, device="cuda"), len(rp)))
            maps = [torch.as_tensor(axis_sigma_map(self.mesh, ax), dtype=tdt, device="cuda")
                    for ax in range(self.mesh.dim)]
            self._sig_dev = (key, sig, maps)
        return self._sig_dev[1], self._sig_dev[2]

    def _field_ptrs(self, vec):
        """(u, aux...) device pointers of a device wavefield vector."""
        d = vec.data
        dof = vec.dof
        return [d[i * dof:(i + 1) * dof].data_ptr() for i in range(vec.n_fields)]

    def time_step(self, solver_data, rhs_k, rhs_kp1=None):
        """Advance solver_data.kp1 from (km1, k) and the padded source term rhs_k."""
        torch = _native.require_cuda()
        host = isinstance(solver_data.k.data, np.ndarray)
        tdt = torch.float64 if self.dtype == np.double else torch.float32
        if host:
            dev = [torch.as_tensor(np.ascontiguousarray(v.data.reshape(-1)), dtype=tdt, device="cuda")
                   for v in (solver_data.km1, solver_data.k)]
            out = torch.empty_like(dev[1])
            vkm1, vk = dev
        else:
            vkm1, vk, out = solver_data.km1.data, solver_data.k.data, solver_data.kp1.data
        if isinstance(rhs_k, np.ndarray):
            rhs = torch.as_tensor(np.ascontiguousarray(rhs_k.reshape(-1)), dtype=tdt, device="cuda")
        else:
            rhs = rhs_k.reshape(-1).to(dtype=tdt)
        C = self.device_model().to(tdt) if tdt != torch.float64 else self.device_model()
        dof = self.mesh.dof(include_bc=True)
        f = lambda t, i: t.reshape(-1)[i * dof:(i + 1) * dof].data_ptr()  # noqa: E731
        self._launch_step(f, vkm1, vk, out, C, rhs)
        if host:
            solver_data.kp1.data[:] = out.reshape(-1, 1).cpu().numpy()

    def compute_dWaveOp(self, regime, *args):
        if regime != "time":
            raise NotImplementedError("only the 'time' regime exists for this solver")
        return self._compute_dWaveOp_time(*args)

    def _compute_dWaveOp_time(self, solver_data):
        """(u+ - 2u + u-)/dt^2 + sigma terms (constant_density_acoustic_base.py:24-40), on the GPU."""
        torch = _native.require_cuda()
        lib = _native.load()
        host = isinstance(solver_data.k.data, np.ndarray)
        tdt = torch.float64 if self.dtype == np.double else torch.float32
        dof = self.mesh.dof(include_bc=True)

        def dev(v, i=0):
            d = v.data
            if host:
                return torch.as_tensor(np.ascontiguousarray(d[i * dof:(i + 1) * dof].reshape(-1)), dtype=tdt,
                                       device="cuda")
            return d[i * dof:(i + 1) * dof].reshape(-1)

        um, uc, up = dev(solver_data.km1), dev(solver_data.k), dev(solver_data.kp1)
        psi = None
        if self.mesh.dim == 3:
            psi = dev(solver_data.k, 1 + self._aux_names.index("psi"))
        _, maps = self._device_sigmas()
        out = torch.empty(dof, dtype=tdt, device="cuda")
        sh = self.mesh.shape(include_bc=True, as_grid=True)
        if self.mesh.dim == 1:
            nx, ny, nz = 1, 1, sh[0]
            sx, sy, sz = None, None, maps[0].data_ptr()
        elif self.mesh.dim == 2:
            nx, ny, nz = sh[0], 1, sh[1]
            sx, sy, sz = maps[0].data_ptr(), None, maps[1].data_ptr()
        else:
            nx, ny, nz = sh
            sx, sy, sz = maps[0].data_ptr(), maps[1].data_ptr(), maps[2].data_ptr()
        _native.check(lib.pysit_cda_dwaveop(_native.PYSIT_F64 if tdt == torch.float64 else _native.PYSIT_F32,
                                            self.mesh.dim, um.data_ptr(), uc.data_ptr(), up.data_ptr(),
                                            psi.data_ptr() if psi is not None else None, sx, sy, sz,
                                            nx, ny, nz, self.dt, out.data_ptr(), _native.stream_handle()))
        out = out.reshape(-1, 1)
        return out.cpu().numpy() if host else out

    def _launch_step(self, f, vkm1, vk, out, C, rhs):
        raise NotImplementedError


class ConstantDensityAcousticTimeScalar_1D_cuda(_CDATimeScalarCuda):
    _dim = 1
    _aux_names = ["Phiz"]
    supports = dict(_CDATimeScalarCuda.supports, spatial_dimension=1)

    def _launch_step(self, f, vkm1, vk, out, C, rhs):
        lib = _native.load()
        sig, _ = self._device_sigmas()
        zl, nzl, zr, nzr = sig[0]
        nz = self.mesh.dof(include_bc=True)
        dt = _native.PYSIT_F64 if self.dtype == np.double else _native.PYSIT_F32
        _native.check(lib.pysit_cda_step_1d(dt, self.spatial_accuracy_order, f(vkm1, 0), f(vk, 1), f(vk, 0),
                                            C.data_ptr(), rhs.data_ptr(), zl.data_ptr(), nzl, zr.data_ptr(), nzr,
                                            self.dt, self.mesh.z.delta, nz, f(out, 1), f(out, 0),
                                            _native.stream_handle()))


class ConstantDensityAcousticTimeScalar_2D_cuda(_CDATimeScalarCuda):
    _dim = 2
    _aux_names = ["Phix", "Phiz"]
    supports = dict(_CDATimeScalarCuda.supports, spatial_dimension=2)

    def _launch_step(self, f, vkm1, vk, out, C, rhs):
        lib = _native.load()
        sig, _ = self._device_sigmas()
        (xl, nxl, xr, nxr), (zl, nzl, zr, nzr) = sig
        nx, nz = self.mesh.shape(include_bc=True, as_grid=True)
        dt = _native.PYSIT_F64 if self.dtype == np.double else _native.PYSIT_F32
        _native.check(lib.pysit_cda_step_2d(dt, self.spatial_accuracy_order, f(vkm1, 0), f(vk, 1), f(vk, 2),
                                            f(vk, 0), C.data_ptr(), rhs.data_ptr(), xl.data_ptr(), nxl,
                                            xr.data_ptr(), nxr, zl.data_ptr(), nzl, zr.data_ptr(), nzr, self.dt,
                                            self.mesh.x.delta, self.mesh.z.delta, nx, nz, f(out, 1), f(out, 2),
                                            f(out, 0), _native.stream_handle()))


class ConstantDensityAcousticTimeScalar_3D_cuda(_CDATimeScalarCuda):
    _dim = 3
    _aux_names = ["psi", "Phix", "Phiy", "Phiz"]
    supports = dict(_CDATimeScalarCuda.supports, spatial_dimension=3)

    def _launch_step(self, f, vkm1, vk, out, C, rhs):
        lib = _native.load()
        sig, _ = self._device_sigmas()
        (xl, nxl, xr, nxr), (yl, nyl, yr, nyr), (zl, nzl, zr, nzr) = sig
        nx, ny, nz = self.mesh.shape(include_bc=True, as_grid=True)
        dt = _native.PYSIT_F64 if self.dtype == np.double else _native.PYSIT_F32
        # aux order in the stacked vector: psi, Phix, Phiy, Phiz (…_3D.py:69-71)
        _native.check(lib.pysit_cda_step_3d(dt, self.spatial_accuracy_order, f(vkm1, 0), f(vk, 2), f(vk, 3),
                                            f(vk, 4), f(vk, 1), f(vk, 0), C.data_ptr(), rhs.data_ptr(),
                                            xl.data_ptr(), nxl, xr.data_ptr(), nxr, yl.data_ptr(), nyl,
                                            yr.data_ptr(), nyr, zl.data_ptr(), nzl, zr.data_ptr(), nzr, self.dt,
                                            self.mesh.x.delta, self.mesh.y.delta, self.mesh.z.delta, nx, ny, nz,
                                            f(out, 2), f(out, 3), f(out, 4), f(out, 1), f(out, 0),
                                            _native.stream_handle()))
