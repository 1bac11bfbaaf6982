"""Drop-in registration into an installed PySIT.

``pysit_gb300.plugin.register()`` adds ConstantDensityAcousticTimeScalar_{1,2,3}D_cuda
to PySIT's own solver factory (the object
pysit.solvers.wave_factory.ConstantDensityAcousticWave, registered the way
wave_factory.py:49-61 registers the cpp solvers).  Afterwards an unchanged PySIT
script selects the GPU solver with

    ConstantDensityAcousticWave(mesh, spatial_accuracy_order=8, kernel_implementation='cuda', ...)

Each class subclasses the reference's ConstantDensityAcousticTimeScalar_{n}D,
with the reference's ``supports`` dictionaries extended by
``{'kernel_implementation': 'cuda', 'spatial_accuracy_order': [2, 4, 6, 8],
'precision': ['single', 'double']}`` (the pattern of _2D.py:154-159).
``time_step`` and ``compute_dWaveOp`` run the sm_103a kernels on the
reference's numpy solver data, so PySIT's own generate_seismic_data /
TemporalModeling / TemporalLeastSquares loops work unchanged.  ``patch_objective=True``
additionally routes TemporalLeastSquares.evaluate / compute_gradient of a cuda
solver through the batched checkpointed plan (one device call for all shots).
"""
from __future__ import annotations

import numpy as np

from .solvers import cda_time

__all__ = ["register", "ReferenceShotAdapter"]

_REGISTERED = {}


class _RefSources:
    """taps()/amplitudes() of a reference PointSource (adjoint_sampling_operator)."""

    def __init__(self, src, mesh):
        self.src = src
        self.mesh = mesh
        self.source_count = 1

    def taps(self):
        import scipy.sparse as spsp
        op = self.src.adjoint_sampling_operator
        op = spsp.csr_matrix(op) if not hasattr(op, "tocoo") else op
        coo = op.tocoo()
        return np.asarray(coo.row, np.int64), np.zeros(coo.nnz, np.int32), np.asarray(coo.data, float)

    def amplitudes(self, ts):
        return (self.src.intensity * np.asarray([self.src.w(t) for t in ts], float)).reshape(-1, 1)


class _RefReceivers:
    """taps()/interpolate_data() of a reference ReceiverSet."""

    def __init__(self, rec):
        self.rec = rec
        self.receiver_count = rec.receiver_count

    def taps(self):
        import scipy.sparse as spsp
        S = self.rec.sampling_operator
        S = spsp.csr_matrix(S) if not hasattr(S, "tocoo") else S
        A = self.rec.adjoint_sampling_operator
        A = spsp.csr_matrix(A) if not hasattr(A, "tocoo") else A
        s = S.tocoo()
        a = A.T.tocsr()
        winj = np.asarray(a[s.row, s.col]).reshape(-1)
        return np.asarray(s.col, np.int64), np.asarray(s.row, np.int32), np.asarray(s.data, float), winj

    def interpolate_data(self, ts):
        return self.rec.interpolate_data(ts)


class ReferenceShotAdapter:
    """Presents a reference Shot with the taps interface of the batched engine."""

    def __init__(self, shot, mesh):
        self.shot = shot
        self.sources = _RefSources(shot.sources, mesh)
        self.receivers = _RefReceivers(shot.receivers)


def _make_class(pysit, dim):
    from pysit.util.solvers import inherit_dict
    import importlib
    mod = importlib.import_module("pysit.solvers.constant_density_acoustic.time.scalar."
                                  f"constant_density_acoustic_time_scalar_{dim}D")
    base = getattr(mod, f"ConstantDensityAcousticTimeScalar_{dim}D")
    mine = {1: cda_time.ConstantDensityAcousticTimeScalar_1D_cuda,
            2: cda_time.ConstantDensityAcousticTimeScalar_2D_cuda,
            3: cda_time.ConstantDensityAcousticTimeScalar_3D_cuda}[dim]

    @inherit_dict("supports", "_local_support_spec")
    class Cuda(base):
        _local_support_spec = {"kernel_implementation": "cuda", "spatial_accuracy_order": [2, 4, 6, 8],
                               "precision": ["single", "double"]}

        def __init__(self, mesh, spatial_accuracy_order=4, checkpoint_every=None, shots_per_launch=None,
                     use_graph=True, **kwargs):
            base.__init__(self, mesh, spatial_accuracy_order=spatial_accuracy_order, **kwargs)
            self.checkpoint_every = checkpoint_every
            self.shots_per_launch = shots_per_launch
            self.use_graph = use_graph
            self._C_dev = None
            self._sig_dev = None
            self._plans = {}
            self._aux_names = list(mine._aux_names)

        def _process_mp_reset(self, *args, **kwargs):
            base._process_mp_reset(self, *args, **kwargs)
            self._C_dev = None

        # GPU implementations shared with the standalone solver classes
        _profiles = mine._profiles
        device_model = mine.device_model
        release_plans = mine.release_plans
        _device_sigmas = mine._device_sigmas
        time_step = mine.time_step
        _launch_step = mine._launch_step
        _compute_dWaveOp_time = mine._compute_dWaveOp_time

    Cuda.__name__ = Cuda.__qualname__ = f"ConstantDensityAcousticTimeScalar_{dim}D_cuda"
    return Cuda


def _patch_objective(pysit):
    from .engine import plan_for
    TLS = pysit.TemporalLeastSquares
    if getattr(TLS, "_pysit_gb300_patched", False):
        return
    orig_eval, orig_grad = TLS.evaluate, TLS.compute_gradient

    def _plan(self, shots, m0):
        self.solver.model_parameters = m0
        adapted = [ReferenceShotAdapter(s, self.solver.mesh) for s in shots]
        plan = plan_for(self.solver, adapted, self.imaging_period)
        plan.load_observed()
        return plan

    def evaluate(self, shots, m0, **kw):
        if type(self.solver).__name__.endswith("_cuda") and not self.parallel_wrap_shot.use_parallel:
            plan = _plan(self, shots, m0)
            rn = float(plan.misfit().item())
            plan.check_status()
            return 0.5 * rn * self.solver.dt
        return orig_eval(self, shots, m0, **kw)

    def compute_gradient(self, shots, m0, aux_info={}, **kw):
        phd = ("pseudo_hess_diag" in aux_info) and aux_info["pseudo_hess_diag"][0]
        if type(self.solver).__name__.endswith("_cuda") and not phd and not self.parallel_wrap_shot.use_parallel:
            plan = _plan(self, shots, m0)
            g, rn = plan.gradient()
            plan.check_status()
            grad = m0.perturbation(data=g.cpu().numpy().reshape(-1, 1))
            r_norm2 = float(rn.item()) * self.solver.dt
            if ("residual_norm" in aux_info) and aux_info["residual_norm"][0]:
                aux_info["residual_norm"] = (True, np.sqrt(r_norm2))
            if ("objective_value" in aux_info) and aux_info["objective_value"][0]:
                aux_info["objective_value"] = (True, 0.5 * r_norm2)
            return grad
        return orig_grad(self, shots, m0, aux_info, **kw)

    TLS.evaluate = evaluate
    TLS.compute_gradient = compute_gradient
    TLS._pysit_gb300_patched = True


def register(pysit=None, patch_objective=False):
    """Register the cuda solvers with PySIT's factory; returns the three classes."""
    if pysit is None:
        import pysit  # noqa: F811
    key = id(pysit)
    if key in _REGISTERED:
        classes = _REGISTERED[key]
    else:
        from pysit.solvers.wave_factory import ConstantDensityAcousticWave
        classes = tuple(_make_class(pysit, d) for d in (1, 2, 3))
        for c in classes:
            ConstantDensityAcousticWave.register(c)
        _REGISTERED[key] = classes
    if patch_objective:
        _patch_objective(pysit)
    return classes
