"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public dataset is involved: each model is generated from a named seed.
  cfg2  2D batched FWI gradient: 1152 x 384 cells at 12.5 m + 40-cell PML, order 8,
        layered model 1500 -> 4500 m/s in 12 layers + Gaussian-smoothed (sigma = 8
        cells) +-10 % random perturbation clipped to [1500, 5500], 64 surface shots,
        8 Hz Ricker, 1152 receivers, 4000 steps, checkpoints every 64 steps; the
        gradient is taken at a Gaussian-smoothed (sigma = 30 cells) start model.
  cfg3  3D FWI gradient: 400 x 400 x 300 cells at 15 m + 20-cell PML, order 8,
        layered + smoothed perturbation + Gaussian salt body at 4500 m/s,
        8 shots, 100 x 100 receivers, 6 Hz, 3000 steps.
  cfg4  uneven batch: 256 shots over three 2D grids of one model (288 x 96 at
        50 m / 2000 steps / 3 Hz, 576 x 192 at 25 m / 3000 / 5 Hz, 1152 x 384 at
        12.5 m / 4000 / 8 Hz; 500 m of PML each), order 6, FP32, seeded random
        source positions and record lengths; the three gradients run as one
        plan group (one CUDA graph).
  cfg5  end-to-end FWI: PySIT's LBFGS (memory 10, backtracking) for 20 iterations
        on the cfg2 model with 128 shots, from the sigma = 30 smoothed model.
``scale`` shrinks a workload uniformly (cells per axis, shots, steps) for tests.

``python -m pysit_gb300.workloads cfg5 [--iterations N] [--shots N] [--scale s]
[--nsteps N] [--plain]`` runs the FWI and prints one JSON line (objective history,
relative L2 error of the final model, wall time); ``... cfg4`` times the uneven
batch, grid by grid and as one group; ``... steps2d`` / ``steps3d`` time the three
step kernels of the cfg2 / cfg3 grids alone; ``... gradient`` times the cfg2 gradient alone
(inside an NVTX range for profilers), ``... gradient3d`` the cfg3 gradient; ``... hessian``
times the gradient, Born
modelling and the Gauss-Newton Hessian application of the cfg2 workload; ``... gn``
runs Gauss-Newton iterations (GMRES on the GPU Hessian) on the cfg5 model.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.ndimage import gaussian_filter

from . import core, solvers

__all__ = ["layered_model", "cfg1", "run_cfg1", "run_gradient", "run_gradient3d", "cfg2", "cfg3", "cfg4", "cfg5", "run_lbfgs", "run_uneven_batch", "run_hessian",
           "run_gauss_newton", "run_steps"]


def layered_model(shape, nlayers, vmin, vmax, sigma_cells, amp, seed, clip=(1500.0, 5500.0)):
    """Layers along z (last axis) plus a smoothed uniform perturbation of relative size `amp`."""
    rng = np.random.default_rng(seed)
    nz = shape[-1]
    layer = np.minimum((np.arange(nz) * nlayers) // nz, nlayers - 1)
    v1d = vmin + (vmax - vmin) * layer / max(nlayers - 1, 1)
    C = np.broadcast_to(v1d, shape).astype(float).copy()
    p = gaussian_filter(rng.uniform(-1.0, 1.0, size=shape), sigma=sigma_cells, mode="nearest")
    p /= max(np.abs(p).max(), 1e-30)
    C *= 1.0 + amp * p
    return np.clip(C, *clip)


def _steps_T(C0, deltas, cfl, nsteps):
    dt = cfl * min(deltas) / float(np.abs(C0).max())
    return (nsteps - 0.5) * dt


def cfg1(precision="double"):
    """(mesh, shots, solver, C_true, C_start) of the small CPU-sized case: 121 x 61 nodes at
    10 m with 10-cell PML (amplitude 180 = 3 c_max ln(1e3) / (2 L)), order 4, a Gaussian
    horizontal reflector (1500 m/s, +15 % at 350 m depth, 20 m wide), one 10 Hz Ricker source at
    the surface centre, 121 surface receivers, T = 1.2 s at CFL 0.5 (414 steps on the true model,
    360 on the start model); the gradient is
    taken at the constant 1500 m/s model."""
    pml = core.PML(100.0, 180.0)
    d = core.RectangularDomain((0.0, 1200.0, pml, pml), (0.0, 600.0, pml, pml))
    m = core.CartesianMesh(d, 121, 61)
    z = m.mesh_coords()[-1]
    C = 1500.0 * (1 + 0.15 * np.exp(-(z - 350.0) ** 2 / (2 * 20.0 ** 2)))
    C0 = 1500.0 * np.ones_like(C)
    shots = core.equispaced_acquisition(m, core.RickerWavelet(10.0), sources=1, receivers="max",
                                        source_depth=0.0, receiver_depth=0.0)
    solver = solvers.ConstantDensityAcousticWave(m, spatial_accuracy_order=4, trange=(0.0, 1.2),
                                                 kernel_implementation="cuda", precision=precision,
                                                 cfl_safety=0.5, autotune=True, gradient_schedule="auto")
    return m, shots, solver, C, C0


def run_cfg1(repeats=20):
    """Gradient of the small case through the batched plan (FP64) and through the plain
    per-step loop (FP64), each the mean of `repeats` calls after a warm-up."""
    import time

    import torch

    from .modeling import generate_seismic_data
    from .objective_functions import TemporalLeastSquares

    m, shots, solver, C, C0 = cfg1()
    generate_seismic_data(shots, solver, solver.ModelParameters(m, {"C": C}))
    m0 = solver.ModelParameters(m, {"C": C0})
    out = {"grid": [int(v) for v in m.shape(include_bc=True, as_grid=True)]}
    for name, batched, reps in (("batched", True, repeats), ("plain", False, max(1, repeats // 10))):
        obj = TemporalLeastSquares(solver, batched=batched)
        aux = {"objective_value": (True, None)}
        obj.compute_gradient(shots, m0, aux)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            obj.compute_gradient(shots, m0, aux)
        torch.cuda.synchronize()
        t = (time.perf_counter() - t0) / reps
        out[name] = {"seconds": t, "shots_per_s": 1.0 / t, "objective": float(aux["objective_value"][1])}
    out["nsteps"] = int(solver.nsteps)
    out["batched_over_plain"] = out["plain"]["seconds"] / out["batched"]["seconds"]
    return out


def cfg2(scale=1.0, nshots=64, nsteps=4000, order=8, precision="single", cfl=0.4, checkpoint_every=64,
         shots_per_launch=None, seed=2026, gradient_schedule="checkpoint"):
    """(mesh, shots, solver, C_true, C_start) of the 2D batched-gradient workload."""
    nx, nz = max(16, int(round(1152 * scale))), max(12, int(round(384 * scale)))
    npml = max(4, int(round(40 * scale)))
    dx = 12.5
    amp = 3 * 4500.0 * math.log(1e3) / (2 * npml * dx)  # 1e-3 reflection for a quadratic profile
    pml = core.PML(npml * dx, amp)
    d = core.RectangularDomain((0.0, (nx - 1) * dx, pml, pml), (0.0, (nz - 1) * dx, pml, pml))
    m = core.CartesianMesh(d, nx, nz)
    C = layered_model((nx, nz), 12, 1500.0, 4500.0, 8 * max(scale, 0.125), 0.10, seed)
    C0 = gaussian_filter(C, sigma=30 * max(scale, 0.05), mode="nearest")
    T = _steps_T(C0, m.deltas, cfl, nsteps)
    shots = core.equispaced_acquisition(m, core.RickerWavelet(8.0), sources=nshots, receivers="max",
                                        source_depth=0.0, receiver_depth=0.0)
    solver = solvers.ConstantDensityAcousticWave(m, spatial_accuracy_order=order, trange=(0.0, T),
                                                 kernel_implementation="cuda", precision=precision,
                                                 cfl_safety=cfl, checkpoint_every=checkpoint_every,
                                                 shots_per_launch=shots_per_launch, autotune=True,
                                                 gradient_schedule=gradient_schedule)
    return m, shots, solver, C, C0


def cfg3(scale=1.0, nshots=8, nsteps=3000, order=8, precision="single", cfl=0.35, checkpoint_every=None,
         shots_per_launch=1, seed=2027, pml_psi="consistent"):
    """(mesh, shots, solver, C_true, C_start) of the 3D gradient workload.

    Its PML amplitude (1e-3 reflection over 20 cells) makes the reference's 3D
    step diverge (C^2 on sigma_x sigma_y sigma_z psi, _3D.h:219), so the workload
    uses the consistent form by default; ``pml_psi="reference"`` reproduces the
    reference's step.  Checkpoints every sqrt(nsteps) steps (55 for 3000) unless
    ``checkpoint_every`` is given."""
    if checkpoint_every is None:
        checkpoint_every = max(1, int(round(math.sqrt(nsteps))))
    nx, ny, nz = (max(12, int(round(n * scale))) for n in (400, 400, 300))
    npml = max(4, int(round(20 * scale)))
    dx = 15.0
    amp = 3 * 4500.0 * math.log(1e3) / (2 * npml * dx)
    pml = core.PML(npml * dx, amp)
    d = core.RectangularDomain((0.0, (nx - 1) * dx, pml, pml), (0.0, (ny - 1) * dx, pml, pml),
                               (0.0, (nz - 1) * dx, pml, pml))
    m = core.CartesianMesh(d, nx, ny, nz)
    C = layered_model((nx, ny, nz), 12, 1500.0, 4000.0, 8 * max(scale, 0.125), 0.10, seed)
    x, y, z = m.mesh_coords()
    cx, cy, cz = (nx - 1) * dx / 2, (ny - 1) * dx / 2, (nz - 1) * dx * 0.55
    r2 = ((x - cx) ** 2 + (y - cy) ** 2) / (0.15 * nx * dx) ** 2 + (z - cz) ** 2 / (0.12 * nz * dx) ** 2
    salt = np.exp(-r2) > 0.5
    C = np.where(salt.reshape(C.shape), 4500.0, C)
    C0 = gaussian_filter(C, sigma=10 * max(scale, 0.1), mode="nearest")
    T = _steps_T(C0, m.deltas, cfl, nsteps)
    # a source grid of exactly nshots points, as square as the divisors allow
    nsx = max(d for d in range(1, int(math.isqrt(nshots)) + 1) if nshots % d == 0)
    shots = core.equispaced_acquisition(m, core.RickerWavelet(6.0), sources=(nshots // nsx, nsx),
                                        receivers=(min(100, nx), min(100, ny)), source_depth=0.0,
                                        receiver_depth=0.0)
    solver = solvers.ConstantDensityAcousticWave(m, spatial_accuracy_order=order, trange=(0.0, T),
                                                 kernel_implementation="cuda", precision=precision,
                                                 cfl_safety=cfl, checkpoint_every=checkpoint_every,
                                                 shots_per_launch=shots_per_launch, pml_psi=pml_psi,
                                                 autotune=True)
    return m, shots, solver, C, C0


def cfg5(scale=1.0, nshots=128, nsteps=4000, precision="single", shots_per_launch=None, gradient_schedule="auto",
         **kw):
    """(mesh, shots, solver, C_true, C_start) of the end-to-end FWI workload: the cfg2 model
    and start model with 128 shots.  The default schedule keeps dWaveOp in HBM with as many
    shots per launch as fit; ``gradient_schedule="checkpoint", shots_per_launch=64`` is the
    checkpointed configuration."""
    return cfg2(scale=scale, nshots=nshots, nsteps=nsteps, precision=precision,
                shots_per_launch=shots_per_launch, gradient_schedule=gradient_schedule, **kw)


def run_lbfgs(m, shots, solver, C, C0, iterations=20, memory_length=10, batched=True, verbose=False):
    """PySIT's LBFGS on data modelled at C, started from C0, with the GPU objective.
    Returns the objective history, the relative L2 error of the final model to C,
    and the wall time of the optimisation (the data modelling excluded)."""
    import time

    from .modeling import generate_seismic_data
    from .objective_functions import TemporalLeastSquares
    from .optimization import LBFGS

    generate_seismic_data(shots, solver, solver.ModelParameters(m, {"C": C}))
    objective = TemporalLeastSquares(solver, batched=batched)
    opt = LBFGS(objective, memory_length=memory_length)
    t0 = time.perf_counter()
    final = opt(shots, solver.ModelParameters(m, {"C": C0}), iterations, line_search="backtrack",
                status_configuration={"objective_frequency": 1, "gradient_length_frequency": 1},
                verbose=verbose)
    seconds = time.perf_counter() - t0
    _, hist = opt.retrieve_history("objective")
    _, alpha = opt.retrieve_history("alpha")
    Cf = np.asarray(final.C).reshape(-1)
    Ct = np.asarray(C).reshape(-1)
    C0f = np.asarray(C0).reshape(-1)
    return {"objective": [float(v) for v in hist], "alpha": [float(a) for a in alpha],
            "rel_model_error": float(np.linalg.norm(Cf - Ct) / np.linalg.norm(Ct)),
            "rel_model_error_start": float(np.linalg.norm(C0f - Ct) / np.linalg.norm(Ct)),
            "seconds": seconds, "iterations": iterations, "shots": len(shots), "nsteps": solver.nsteps,
            "plan": ({"schedule": objective.last_plan.gradient_schedule,
                      "shots_per_launch": objective.last_plan.shots_per_launch} if objective.last_plan else None)}


def cfg4(scale=1.0, nshots=256, order=6, precision="single", seed=2028, cfl=0.4, gradient_schedule="checkpoint"):
    """The uneven batch: a list of three grids, each (mesh, shots, solver, C, C0, record_steps).

    One model (the cfg2 model at 12.5 m) sampled every 4th / 2nd / 1st cell; shots split as
    evenly as possible, source x seeded-random at the surface, all grid columns as
    receivers, record lengths seeded-random in [nsteps/2, nsteps]."""
    rng = np.random.default_rng(seed)
    nx_f, nz_f = max(32, int(round(1152 * scale))) // 4 * 4, max(16, int(round(384 * scale))) // 4 * 4
    C_f = layered_model((nx_f, nz_f), 12, 1500.0, 4500.0, 8 * max(scale, 0.125), 0.10, 2026)
    grids = [(4, 50.0, 2000, 3.0), (2, 25.0, 3000, 5.0), (1, 12.5, 4000, 8.0)]
    counts = [nshots // 3 + (1 if i < nshots % 3 else 0) for i in range(3)]
    out = []
    for (step, dx, nsteps, freq), ns in zip(grids, counts):
        nsteps = max(16, int(round(nsteps * min(1.0, scale))))
        C = np.ascontiguousarray(C_f[::step, ::step])
        nx, nz = C.shape
        npml = max(4, int(round(500.0 / dx * min(1.0, max(scale, 0.25)))))
        amp = 3 * 4500.0 * math.log(1e3) / (2 * npml * dx)
        pml = core.PML(npml * dx, amp)
        d = core.RectangularDomain((0.0, (nx - 1) * dx, pml, pml), (0.0, (nz - 1) * dx, pml, pml))
        m = core.CartesianMesh(d, nx, nz)
        C0 = gaussian_filter(C, sigma=30.0 / step * max(scale, 0.05), mode="nearest")
        T = _steps_T(C0, m.deltas, cfl, nsteps)
        w = core.RickerWavelet(freq)
        xs = rng.uniform(0.05, 0.95, size=ns) * (nx - 1) * dx
        rec_x = np.arange(nx) * dx
        shots = []
        for x in xs:
            src = core.PointSource(m, (float(x), 0.0), w)
            rec = core.ReceiverSet(m, [core.PointReceiver(m, (float(r), 0.0)) for r in rec_x])
            shots.append(core.Shot(src, rec))
        solver = solvers.ConstantDensityAcousticWave(m, spatial_accuracy_order=order, trange=(0.0, T),
                                                     kernel_implementation="cuda", precision=precision,
                                                     cfl_safety=cfl, checkpoint_every=64, autotune=True,
                                                     gradient_schedule=gradient_schedule)
        record = rng.integers(nsteps // 2, nsteps + 1, size=ns)
        out.append((m, shots, solver, C.reshape(-1, 1), C0.reshape(-1, 1), record))
    return out


def run_uneven_batch(grids, repeats=2):
    """Observed data on the true models, then the gradients of all grids at the start models:
    timed grid after grid (one plan call each) and as one plan group.  Returns shots/s of both."""
    import time

    import torch

    from .engine import PlanGroup, WavePlan

    # plans are built largest first (cells x steps x shots): with an 'auto' schedule the grid
    # with the most work gets first claim on the memory that keeping dWaveOp needs
    def work(g):
        m, shots, solver, C, C0, record = g
        solver.model_parameters = solver.ModelParameters(m, {"C": C0})
        return int(np.prod(m.shape(include_bc=True, as_grid=True))) * solver.nsteps * len(shots)

    order = sorted(range(len(grids)), key=lambda i: -work(grids[i]))
    built = {}
    for i in order:
        m, shots, solver, C, C0, record = grids[i]
        solver.model_parameters = solver.ModelParameters(m, {"C": C})
        obs_plan = WavePlan(solver, shots, forward_only=True)
        obs = obs_plan.forward().clone()
        ts_true = solver.ts()
        del obs_plan
        solver.model_parameters = solver.ModelParameters(m, {"C": C0})
        # record lengths are counted on the start model's time axis
        rec = np.minimum(record, solver.nsteps)
        p = WavePlan(solver, shots, record_steps=rec)
        p.autotune()
        from .autograd import resample_linear
        p.dobs.copy_(resample_linear(obs, ts_true, solver.ts()))
        del obs
        torch.cuda.empty_cache()
        built[i] = p
    plans = [built[i] for i in range(len(grids))]
    nshots = sum(len(g[1]) for g in grids)
    group = PlanGroup(plans)
    for p in plans:
        p.gradient()
    group.gradient()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(repeats):
        for p in plans:
            p.gradient()
    torch.cuda.synchronize()
    t_seq = (time.perf_counter() - t0) / repeats
    t0 = time.perf_counter()
    for _ in range(repeats):
        group.gradient()
    torch.cuda.synchronize()
    t_grp = (time.perf_counter() - t0) / repeats
    status = [p.status() for p in plans]
    return {"shots": nshots, "grids": [[int(s) for s in g[0].shape(as_grid=True)] for g in grids],
            "shots_per_grid": [len(g[1]) for g in grids], "nsteps": [int(p.nsteps) for p in plans],
            "tile_x": [int(p.tile_x) for p in plans], "schedules": [p.gradient_schedule for p in plans],
            "shots_per_launch": [int(p.shots_per_launch) for p in plans],
            "sequential_s": t_seq, "group_s": t_grp, "shots_per_s_sequential": nshots / t_seq,
            "shots_per_s_group": nshots / t_grp, "group_speedup": t_seq / t_grp, "status": status}


def run_hessian(m, shots, solver, C, C0, repeats=2):
    """Observed data on the true model, then at the start model: the batched gradient, Born
    modelling F m1 and the Gauss-Newton Hessian application sum_s F_s* F_s m1 of all shots, each
    timed as one plan call (m1 a seeded smooth perturbation of 1 % of m0).  Returns seconds and
    shots/s of each."""
    import time

    import torch

    from .engine import WavePlan

    solver.model_parameters = solver.ModelParameters(m, {"C": C})
    obs = WavePlan(solver, shots, forward_only=True).forward().clone()
    ts_true = solver.ts()
    torch.cuda.empty_cache()
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    plan = WavePlan(solver, shots)
    plan.autotune()
    from .autograd import resample_linear
    plan.dobs.copy_(resample_linear(obs, ts_true, solver.ts()))
    del obs
    torch.cuda.empty_cache()
    shape = tuple(m.shape(as_grid=True))
    rng = np.random.default_rng(2029)
    m1 = 0.01 * gaussian_filter(rng.standard_normal(shape), 4.0).reshape(-1) / np.asarray(C0).reshape(-1) ** 2
    out = {"shots": len(shots), "grid": [int(v) for v in shape], "nsteps": int(plan.nsteps), "tile_x": int(plan.tile_x),
           "schedule": plan.gradient_schedule, "shots_per_launch": plan.shots_per_launch}
    for name, fn in (("gradient", plan.gradient), ("born", lambda: plan.born(m1)),
                     ("hessian", lambda: plan.hessian(m1))):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(repeats):
            fn()
        torch.cuda.synchronize()
        t = (time.perf_counter() - t0) / repeats
        out[f"{name}_s"] = t
        out[f"{name}_shots_per_s"] = len(shots) / t
        out[f"{name}_launches"] = plan.launches()
    out["hessian_norm"] = float(plan.hess.norm().item())
    out["status"] = plan.status()
    return out


def run_gradient(scale=1.0, nshots=64, nsteps=4000, shots_per_launch=None, schedule="auto", repeats=1):
    """The 2D batched gradient alone: observed data on the true model, one warm-up gradient at
    the start model, then `repeats` gradients inside the NVTX range "timed_gradient" (a profiler
    can select exactly their launches).  Returns seconds per gradient and shots/s."""
    import time

    import torch

    from .autograd import resample_linear
    from .engine import WavePlan

    m, shots, solver, C, C0 = cfg2(scale=scale, nshots=nshots, nsteps=nsteps, gradient_schedule=schedule)
    solver.model_parameters = solver.ModelParameters(m, {"C": C})
    obs = WavePlan(solver, shots, forward_only=True).forward().clone()
    ts_true = solver.ts()
    torch.cuda.empty_cache()
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    plan = WavePlan(solver, shots, shots_per_launch=shots_per_launch)
    plan.autotune()
    plan.dobs.copy_(resample_linear(obs, ts_true, solver.ts()))
    del obs
    plan.gradient()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("timed_gradient")
    t0 = time.perf_counter()
    for _ in range(repeats):
        plan.gradient()
    torch.cuda.synchronize()
    t = (time.perf_counter() - t0) / repeats
    torch.cuda.nvtx.range_pop()
    return {"shots": nshots, "nsteps": int(plan.nsteps), "schedule": plan.gradient_schedule,
            "shots_per_launch": plan.shots_per_launch, "tile_x": plan.tile_x, "seconds": t,
            "shots_per_s": nshots / t, "launches": plan.launches(), "status": plan.status()}


def run_gradient3d(scale=1.0, nshots=8, nsteps=3000, autotune=True):
    """The 3D gradient (cfg3, consistent psi form, checkpointed, one shot per launch): observed
    data on the true model, one warm-up gradient at the start model, then one timed gradient
    (CUDA events).  Returns seconds, shots/s, Gcell/s of the three sweeps and the tuning."""
    import time

    import torch

    from .autograd import resample_linear
    from .engine import WavePlan

    m, shots, solver, C, C0 = cfg3(scale=scale, nshots=nshots, nsteps=nsteps)
    solver.model_parameters = solver.ModelParameters(m, {"C": C})
    ts_obs = solver.ts()
    obs = WavePlan(solver, shots, shots_per_launch=1, forward_only=True).forward().clone()
    torch.cuda.empty_cache()
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    plan = WavePlan(solver, shots, shots_per_launch=1)
    tune = plan.autotune() if autotune else {"chosen": plan.tile_x}
    plan.dobs.copy_(resample_linear(obs, ts_obs, solver.ts()))
    del obs
    plan.gradient()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record()
    plan.gradient()
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    cells = int(np.prod(m.shape(include_bc=True, as_grid=True)))
    return {"shots": nshots, "nsteps": int(plan.nsteps), "grid": [int(v) for v in m.shape(include_bc=True, as_grid=True)],
            "checkpoint_every": plan.checkpoint_every, "workspace_gb": plan.workspace_bytes / 1e9,
            "tile_x": tune["chosen"], "tune_ms": {str(k): v for k, v in tune.get("ms", {}).items()},
            "seconds": t, "wall_s": time.perf_counter() - t0, "shots_per_s": nshots / t,
            "gcell_per_s": 3 * cells * plan.nsteps * nshots / t / 1e9, "status": plan.status()}


def run_steps(workload="cfg2", scale=1.0, nshots=None, nsteps=64, shots_per_launch=None, reps=32,
              schedule="checkpoint"):
    """Per-launch times of the three step kernels (forward, recompute, adjoint) of a workload's
    first shot group, each timed alone with CUDA events (pysit_plan_step_loop), with the
    algorithmic bytes of the step and Gcell/s (a benchmarking aid for profiling)."""
    import torch

    from .engine import WavePlan

    if workload == "cfg2":
        m, shots, solver, C, C0 = cfg2(scale=scale, nshots=nshots or 64, nsteps=nsteps)
        pml_extra = (4, 4)  # Phi_x, Phi_z in and out
    else:
        m, shots, solver, C, C0 = cfg3(scale=scale, nshots=nshots or 1, nsteps=nsteps)
        pml_extra = (8, 8)  # Phi_x, Phi_y, Phi_z, psi in and out
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    # (with the kept schedule the recompute-mode launches also record traces, as its forward sweep does)
    plan = WavePlan(solver, shots, shots_per_launch=shots_per_launch or len(shots), gradient_schedule=schedule)
    plan.forward()
    torch.cuda.synchronize()
    n_all = int(np.prod(m.shape(include_bc=True, as_grid=True)))
    n_int = m.dof()
    n_pml = n_all - n_int
    w = 4 if solver.precision == "single" else 8
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {"workload": workload, "scale": scale, "grid": [int(v) for v in m.shape(include_bc=True, as_grid=True)],
           "shots_per_launch": plan.shots_per_launch, "schedule": plan.gradient_schedule, "modes": {}}
    for mode, name, extra in ((0, "forward", 0), (1, "recompute", 1), (2, "adjoint", 3)):
        plan.step_loop(mode, 4)
        torch.cuda.synchronize()
        e0.record()
        plan.step_loop(mode, reps)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        nb = w * ((4 + extra) * n_int + (4 + pml_extra[0] + extra) * n_pml) * plan.shots_per_launch
        out["modes"][name] = {"launch_ms": ms, "gbs": nb / (ms * 1e-3) / 1e9,
                              "gcell_per_s": n_all * plan.shots_per_launch / (ms * 1e-3) / 1e9}
    out["status"] = plan.status()
    return out


def run_gauss_newton(m, shots, solver, C, C0, iterations=3, krylov_maxiter=5, batched=True, verbose=False):
    """PySIT-style Gauss-Newton (GMRES inner solve on the batched GPU Hessian, backtracking line
    search with alpha0 = 1) from the smoothed start model; objective history, relative model
    error before and after, wall time."""
    import time

    from .modeling import generate_seismic_data
    from .objective_functions import TemporalLeastSquares
    from .optimization import GaussNewton

    generate_seismic_data(shots, solver, solver.ModelParameters(m, {"C": C}))
    obj = TemporalLeastSquares(solver, batched=batched)
    gn = GaussNewton(obj, krylov_maxiter=krylov_maxiter)
    start = solver.ModelParameters(m, {"C": C0})
    t0 = time.perf_counter()
    final = gn(shots, start, iterations, line_search="backtrack", verbose=verbose,
               status_configuration={"objective_frequency": 1})
    wall = time.perf_counter() - t0
    _, objective = gn.retrieve_history("objective")
    _, alpha = gn.retrieve_history("alpha")
    err = lambda c: float(np.linalg.norm(np.asarray(c).reshape(-1) - C.reshape(-1)) / np.linalg.norm(C))  # noqa: E731
    return {"iterations": iterations, "krylov_maxiter": krylov_maxiter, "shots": len(shots),
            "objective": [float(v) for v in objective], "alpha": [float(v) for v in alpha],
            "model_error_start": err(C0), "model_error_final": err(final.C), "wall_s": wall}


def _main(argv=None):
    import argparse
    import json

    ap = argparse.ArgumentParser(prog="python -m pysit_gb300.workloads")
    ap.add_argument("workload", choices=["cfg1", "cfg4", "cfg5", "gradient", "gradient3d", "hessian", "gn", "steps2d",
                                         "steps3d"])
    ap.add_argument("--shots-per-launch", type=int, default=None)
    ap.add_argument("--schedule", default="auto", choices=["checkpoint", "store", "auto"],
                    help="cfg5 / gn / hessian: gradient schedule of the batched plans")
    ap.add_argument("--krylov", type=int, default=5, help="gn: GMRES iterations per Gauss-Newton step")
    ap.add_argument("--iterations", type=int, default=20)
    ap.add_argument("--shots", type=int, default=None, help="default 256 (cfg4), 128 (cfg5)")
    ap.add_argument("--nsteps", type=int, default=4000)
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--plain", action="store_true", help="per-shot FP64 objective instead of the batched FP32 one")
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args(argv)
    if a.workload == "cfg4":
        out = run_uneven_batch(cfg4(scale=a.scale, nshots=a.shots or 256, gradient_schedule=a.schedule))
        out.update(workload="cfg4", scale=a.scale)
        print(json.dumps(out))
        return
    if a.workload == "gradient":
        out = run_gradient(scale=a.scale, nshots=a.shots or 64, nsteps=a.nsteps, shots_per_launch=a.shots_per_launch,
                           schedule=a.schedule)
        out.update(workload="cfg2 gradient")
        print(json.dumps(out))
        return
    if a.workload == "gradient3d":
        out = run_gradient3d(scale=a.scale, nshots=a.shots or 8, nsteps=a.nsteps if a.nsteps != 4000 else 3000)
        out.update(workload="cfg3 gradient")
        print(json.dumps(out))
        return
    if a.workload == "cfg1":
        out = run_cfg1()
        out.update(workload="cfg1: 121 x 61 at 10 m + 10 PML, order 4, FP64, 1 shot, 414 steps")
        print(json.dumps(out))
        return
    if a.workload in ("steps2d", "steps3d"):
        out = run_steps("cfg2" if a.workload == "steps2d" else "cfg3", scale=a.scale, nshots=a.shots,
                        nsteps=a.nsteps, shots_per_launch=a.shots_per_launch,
                        schedule="store" if a.schedule == "store" else "checkpoint")
        print(json.dumps(out))
        return
    if a.workload == "hessian":
        m, shots, solver, C, C0 = cfg2(scale=a.scale, nshots=a.shots or 64, nsteps=a.nsteps,
                                       shots_per_launch=a.shots_per_launch, gradient_schedule=a.schedule)
        out = run_hessian(m, shots, solver, C, C0)
        out.update(workload="hessian on the cfg2 model", scale=a.scale)
        print(json.dumps(out))
        return
    prec = "double" if a.plain else "single"
    if a.workload == "gn":
        m, shots, solver, C, C0 = cfg5(scale=a.scale, nshots=a.shots or 64, nsteps=a.nsteps, precision=prec,
                                       shots_per_launch=a.shots_per_launch, gradient_schedule=a.schedule)
        out = run_gauss_newton(m, shots, solver, C, C0, iterations=a.iterations, krylov_maxiter=a.krylov,
                               batched=not a.plain, verbose=a.verbose)
        out.update(workload="Gauss-Newton on the cfg5 model", path="plain FP64" if a.plain else "batched FP32",
                   scale=a.scale)
        print(json.dumps(out))
        return
    m, shots, solver, C, C0 = cfg5(scale=a.scale, nshots=a.shots or 128, nsteps=a.nsteps, precision=prec,
                                   shots_per_launch=a.shots_per_launch, gradient_schedule=a.schedule)
    out = run_lbfgs(m, shots, solver, C, C0, iterations=a.iterations, batched=not a.plain, verbose=a.verbose)
    out.update(workload=a.workload, path="plain FP64" if a.plain else "batched FP32", scale=a.scale,
               schedule=getattr(solver, "gradient_schedule", None))
    print(json.dumps(out))


if __name__ == "__main__":
    _main()
