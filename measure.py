"""Measurement runners for the workloads of pysit_gb300.workloads (beside bench.py, which
measures the headline configuration).

    python measure.py cfg1                 small case: batched and plain gradient times
    python measure.py gradient             2D workload gradient alone (NVTX range for profilers)
    python measure.py gradient3d           3D workload gradient (8 shots x 3000 steps)
    python measure.py steps2d | steps3d    the three step kernels of the 2D / 3D grids, each alone
    python measure.py cfg4                 uneven batch, grid by grid and as one plan group
    python measure.py cfg5 [--precision double] [--plain]
                                           end-to-end LBFGS FWI (batched FP32 by default; batched
                                           FP64, or the plain per-shot FP64 path)
    python measure.py hessian | gn         Born / Hessian times; Gauss-Newton iterations
Each prints one JSON line.
"""
from __future__ import annotations

import numpy as np

from pysit_gb300.workloads import cfg1, cfg2, cfg3, cfg4, cfg5


def run_cfg1(repeats=20):
    """Gradient of the small case through the batched plan (FP64) and through the plain
    per-step loop (FP64), each the mean of `repeats` calls after a warm-up."""
    import time

    import torch

    from pysit_gb300.modeling import generate_seismic_data
    from pysit_gb300.objective_functions import TemporalLeastSquares

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


def run_lbfgs(m, shots, solver, C, C0, iterations=20, memory_length=10, batched=True, verbose=False):
    """PySIT's LBFGS on data modelled at C, started from C0, with the GPU objective.
    Returns the objective history, the relative L2 error of the final model to C,
    and the wall time of the optimisation (the data modelling excluded)."""
    import time

    from pysit_gb300.modeling import generate_seismic_data
    from pysit_gb300.objective_functions import TemporalLeastSquares
    from pysit_gb300.optimization import LBFGS

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


def run_uneven_batch(grids, repeats=2):
    """Observed data on the true models, then the gradients of all grids at the start models:
    timed grid after grid (one plan call each) and as one plan group.  Returns shots/s of both."""
    import time

    import torch

    from pysit_gb300.engine import PlanGroup, WavePlan

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
        from pysit_gb300.autograd import resample_linear
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

    from pysit_gb300.engine import WavePlan

    solver.model_parameters = solver.ModelParameters(m, {"C": C})
    obs = WavePlan(solver, shots, forward_only=True).forward().clone()
    ts_true = solver.ts()
    torch.cuda.empty_cache()
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    plan = WavePlan(solver, shots)
    plan.autotune()
    from pysit_gb300.autograd import resample_linear
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

    from pysit_gb300.autograd import resample_linear
    from pysit_gb300.engine import WavePlan

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

    from pysit_gb300.autograd import resample_linear
    from pysit_gb300.engine import WavePlan

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
            "tile_x": tune["chosen"], "tile_z": tune.get("chosen_z"),
            "tune_ms": {str(k): v for k, v in tune.get("ms", {}).items()},
            "seconds": t, "wall_s": time.perf_counter() - t0, "shots_per_s": nshots / t,
            "gcell_per_s": 3 * cells * plan.nsteps * nshots / t / 1e9, "status": plan.status()}


def run_steps(workload="cfg2", scale=1.0, nshots=None, nsteps=64, shots_per_launch=None, reps=32,
              schedule="checkpoint", tile=None):
    """Per-launch times of the three step kernels (forward, recompute, adjoint) of a workload's
    first shot group, each timed alone with CUDA events (pysit_plan_step_loop), with the
    algorithmic bytes of the step and Gcell/s (a benchmarking aid for profiling).  `tile` sets
    the x task length (default: the plan's own); the timed loops run inside the NVTX range
    `steps`, so that a profiler can pick out their launches."""
    import torch

    from pysit_gb300.engine import WavePlan

    if workload == "cfg2":
        m, shots, solver, C, C0 = cfg2(scale=scale, nshots=nshots or 64, nsteps=nsteps)
        pml_extra = (4, 4)  # Phi_x, Phi_z in and out
    else:
        m, shots, solver, C, C0 = cfg3(scale=scale, nshots=nshots or 1, nsteps=nsteps)
        pml_extra = (8, 8)  # Phi_x, Phi_y, Phi_z, psi in and out
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    # (with the kept schedule the recompute-mode launches also record traces, as its forward sweep does)
    plan = WavePlan(solver, shots, shots_per_launch=shots_per_launch or len(shots), gradient_schedule=schedule)
    if tile:
        plan.autotune(candidates=[int(tile)], nsteps=4, z_candidates=[0])
    plan.forward()
    torch.cuda.synchronize()
    n_all = int(np.prod(m.shape(include_bc=True, as_grid=True)))
    n_int = m.dof()
    n_pml = n_all - n_int
    w = 4 if solver.precision == "single" else 8
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {"workload": workload, "scale": scale, "grid": [int(v) for v in m.shape(include_bc=True, as_grid=True)],
           "shots_per_launch": plan.shots_per_launch, "schedule": plan.gradient_schedule,
           "tile_x": plan.tile_x or "plan default", "modes": {}}
    for mode, name, extra in ((0, "forward", 0), (1, "recompute", 1), (2, "adjoint", 3)):
        plan.step_loop(mode, 4)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("steps")
        e0.record()
        plan.step_loop(mode, reps)
        e1.record()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
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

    from pysit_gb300.modeling import generate_seismic_data
    from pysit_gb300.objective_functions import TemporalLeastSquares
    from pysit_gb300.optimization import GaussNewton

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

    ap = argparse.ArgumentParser(prog="python measure.py")
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
    ap.add_argument("--tile", type=int, default=None, help="steps2d / steps3d: x task length (default: the plan's)")
    ap.add_argument("--plain", action="store_true", help="per-shot FP64 objective instead of the batched FP32 one")
    ap.add_argument("--precision", default="single", choices=["single", "double"],
                    help="cfg5 / gn: precision of the batched objective")
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
                        schedule="store" if a.schedule == "store" else "checkpoint", tile=a.tile)
        print(json.dumps(out))
        return
    if a.workload == "hessian":
        m, shots, solver, C, C0 = cfg2(scale=a.scale, nshots=a.shots or 64, nsteps=a.nsteps,
                                       shots_per_launch=a.shots_per_launch, gradient_schedule=a.schedule)
        out = run_hessian(m, shots, solver, C, C0)
        out.update(workload="hessian on the cfg2 model", scale=a.scale)
        print(json.dumps(out))
        return
    prec = "double" if a.plain else a.precision
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
    out.update(workload=a.workload, path="plain FP64" if a.plain else f"batched {'FP64' if prec == 'double' else 'FP32'}",
               scale=a.scale,
               schedule=getattr(solver, "gradient_schedule", None))
    print(json.dumps(out))


if __name__ == "__main__":
    _main()
