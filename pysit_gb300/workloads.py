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

The runners that time these workloads are in measure.py at the repository root.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.ndimage import gaussian_filter

from . import core, solvers

__all__ = ["layered_model", "cfg1", "cfg2", "cfg3", "cfg4", "cfg5"]


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
