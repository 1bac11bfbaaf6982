"""Seeded test problems, buildable with either API (the reference ``pysit`` or ``pysit_gb300``).

Each spec fixes a domain, PML, grid, order, velocity model, acquisition and time
range.  ``build(api, name, kernel)`` returns (mesh, shots, solver, C_true, C0);
the same code builds the problem through the live reference (golden fixtures,
tests/golden/make_golden.py) and through pysit_gb300 (parity tests), so the two
runs see identical inputs.  ``oracle_problem`` converts a pysit_gb300 solver and
shot into the plain-array problem of oracle/pipeline.py.
"""
from __future__ import annotations

import numpy as np

# name -> spec.  n = unpadded nodes per axis (x[, y], z); L = physical lengths;
# pml = (cells, amplitude) or None per side; src/rec positions are in metres.
SPECS = {
    # config 1 of the benchmark description: 121x61 @ 10 m + 10-cell PML, order 4,
    # Gaussian horizontal reflector, 10 Hz Ricker at the surface centre, 121 receivers
    "cfg1": dict(dim=2, n=(121, 61), L=(1200.0, 600.0), pml=(10, 180.0), order=4, T=1.2, cfl=0.5,
                 f=10.0, model="reflector", nsrc=1, nrec="max", sdepth=0.0, rdepth=0.0),
    "o2": dict(dim=2, n=(48, 36), L=(470.0, 350.0), pml=(6, 150.0), order=2, T=0.25, cfl=0.4,
               f=25.0, model="layered", nsrc=2, nrec=24, sdepth=30.0, rdepth=20.0),
    "o6": dict(dim=2, n=(53, 41), L=(520.0, 400.0), pml=(8, 160.0), order=6, T=0.3, cfl=0.35,
               f=20.0, model="layered", nsrc=1, nrec=26, sdepth=40.0, rdepth=10.0),
    "o8": dict(dim=2, n=(57, 47), L=(560.0, 460.0), pml=(9, 170.0), order=8, T=0.3, cfl=0.3,
               f=20.0, model="random", nsrc=2, nrec=29, sdepth=50.0, rdepth=30.0),
    "dirichlet": dict(dim=2, n=(45, 39), L=(440.0, 380.0), pml=(7, 160.0), order=6, T=0.25, cfl=0.35,
                      f=22.0, model="layered", nsrc=1, nrec=22, sdepth=60.0, rdepth=40.0, top="dirichlet"),
    "1d": dict(dim=1, n=(151,), L=(1500.0,), pml=(12, 140.0), order=4, T=0.8, cfl=0.5,
               f=8.0, model="layered", src=(300.0,), rec=(150.0, 700.0, 1100.0)),
    # the reference 3D PML is unstable at any positive amplitude (sigma_x sigma_y sigma_z psi
    # is multiplied by C^2, _3D.h:219): small amplitudes keep the fixtures finite
    "3d": dict(dim=3, n=(23, 21, 19), L=(220.0, 200.0, 180.0), pml=(4, 5.0), order=4, T=0.12, cfl=0.3,
               f=30.0, model="layered", nsrc=(1, 1), nrec=(5, 4), sdepth=40.0, rdepth=20.0),
    "3d_o8": dict(dim=3, n=(20, 19, 18), L=(190.0, 180.0, 170.0), pml=(5, 5.0), order=8, T=0.08, cfl=0.25,
                  f=35.0, model="random", nsrc=(1, 1), nrec=(3, 3), sdepth=50.0, rdepth=30.0),
}

# Deep grids (GPU tests against the oracle, no fixtures): the padded z extent (433 cells in 2D,
# 171 in 3D) splits the interior into several z-segments of the step kernels' task tables in
# both precisions, with the sources at mid depth so that the fields cross the segment boundaries.
DEEP_SPECS = {
    "deep": dict(dim=2, n=(41, 401), L=(400.0, 4000.0), pml=(16, 200.0), order=8, T=0.4, cfl=0.4,
                 f=25.0, model="layered", nsrc=2, nrec=20, sdepth=2000.0, rdepth=1800.0),
    "deep3d": dict(dim=3, n=(15, 13, 161), L=(140.0, 120.0, 1600.0), pml=(5, 5.0), order=8, T=0.14, cfl=0.25,
                   f=30.0, model="layered", nsrc=(1, 1), nrec=(3, 3), sdepth=800.0, rdepth=700.0),
    # many receivers (12 shots x 501, about 47 taps each): more receiver threads than the 2D trace
    # recorder's blocks hold at once, so the recorder strides over the receivers in several passes
    "manyrec": dict(dim=2, n=(501, 47), L=(5000.0, 460.0), pml=(9, 170.0), order=8, T=0.3, cfl=0.3,
                    f=20.0, model="random", nsrc=12, nrec="max", sdepth=50.0, rdepth=30.0),
}


def _models(mesh, spec):
    coords = mesh.mesh_coords()
    z = coords[-1]
    kind = spec["model"]
    if kind == "reflector":
        C = 1500.0 * (1 + 0.15 * np.exp(-(z - 350.0) ** 2 / (2 * 20.0 ** 2)))
        C0 = 1500.0 * np.ones_like(C)
        return C, C0
    zmax = spec["L"][-1]
    if kind == "layered":
        C = 1500.0 + 1200.0 * np.floor(4 * z / zmax) / 4.0
        C0 = 1500.0 + 1200.0 * z / zmax * 0.75
        return C, C0
    rng = np.random.default_rng(2026)
    C = 1600.0 + 900.0 * z / zmax + 120.0 * rng.standard_normal(z.shape)
    C0 = 1600.0 + 900.0 * z / zmax
    return C, C0


def build(api, name, kernel="cuda", precision="double", spec_overrides=None, **solver_kw):
    """(mesh, shots, solver, C_true, C_start) of problem `name`; spec_overrides replaces
    entries of its spec (e.g. the PML), solver_kw go to the solver."""
    spec = dict({**SPECS, **DEEP_SPECS}[name], **(spec_overrides or {}))
    cells, amp = spec["pml"]
    dim = spec["dim"]
    deltas = [L / (n - 1) for L, n in zip(spec["L"], spec["n"])]
    axes = []
    for a in range(dim):
        pml = api.PML(cells * deltas[a], amp)
        lbc = pml
        if a == dim - 1 and spec.get("top") == "dirichlet":
            lbc = api.Dirichlet()
        axes.append((0.0, spec["L"][a], lbc, pml))
    d = api.RectangularDomain(*axes)
    m = api.CartesianMesh(d, *spec["n"])
    C, C0 = _models(m, spec)
    w = api.RickerWavelet(spec["f"])
    if dim == 1:
        src = api.PointSource(m, spec["src"], w)
        rec = api.ReceiverSet(m, [api.PointReceiver(m, (z,)) for z in spec["rec"]])
        shots = [api.Shot(src, rec)]
    else:
        shots = api.equispaced_acquisition(m, w, sources=spec["nsrc"], source_depth=spec["sdepth"],
                                           receivers=spec["nrec"], receiver_depth=spec["rdepth"])
    kw = dict(spatial_accuracy_order=spec["order"], trange=(0.0, spec["T"]), kernel_implementation=kernel,
              cfl_safety=spec["cfl"])
    if precision != "double":
        kw["precision"] = precision
    kw.update(solver_kw)
    solver = api.ConstantDensityAcousticWave(m, **kw)
    return m, shots, solver, C, C0


def oracle_problem(solver, shot):
    """Plain-array problem of oracle/pipeline.py for one pysit_gb300 shot (model already set)."""
    from pysit_gb300.engine import padded_cells
    from pysit_gb300.solvers.cda_time import axis_sigma_map
    mesh = solver.mesh
    ts = solver.ts()
    sc, sp, sw = shot.sources.taps()
    rc, rr, rws, rwi = shot.receivers.taps()
    return dict(
        dim=mesh.dim, order=solver.spatial_accuracy_order, shape=list(mesh.shape(include_bc=True, as_grid=True)),
        deltas=list(mesh.deltas), C=np.ascontiguousarray(solver.model_parameters.C.reshape(-1)),
        dt=solver.dt, nsteps=solver.nsteps,
        profiles=[solver._profiles(a) for a in range(mesh.dim)],
        sigmaps=[axis_sigma_map(mesh, a) for a in range(mesh.dim)],
        pads=[(mesh.parameters[a].lbc.n, mesh.parameters[a].rbc.n) for a in range(mesh.dim)],
        src=(padded_cells(mesh, sc), np.asarray(sp), np.asarray(sw), shot.sources.amplitudes(ts)),
        rec=(padded_cells(mesh, rc), np.asarray(rr), np.asarray(rws), np.asarray(rwi),
             shot.receivers.receiver_count),
    )
