"""The synthetic workloads have the shapes, sizes and value ranges their descriptions state
(grids, PML widths, orders, shots, receivers, source frequencies, step counts, velocity ranges),
so that measurements on them measure the configurations they are named for."""
import numpy as np
import pytest

from pysit_gb300 import workloads


def _ricker_hz(shot):
    src = shot.sources
    return src.w.peak_frequency if hasattr(src, "w") else src.sources[0].w.peak_frequency


def test_small_case():
    m, shots, solver, C, C0 = workloads.cfg1()
    assert tuple(m.shape(as_grid=True)) == (121, 61) and tuple(m.deltas) == (10.0, 10.0)
    assert tuple(m.shape(include_bc=True, as_grid=True)) == (141, 81)
    assert solver.spatial_accuracy_order == 4 and solver.dtype == np.double
    assert len(shots) == 1 and shots[0].receivers.receiver_count == 121
    assert shots[0].sources.position == (600.0, 0.0) and _ricker_hz(shots[0]) == 10.0
    assert C.min() == pytest.approx(1500.0) and C.max() == pytest.approx(1725.0, rel=1e-3)
    solver.model_parameters = solver.ModelParameters(m, {"C": C})
    assert solver.nsteps == 414
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    assert solver.nsteps == 360


def test_2d_gradient_workload():
    m, shots, solver, C, C0 = workloads.cfg2()
    assert tuple(m.shape(as_grid=True)) == (1152, 384) and tuple(m.deltas) == (12.5, 12.5)
    assert tuple(m.shape(include_bc=True, as_grid=True)) == (1232, 464)
    assert solver.spatial_accuracy_order == 8 and solver.dtype == np.float32
    assert solver.checkpoint_every == 64
    assert len(shots) == 64 and {s.receivers.receiver_count for s in shots} == {1152}
    xs = [s.sources.position[0] for s in shots]
    assert np.allclose(np.diff(xs), np.diff(xs)[0]) and {_ricker_hz(s) for s in shots} == {8.0}
    assert 1500.0 <= C.min() and C.max() <= 5500.0 and C.max() > 4000.0
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    assert solver.nsteps == 4000


def test_3d_gradient_workload_scaled():
    """The 3D workload at a tenth of its size (its full size holds 66 M cells per field)."""
    m, shots, solver, C, C0 = workloads.cfg3(scale=0.1)
    nx, ny, nz = m.shape(as_grid=True)
    assert (nx, ny, nz) == (40, 40, 30) and tuple(m.deltas) == (15.0, 15.0, 15.0)
    assert solver.spatial_accuracy_order == 8 and solver.dtype == np.float32
    assert solver.checkpoint_every == 55  # sqrt(3000)
    assert len(shots) == 8 and {s.receivers.receiver_count for s in shots} == {min(100, nx) * min(100, ny)}
    assert {_ricker_hz(s) for s in shots} == {6.0}
    assert np.any(C == 4500.0) and 1500.0 <= C.min()  # the salt body at 4500 m/s
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    assert solver.nsteps == 3000


def test_uneven_batch_grids():
    grids = workloads.cfg4(nshots=6)
    want = [((288, 96), 50.0, 2000, 3.0), ((576, 192), 25.0, 3000, 5.0), ((1152, 384), 12.5, 4000, 8.0)]
    for (m, shots, solver, C, C0, record), (shape, dx, nsteps, hz) in zip(grids, want):
        assert tuple(m.shape(as_grid=True)) == shape and tuple(m.deltas) == (dx, dx)
        assert solver.spatial_accuracy_order == 6 and solver.dtype == np.float32
        assert len(shots) == 2 and {_ricker_hz(s) for s in shots} == {hz}
        assert {s.receivers.receiver_count for s in shots} == {shape[0]}
        solver.model_parameters = solver.ModelParameters(m, {"C": C0})
        assert solver.nsteps == nsteps
        assert np.all(record >= nsteps // 2) and np.all(record <= nsteps)
