"""Host-side mirror of the reference API (geometry, acquisition, factory, model
arithmetic) against the reference's own outputs (golden fixtures, and the live
reference where it is importable)."""
import json

import numpy as np
import pytest

import problems
import pysit_gb300 as api
from pysit_gb300.engine import default_checkpoint_every, padded_cells
from pysit_gb300.solvers.model_parameter import fold_padding


@pytest.mark.parametrize("name", list(problems.SPECS))
def test_geometry_and_operators_match_golden(name, golden):
    g = golden(name)
    m, shots, solver, C, C0 = problems.build(api, name)
    solver.model_parameters = solver.ModelParameters(m, {"C": C})
    assert solver.nsteps == int(g["nsteps_true"]) and solver.dt == float(g["dt_true"])
    for a in range(m.dim):
        p = m.parameters[a]
        for side, bc in (("l", p.lbc), ("r", p.rbc)):
            if bc.type == "pml":
                np.testing.assert_allclose(bc.sigma, g[f"sigma_{a}{side}"], rtol=0, atol=1e-12)
        axis = {1: "z", 2: "xz", 3: "xyz"}[m.dim][a]
        np.testing.assert_allclose(solver.operator_components["s" + axis], np.ravel(g[f"sigmap_{a}"]), atol=1e-12)
    cells, _, w = shots[0].sources.taps()
    order = np.argsort(cells)
    np.testing.assert_array_equal(cells[order], g["src_rows"])
    np.testing.assert_allclose(w[order], g["src_vals"], rtol=1e-15)
    rc, rr, ws, _ = shots[0].receivers.taps()
    order = np.lexsort((rc, rr))
    np.testing.assert_array_equal(rr[order], g["rec_rows"])
    np.testing.assert_array_equal(rc[order], g["rec_cols"])
    np.testing.assert_allclose(ws[order], g["rec_vals"], rtol=1e-15)
    f = problems.SPECS[name]["f"]
    np.testing.assert_allclose([api.RickerWavelet(f)(t) for t in (0.0, 0.01, 0.05, 0.1)], g["ricker"], rtol=1e-15)


def test_padded_cells_roundtrip():
    m, shots, solver, C, C0 = problems.build(api, "o6")
    u = np.arange(m.dof()).astype(float)
    pad = m.pad_array(u.reshape(-1, 1)).reshape(-1)
    cells = np.arange(m.dof())
    np.testing.assert_array_equal(pad[padded_cells(m, cells)], u)
    np.testing.assert_array_equal(m.unpad_array(pad.reshape(-1, 1)).reshape(-1), u)


def test_fold_padding_sums_strips_and_preserves_total():
    m, *_ = problems.build(api, "dirichlet")
    rng = np.random.default_rng(1)
    a = rng.standard_normal(m.dof(include_bc=True))
    f = fold_padding(m, a)
    assert f.shape == (m.dof(), 1)
    assert f.sum() == pytest.approx(a.sum(), rel=1e-12)


def test_linear_interpolation_matches_scipy():
    from scipy.interpolate import interp1d
    rng = np.random.default_rng(5)
    ts = np.arange(40) * 0.013
    d = rng.standard_normal((40, 3))
    tn = np.arange(55) * 0.0101
    ref = interp1d(ts, d, axis=0, kind="linear", bounds_error=False, fill_value=0.0)(tn)
    np.testing.assert_allclose(api.linear_interpolate(ts, d, tn), ref, rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("dim,cls", [(1, "ConstantDensityAcousticTimeScalar_1D_cuda"),
                                     (2, "ConstantDensityAcousticTimeScalar_2D_cuda"),
                                     (3, "ConstantDensityAcousticTimeScalar_3D_cuda")])
@pytest.mark.parametrize("order", [2, 4, 6, 8])
def test_factory_resolves_cuda_solvers(dim, cls, order):
    """Mirror of pysit/solvers/tests/test_factories.py:55-79 for kernel_implementation='cuda'."""
    name = {1: "1d", 2: "o6", 3: "3d"}[dim]
    m, *_ = problems.build(api, name)
    s = api.ConstantDensityAcousticWave(m, spatial_accuracy_order=order, kernel_implementation="cuda")
    assert type(s).__name__ == cls
    assert s.spatial_accuracy_order == order


def test_factory_errors():
    m, *_ = problems.build(api, "o6")
    with pytest.raises(api.NoMatchError):
        api.ConstantDensityAcousticWave(m, kernel_implementation="cpp")
    with pytest.raises(api.NoMatchError):
        api.ConstantDensityAcousticWave(m, spatial_accuracy_order=5, kernel_implementation="cuda")
    with pytest.raises(api.NoMatchError):
        api.ConstantDensityAcousticWave(m, precision="half", kernel_implementation="cuda")


def test_model_arithmetic_is_linear_in_m():
    m, shots, solver, C, C0 = problems.build(api, "o6")
    a = api.ConstantDensityAcousticParameters(m, {"C": C})
    b = api.ConstantDensityAcousticParameters(m, {"C": C0})
    d = a - b
    np.testing.assert_allclose(d.data, C.reshape(-1, 1) ** -2 - C0.reshape(-1, 1) ** -2)
    c = b + d
    np.testing.assert_allclose(c.C, a.C, rtol=1e-12)
    p = a.with_padding(padding_mode="edge")
    assert p.data.shape == (m.dof(include_bc=True), 1)
    np.testing.assert_allclose(p.without_padding().C, a.C)
    assert d.inner_product(d) == pytest.approx(float(np.sum(d.data ** 2)) * np.prod(m.deltas))


def test_default_checkpoint_interval():
    assert default_checkpoint_every(4000, 2) == 126
    assert default_checkpoint_every(3000, 3) == 134
    assert default_checkpoint_every(3, 2) == 3


def test_cuda_path_has_no_cpu_fallback(monkeypatch):
    import torch
    from pysit_gb300 import _native
    monkeypatch.setattr(torch.cuda, "is_available", lambda: False)
    with pytest.raises(_native.PysitCudaError):
        _native.require_cuda()


def test_observed_data_fingerprint_sees_in_place_edits():
    """The device copy of the recorded traces is reused while every shot holds the same array
    with the same sampled values; an in-place edit of the array changes its fingerprint."""
    from pysit_gb300.engine import _fingerprint
    rng = np.random.default_rng(0)
    a = rng.standard_normal((4000, 1152))
    fp = _fingerprint(a)
    assert _fingerprint(a) == fp
    a *= 2.0
    assert _fingerprint(a) != fp
    b = a.copy()
    b[-1, 5] += 1.0          # last row
    assert _fingerprint(b) != _fingerprint(a)
    c = a.copy()
    c.reshape(-1)[4099 * 7] += 1.0   # a sampled element
    assert _fingerprint(c) != _fingerprint(a)


def test_solver_rejects_unknown_gradient_schedule():
    d = api.RectangularDomain((0.0, 100.0, api.PML(20.0, 100.0), api.PML(20.0, 100.0)),
                              (0.0, 100.0, api.PML(20.0, 100.0), api.PML(20.0, 100.0)))
    m = api.CartesianMesh(d, 11, 11)
    with pytest.raises(ValueError):
        api.ConstantDensityAcousticWave(m, kernel_implementation="cuda", gradient_schedule="fast")
    s = api.ConstantDensityAcousticWave(m, kernel_implementation="cuda", gradient_schedule="auto")
    assert s.gradient_schedule == "auto"


def test_observed_cache_follows_the_data_arrays():
    """The device copy of recorded traces is found again for the same arrays with the same values,
    missed after an in-place edit, and released when one of the arrays is freed."""
    import gc
    from pysit_gb300.engine import _ObservedCache
    rng = np.random.default_rng(3)
    a, b = rng.standard_normal((50, 4)), rng.standard_normal((50, 4))
    cache = _ObservedCache()
    key = (id(a), id(b))
    payload = object()
    cache.put(key, payload, [a, b])
    assert cache.get(key, [a, b]) is payload
    assert cache.get(key, [a, b.copy()]) is None
    b[-1, 0] += 1.0  # the last row is part of the fingerprint
    assert cache.get(key, [a, b]) is None
    cache.put(key, payload, [a, b])
    assert cache.get(key, [a, b]) is payload
    del b
    gc.collect()
    assert cache._entry is None
    cache.put((id(a),), payload, [[1.0, 2.0]])   # not weakly referable: not cached
    assert cache._entry is None


def test_release_plans_empties_the_plan_cache():
    m, shots, solver, C, C0 = problems.build(api, "o6")
    solver._plans["key"] = object()
    solver.release_plans()
    assert solver._plans == {}


def _schedule_case(monkeypatch, nshots, free_gb, per_shot_gb, fixed=None, base_gb=1.0, nsteps=4000, nrec=1152,
                   ckpt_per_shot_gb=None):
    """WavePlan._choose_schedule with a fake device (free memory) and a linear workspace model."""
    import types
    from pysit_gb300 import _native
    from pysit_gb300.engine import WavePlan
    GB = 1 << 30
    fake_torch = types.SimpleNamespace(float64="f64", float32="f32",
                                       cuda=types.SimpleNamespace(mem_get_info=lambda: (int(free_gb * GB), 0)))
    monkeypatch.setattr(_native, "require_cuda", lambda: fake_torch)
    calls = []

    def workspace(lib, d, G, store, lanes=1):
        calls.append((G, store, lanes))
        per = per_shot_gb if store or ckpt_per_shot_gb is None else ckpt_per_shot_gb
        return int((base_gb + G * per) * GB)
    plan = types.SimpleNamespace(nshots=nshots, nsteps=nsteps, tdtype="f32", shots_per_launch=fixed or nshots,
                                 lanes=1, _workspace_for=workspace)
    sched = WavePlan._choose_schedule(plan, None, None, fixed is not None, nrec)
    return sched, plan.shots_per_launch, calls


def test_auto_schedule_takes_the_largest_balanced_launch(monkeypatch):
    # 64 shots of 9.5 GB each on 280 GB free: 27 would fit, so three balanced launches of 22
    sched, G, _ = _schedule_case(monkeypatch, 64, 280.0, 9.5)
    assert (sched, G) == ("store", 22)
    # 128 shots of the same size: five launches, ceil(128 / 5) = 26 (the end-to-end FWI's launch)
    sched, G, _ = _schedule_case(monkeypatch, 128, 280.0, 9.5)
    assert (sched, G) == ("store", 26)
    # few shots that all fit: one launch of all of them
    sched, G, _ = _schedule_case(monkeypatch, 8, 280.0, 9.5)
    assert (sched, G) == ("store", 8)


def test_auto_schedule_falls_back_to_checkpoints(monkeypatch):
    # fewer than 8 shots per launch would keep dWaveOp: the checkpointed schedule, with the
    # largest balanced launch whose checkpoints fit (21 of 2.5 GB fit beside the traces in 60 GB:
    # four launches of 16)
    sched, G, _ = _schedule_case(monkeypatch, 64, 60.0, 9.5, ckpt_per_shot_gb=2.5)
    assert (sched, G) == ("checkpoint", 16)
    # 11 shots keep dWaveOp in 120 GB: enough for the kept schedule
    sched, G, _ = _schedule_case(monkeypatch, 64, 120.0, 9.5)
    assert (sched, G) == ("store", 11)
    # a fixed launch size is kept and decides alone
    sched, G, calls = _schedule_case(monkeypatch, 64, 280.0, 9.5, fixed=32)
    assert (sched, G) == ("checkpoint", 32) and calls == [(32, True, 1)]
    sched, G, _ = _schedule_case(monkeypatch, 64, 280.0, 9.5, fixed=8)
    assert (sched, G) == ("store", 8)


def test_misfit_backward_maps_the_m_gradient_to_velocity(monkeypatch):
    """MisfitFunction's backward turns the gradient g in m = C**-2 (cell-volume inner product)
    into dJ/dC = g * dV * (-2 C**-3): checked on a misfit whose value is dV * sum(g * C**-2)."""
    import types
    import torch
    from pysit_gb300 import _native, autograd
    monkeypatch.setattr(_native, "require_cuda", lambda: torch)
    rng = np.random.default_rng(4)
    deltas = (12.5, 10.0)
    dV = float(np.prod(deltas))
    g = torch.as_tensor(rng.standard_normal((6, 5)), dtype=torch.float64)

    class Obj:
        solver = types.SimpleNamespace(mesh=types.SimpleNamespace(deltas=deltas))

        def _run(self, C, want_grad):
            J = dV * (g * C.detach().double() ** -2).sum()
            return J.to(C.dtype), (g.clone() if want_grad else None)

    C0 = torch.as_tensor(1500.0 + 500.0 * rng.random((6, 5)), dtype=torch.float64)
    C = C0.clone().requires_grad_()
    J = autograd._make_function().apply(C, Obj())
    J.backward()
    Cr = C0.clone().requires_grad_()
    (dV * (g * Cr ** -2).sum()).backward()
    torch.testing.assert_close(C.grad, Cr.grad, rtol=1e-13, atol=0)
    assert float(J.detach()) == pytest.approx(float(dV * (g * C0 ** -2).sum()), rel=1e-15)


@pytest.mark.parametrize("n_src", [1, 2, 7])
def test_resampling_arithmetic_equals_host_interpolation(monkeypatch, n_src):
    """The device resampler's arithmetic, run here on CPU tensors, against linear_interpolate
    (a single sample is kept at its own time only)."""
    import torch
    from pysit_gb300 import _native
    from pysit_gb300.autograd import resample_linear
    monkeypatch.setattr(_native, "require_cuda", lambda: torch)
    rng = np.random.default_rng(n_src)
    ts_src = 0.004 * np.arange(n_src) + 0.002
    ts_new = np.concatenate([[-0.003, 0.0, ts_src[0]], 0.0035 * np.arange(1, 9), [ts_src[-1], 0.2]])
    data = rng.standard_normal((3, n_src, 5))
    want = np.stack([api.linear_interpolate(ts_src, d, ts_new) for d in data])
    got = resample_linear(torch.as_tensor(data), ts_src, ts_new).numpy()
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-15)


def test_device_edge_padding_equals_numpy(monkeypatch):
    import torch
    from pysit_gb300 import _native
    from pysit_gb300.autograd import _edge_pad
    monkeypatch.setattr(_native, "require_cuda", lambda: torch)
    for name in ("o6", "dirichlet", "3d", "1d"):
        m, *_ = problems.build(api, name)
        shape = tuple(m.shape(as_grid=True))
        a = np.random.default_rng(0).standard_normal(shape)
        pads = [(m.parameters[k].lbc.n, m.parameters[k].rbc.n) for k in range(m.dim)]
        np.testing.assert_array_equal(_edge_pad(torch.as_tensor(a), m).numpy(), np.pad(a, pads, mode="edge"))


def test_fwi_misfit_checks_the_observed_data_shape():
    import torch
    from pysit_gb300.autograd import FWIMisfit
    m, shots, solver, C, C0 = problems.build(api, "o2")
    nrec = shots[0].receivers.receiver_count
    ts = np.arange(50) * 1e-3
    FWIMisfit(solver, shots, torch.zeros((len(shots), 50, nrec)), ts)
    for bad in ((len(shots) + 1, 50, nrec), (len(shots), 49, nrec), (len(shots), 50, nrec + 1),
                (len(shots), 50, nrec - 1), (50, nrec)):
        with pytest.raises(ValueError):
            FWIMisfit(solver, shots, torch.zeros(bad), ts)


def test_tuning_cache_file_round_trip(monkeypatch, tmp_path):
    """PYSIT_CUDA_TUNE_CACHE: a tuning written by one process is found by the next; an
    unreadable file is ignored; without the variable nothing is written."""
    from pysit_gb300 import engine
    key = (2, 8, (1232, 464), str(np.float32), 0, np.int64(22), "store", False, 1)
    value = (16, (0.25, 0.3, 0.35), 96)
    path = tmp_path / "tunings.json"
    monkeypatch.setattr(engine, "_TUNED", {})
    monkeypatch.setattr(engine, "_TUNE_FILES_READ", set())
    monkeypatch.delenv("PYSIT_CUDA_TUNE_CACHE", raising=False)
    engine._tuning_put(key, value)
    assert not path.exists() and engine._tuning_get(key) == value
    monkeypatch.setenv("PYSIT_CUDA_TUNE_CACHE", str(path))
    engine._tuning_put(key, value)
    assert path.exists()
    # a later process: empty in-memory table, same file
    monkeypatch.setattr(engine, "_TUNED", {})
    monkeypatch.setattr(engine, "_TUNE_FILES_READ", set())
    assert engine._tuning_get(key) == value
    assert engine._tuning_get(key[:-1] + (2,)) is None
    # a file written before z extents were tuned: rows of three entries read as the full width
    path.write_text(json.dumps([[repr(engine._plain_key(key)), 16, [0.25, 0.3, 0.35]]]))
    monkeypatch.setattr(engine, "_TUNED", {})
    monkeypatch.setattr(engine, "_TUNE_FILES_READ", set())
    assert engine._tuning_get(key) == (16, (0.25, 0.3, 0.35), 0)
    path.write_text("not json")
    monkeypatch.setattr(engine, "_TUNED", {})
    monkeypatch.setattr(engine, "_TUNE_FILES_READ", set())
    assert engine._tuning_get(key) is None
