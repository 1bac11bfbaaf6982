"""Edge cases of the batched path against the oracle and the host code.

- The device resampling of observed traces equals the host's linear_interpolate (the restated
  interp1d of ReceiverBase.interpolate_data, receivers.py:75-105) for series of one, two and
  seven samples, with target times before, inside and past the series.
- Records of one, two and three steps: the batched FP64 gradient and objective under both
  gradient schedules equal the oracle's (relative L2 <= 1e-9, objective <= 1e-10).
"""
import numpy as np
import pytest

import pipeline
import problems
import pysit_gb300 as api

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.ravel(np.asarray(a, float)), np.ravel(np.asarray(b, float))
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("n_src", [1, 2, 7])
def test_device_resampling_equals_host_interpolation(n_src):
    import torch
    from pysit_gb300.autograd import resample_linear
    rng = np.random.default_rng(n_src)
    ts_src = 0.004 * np.arange(n_src) + 0.002
    ts_new = np.concatenate([[-0.003, 0.0, ts_src[0]], 0.0035 * np.arange(1, 9), [ts_src[-1], 0.2]])
    data = rng.standard_normal((3, n_src, 5))
    host = np.stack([api.linear_interpolate(ts_src, d, ts_new) for d in data])
    dev = resample_linear(torch.as_tensor(data, device="cuda"), ts_src, ts_new).cpu().numpy()
    assert dev.shape == host.shape
    np.testing.assert_allclose(dev, host, rtol=1e-13, atol=1e-15)
    if n_src == 1:
        assert np.count_nonzero(dev) == 2 * data.shape[0] * data.shape[2]  # t = ts_src[0] listed twice


def _short_record(nsteps, schedule):
    m, shots, solver, C, C0 = problems.build(api, "o6")
    dt0 = solver.cfl_safety * min(m.deltas) / float(np.max(C0))
    m, shots, solver, C, C0 = problems.build(api, "o6", spec_overrides=dict(T=(nsteps - 0.5) * dt0),
                                             gradient_schedule=schedule)
    m0 = solver.ModelParameters(m, {"C": C0})
    solver.model_parameters = m0
    assert solver.nsteps == nsteps
    rng = np.random.default_rng(nsteps)
    for s in shots:
        s.reset_time_series(solver.ts())
        s.receivers.data[:] = rng.standard_normal(s.receivers.data.shape)
    return m, shots, solver, m0


@pytest.mark.parametrize("schedule", ["checkpoint", "store"])
@pytest.mark.parametrize("nsteps", [1, 2, 3])
def test_records_of_a_few_steps_match_the_oracle(nsteps, schedule):
    m, shots, solver, m0 = _short_record(nsteps, schedule)
    obj = api.TemporalLeastSquares(solver)
    aux = {"objective_value": (True, None)}
    grad = obj.compute_gradient(shots, m0, aux)
    Ps = [problems.oracle_problem(solver, s) for s in shots]
    dobs = [s.receivers.interpolate_data(solver.ts()) for s in shots]
    ref, r2 = pipeline.gradient(Ps, dobs)
    assert np.all(np.isfinite(grad.data))
    if np.linalg.norm(ref) > 0:
        assert _rel(grad.data, ref) < 1e-9
    else:  # one step: the field that meets the residual is still zero
        assert np.linalg.norm(grad.data) == 0
    assert aux["objective_value"][1] == pytest.approx(0.5 * solver.dt * r2, rel=1e-10)
