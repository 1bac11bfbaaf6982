"""Source-encoded supershots on the GPU: a supershot is one shot of the batched plan with one
injection point per member source.  Checks (FP64 unless stated):
  traces    = sum_i code_i * traces of member i (plan) and = the oracle's supershot traces, 1e-11
  gradient  = the oracle's gradient of the supershot misfit, 1e-9 (FP32: 1e-3)
  re-encoding builds a new plan whose traces follow the new codes.
"""
import numpy as np
import pytest

import pipeline
import problems
import pysit_gb300 as api
from pysit_gb300.engine import WavePlan

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.ravel(np.asarray(a, float)), np.ravel(np.asarray(b, float))
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _observed(name, precision="double", spec_overrides=None):
    m, shots, solver, C, C0 = problems.build(api, name, precision=precision, spec_overrides=spec_overrides)
    api.generate_seismic_data(shots, solver, solver.ModelParameters(m, {"C": C}))
    return m, shots, solver, C, C0


@pytest.mark.parametrize("name", ["o2", "o8"])
def test_supershot_traces_are_the_encoded_sum(name):
    m, shots, solver, C, C0 = _observed(name)
    ss = api.SourceEncodedSupershot(shots, rng=np.random.default_rng(4))
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    tr_ss = WavePlan(solver, [ss]).forward()[0].double().cpu().numpy()
    tr = WavePlan(solver, shots).forward().double().cpu().numpy()
    expect = np.tensordot(ss.codes, tr, axes=1)
    assert _rel(tr_ss, expect) < 1e-11
    oracle = pipeline.forward(problems.oracle_problem(solver, ss))[0]
    assert _rel(tr_ss[:, :oracle.shape[1]], oracle) < 1e-11


@pytest.mark.parametrize("precision,tol", [("double", 1e-9), ("single", 1e-3)])
def test_supershot_gradient_matches_the_oracle(precision, tol):
    m, shots, solver, C, C0 = _observed("o8", precision)
    ss = api.SourceEncodedSupershot(shots, weight_type="krebs", rng=np.random.default_rng(2))
    m0 = solver.ModelParameters(m, {"C": C0})
    aux = {"objective_value": (True, None)}
    g = api.TemporalLeastSquares(solver).compute_gradient([ss], m0, aux)
    solver.model_parameters = m0
    P = problems.oracle_problem(solver, ss)
    grad, r2 = pipeline.gradient([P], [ss.receivers.interpolate_data(solver.ts())])
    assert _rel(g.data, grad) < tol
    assert aux["objective_value"][1] == pytest.approx(0.5 * r2 * solver.dt, rel=10 * tol)


def test_reencoding_builds_a_new_plan():
    m, shots, solver, C, C0 = _observed("o2")
    ss = api.SourceEncodedSupershot(shots, rng=np.random.default_rng(5))
    m0 = solver.ModelParameters(m, {"C": C0})
    tm = api.TemporalModeling(solver)
    d_a = tm.forward_model(ss, m0, return_parameters=["simdata"])["simdata"]
    codes_a = ss.codes.copy()
    ss.encode()
    d_b = tm.forward_model(ss, m0, return_parameters=["simdata"])["simdata"]
    tr = WavePlan(solver, shots).forward().double().cpu().numpy()
    nrec = shots[0].receivers.receiver_count
    assert _rel(d_a, np.tensordot(codes_a, tr, axes=1)[:, :nrec]) < 1e-11
    assert _rel(d_b, np.tensordot(ss.codes, tr, axes=1)[:, :nrec]) < 1e-11


def test_several_supershots_in_one_plan():
    """Eight supershots of the same eight shots with independent codes, as one batch."""
    spec = dict(nsrc=8)
    m, shots, solver, C, C0 = _observed("o8", spec_overrides=spec)
    rng = np.random.default_rng(6)
    sss = [api.SourceEncodedSupershot(shots, rng=rng) for _ in range(8)]
    m0 = solver.ModelParameters(m, {"C": C0})
    g = api.TemporalLeastSquares(solver).compute_gradient(sss, m0)
    solver.model_parameters = m0
    Ps = [problems.oracle_problem(solver, s) for s in sss]
    grad, _ = pipeline.gradient(Ps, [s.receivers.interpolate_data(solver.ts()) for s in sss])
    assert _rel(g.data, grad) < 1e-9
