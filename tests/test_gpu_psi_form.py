"""The batched 3D path with pml_psi='consistent' against the oracle's consistent form,
on the 3D problem with a realistic PML amplitude (where the reference's own form
diverges): traces, gradient and misfit, FP64 and FP32."""
import os
import sys

import numpy as np
import pytest

import problems
import pysit_gb300 as api

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import pipeline  # noqa: E402

pytestmark = pytest.mark.gpu

STRONG = dict(pml=(4, 160.0))


def _rel(a, b):
    a, b = np.asarray(a, float).reshape(-1), np.asarray(b, float).reshape(-1)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def oracle_run():
    m, shots, solver, C, C0 = problems.build(api, "3d", spec_overrides=STRONG)
    try:
        pipeline.set_psi_consistent(True)
        solver.model_parameters = solver.ModelParameters(m, {"C": C})
        traces = [pipeline.forward(problems.oracle_problem(solver, s))[0] for s in shots]
        ts_true = solver.ts()
        solver.model_parameters = solver.ModelParameters(m, {"C": C0})
        ts0 = solver.ts()
        # observed data on the starting model's time axis: linear, zero outside (interp1d semantics)
        dobs = [np.stack([np.interp(ts0, ts_true, tr[:, r], left=0.0, right=0.0) for r in range(tr.shape[1])],
                         axis=1) for tr in traces]
        Ps = [problems.oracle_problem(solver, s) for s in shots]
        grad, r2 = pipeline.gradient(Ps, dobs)
    finally:
        pipeline.set_psi_consistent(False)
    return dict(traces=traces, dobs=dobs, grad=grad, r2=r2, dt0=solver.dt)


@pytest.mark.parametrize("precision,tr_tol,g_tol", [("double", 1e-11, 1e-9), ("single", 1e-4, 1e-3)])
def test_consistent_psi_form_matches_the_oracle(oracle_run, precision, tr_tol, g_tol):
    import torch
    from pysit_gb300.engine import WavePlan
    m, shots, solver, C, C0 = problems.build(api, "3d", precision=precision, spec_overrides=STRONG,
                                             pml_psi="consistent")
    solver.model_parameters = solver.ModelParameters(m, {"C": C})
    plan = WavePlan(solver, shots)
    traces = plan.forward().double().cpu().numpy()
    assert plan.status() == 0
    for s, ref in enumerate(oracle_run["traces"]):
        assert _rel(traces[s], ref) < tr_tol
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    assert solver.dt == pytest.approx(oracle_run["dt0"], rel=1e-15)
    plan = WavePlan(solver, shots)
    plan.dobs.copy_(torch.as_tensor(np.stack(oracle_run["dobs"])))
    g, rn = plan.gradient()
    assert plan.status() == 0
    assert _rel(g.cpu().numpy(), oracle_run["grad"]) < g_tol
    assert float(rn) == pytest.approx(oracle_run["r2"], rel=max(tr_tol * 10, 1e-10))
