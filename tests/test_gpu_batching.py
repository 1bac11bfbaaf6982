"""Uneven batches: per-shot record lengths inside one plan, and plans of different grids
run together as one group (one CUDA graph)."""
import numpy as np
import pytest

import problems
import pysit_gb300 as api

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a, float).reshape(-1), np.asarray(b, float).reshape(-1)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _observed(name, **overrides):
    m, shots, solver, C, C0 = problems.build(api, name, spec_overrides=overrides or None)
    api.generate_seismic_data(shots, solver, solver.ModelParameters(m, {"C": C}))
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    return m, shots, solver, C, C0


def test_shorter_record_equals_a_run_of_that_length():
    from pysit_gb300.engine import WavePlan
    m, shots, solver, C, C0 = _observed("o8")
    assert len(shots) == 2
    N, dt = solver.nsteps, solver.dt
    n_short = N - 20
    plan = WavePlan(solver, shots, record_steps=[N, n_short])
    plan.load_observed()
    g_mix, rn_mix = (t.cpu().numpy().copy() for t in plan.gradient())
    # shot 0 over the whole record
    full = WavePlan(solver, shots[:1])
    full.load_observed()
    g0, rn0 = (t.cpu().numpy().copy() for t in full.gradient())
    # shot 1 with a solver whose time range ends at its record length
    m2, shots2, solver2, C_, C0_ = problems.build(api, "o8", spec_overrides=dict(T=(n_short - 0.5) * dt))
    solver2.model_parameters = solver2.ModelParameters(m2, {"C": C0})
    assert solver2.dt == dt and solver2.nsteps == n_short
    s1 = shots[1]
    short = WavePlan(solver2, [s1])
    short.load_observed()
    g1, rn1 = (t.cpu().numpy().copy() for t in short.gradient())
    assert _rel(g_mix, g0 + g1) < 1e-10
    assert float(rn_mix[0]) == pytest.approx(float(rn0[0] + rn1[0]), rel=1e-10)
    assert plan.status() == 0


def test_plan_group_matches_its_plans():
    from pysit_gb300.engine import PlanGroup, WavePlan
    plans, ref = [], []
    for name in ("o8", "o6"):
        m, shots, solver, C, C0 = _observed(name)
        p = WavePlan(solver, shots)
        p.load_observed()
        g, rn = p.gradient()
        ref.append((g.cpu().numpy().copy(), float(rn.item())))
        plans.append(p)
    group = PlanGroup(plans)
    for _ in range(2):  # the second call replays the cached graph
        for p in plans:
            p.grad.zero_()
            p.rnorm2.zero_()
        out = group.gradient()
        for (g, rn), (g_ref, rn_ref) in zip(out, ref):
            assert _rel(g.cpu().numpy(), g_ref) < 1e-12
            assert float(rn.item()) == pytest.approx(rn_ref, rel=1e-12)
