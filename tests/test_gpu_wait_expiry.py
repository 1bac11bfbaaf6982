"""Bounded device waits: a wait that runs out is reported and leaves the device usable.

The 2D step kernels wait on mbarriers for the bulk copies that fill their shared-memory
rows, each wait bounded.  A plan built with ``wait_fault=True`` (a test aid) makes every task
first wait, with ``wait_polls`` = 1 non-blocking test, on a barrier on which nothing ever
arrives: the wait runs out with the task's copies in flight.  The warp then waits (with the
full limit) for those copies, stops taking tasks and sets bit 0 of the plan's status word.
Nothing faults or hangs; the results of that run are invalid, the host layer raises
PYSIT_ETIMEOUT, and a plan with the default limits on the same device then matches the
oracle again.
"""
import numpy as np
import pytest

import pipeline
import problems
import pysit_gb300 as api
from pysit_gb300 import _native
from pysit_gb300.engine import WavePlan

pytestmark = pytest.mark.gpu


def _problem():
    m, shots, solver, C, C0 = problems.build(api, "o8")
    api.generate_seismic_data(shots, solver, solver.ModelParameters(m, {"C": C}))
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    return m, shots, solver


def test_expired_wait_sets_the_status_and_the_host_raises():
    m, shots, solver = _problem()
    plan = WavePlan(solver, shots, wait_polls=1, wait_fault=True, use_graph=False)
    plan.load_observed()
    plan.gradient()
    assert plan.status() & 1  # a wait expired (the status word is cleared by the read)
    plan.gradient()
    with pytest.raises(_native.PysitCudaError, match="expired") as e:
        plan.check_status()
    assert e.value.code == _native.PYSIT_ETIMEOUT
    assert plan.status() == 0  # check_status cleared the word


def test_default_limit_after_an_expiry_matches_the_oracle():
    m, shots, solver = _problem()
    bad = WavePlan(solver, shots, wait_polls=1, wait_fault=True, use_graph=False)
    bad.load_observed()
    bad.gradient()
    assert bad.status() & 1
    del bad
    plan = WavePlan(solver, shots)
    plan.load_observed()
    g, rn = plan.gradient()
    assert plan.check_status() == 0
    P = [problems.oracle_problem(solver, s) for s in shots]
    dobs = [s.receivers.interpolate_data(solver.ts()) for s in shots]
    ref_g, ref_rn = pipeline.gradient(P, dobs)
    g = g.cpu().numpy()
    assert np.linalg.norm(g - ref_g) <= 1e-9 * np.linalg.norm(ref_g)
