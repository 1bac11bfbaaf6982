"""GPU parity of the modelling / gradient pipeline against the reference.

Reference outputs come from tests/golden/ (the unmodified reference run with
kernel_implementation='cpp', FP64) and from the CPU oracle (pinned to the same
reference).  Tolerances (relative L2):
  FP64  traces <= 1e-11, gradient <= 1e-9, objective <= 1e-10
  FP32  traces <= 1e-4,  gradient <= 1e-3 (against the FP64 reference)
"""
import numpy as np
import pytest

import pipeline
import problems
import pysit_gb300 as api

pytestmark = pytest.mark.gpu

NAMES_2D = ["cfg1", "o2", "o6", "o8", "dirichlet"]
NAMES_ALL = NAMES_2D + ["1d", "3d", "3d_o8"]


def _rel(a, b):
    a, b = np.ravel(np.asarray(a, float)), np.ravel(np.asarray(b, float))
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _setup(name, g, precision="double", **solver_kw):
    m, shots, solver, C, C0 = problems.build(api, name, precision=precision)
    for k, v in solver_kw.items():
        setattr(solver, k, v)
    ts_true = np.arange(int(g["nsteps_true"])) * float(g["dt_true"])
    for s, d in zip(shots, g["traces"]):
        s.reset_time_series(ts_true)
        s.receivers.data[:] = d
    return m, shots, solver, C, C0


@pytest.mark.parametrize("name", NAMES_ALL)
def test_generate_seismic_data_matches_reference(name, golden):
    g = golden(name)
    m, shots, solver, C, C0 = problems.build(api, name)
    api.generate_seismic_data(shots, solver, solver.ModelParameters(m, {"C": C}))
    assert solver.nsteps == int(g["nsteps_true"])
    tr = np.stack([s.receivers.data for s in shots])
    assert _rel(tr, g["traces"]) < 1e-11


@pytest.mark.parametrize("name", NAMES_ALL)
def test_batched_gradient_matches_reference(name, golden):
    g = golden(name)
    m, shots, solver, C, C0 = _setup(name, g)
    obj = api.TemporalLeastSquares(solver)
    aux = {"objective_value": (True, None), "residual_norm": (True, None)}
    grad = obj.compute_gradient(shots, solver.ModelParameters(m, {"C": C0}), aux)
    assert solver.nsteps == int(g["nsteps0"])
    assert _rel(grad.data, g["grad"]) < 1e-9
    assert aux["objective_value"][1] == pytest.approx(float(g["objective"]), rel=1e-10)
    assert aux["residual_norm"][1] == pytest.approx(float(g["residual_norm"]), rel=1e-10)
    assert obj.evaluate(shots, solver.ModelParameters(m, {"C": C0})) == pytest.approx(float(g["objective"]),
                                                                                        rel=1e-10)


@pytest.mark.parametrize("name", ["cfg1", "o8", "1d", "3d"])
def test_plain_per_shot_gradient_matches_reference(name, golden):
    g = golden(name)
    m, shots, solver, C, C0 = _setup(name, g)
    obj = api.TemporalLeastSquares(solver, batched=False)
    aux = {"objective_value": (True, None)}
    grad = obj.compute_gradient(shots, solver.ModelParameters(m, {"C": C0}), aux)
    assert _rel(grad.data, g["grad"]) < 1e-10
    assert aux["objective_value"][1] == pytest.approx(float(g["objective"]), rel=1e-10)


@pytest.mark.parametrize("name", NAMES_2D + ["3d"])
def test_fp32_batched_gradient_within_tolerance(name, golden):
    g = golden(name)
    m, shots, solver, C, C0 = problems.build(api, name, precision="single")
    api.generate_seismic_data(shots, solver, solver.ModelParameters(m, {"C": C}))
    tr = np.stack([s.receivers.data for s in shots])
    assert _rel(tr, g["traces"]) < 1e-4
    m, shots, solver, C, C0 = _setup(name, g, precision="single")
    grad = api.TemporalLeastSquares(solver).compute_gradient(shots, solver.ModelParameters(m, {"C": C0}))
    assert _rel(grad.data, g["grad"]) < 1e-3


@pytest.mark.parametrize("name,p", [("o6", 2), ("o6", 3), ("3d", 2)])
def test_imaging_period_matches_reference(name, p, golden):
    """Imaging every p steps: the reference's own gradient (tests/golden/period<p>_<name>.npz)
    and the oracle's."""
    g = golden(name)
    m, shots, solver, C, C0 = _setup(name, g)
    aux = {"objective_value": (True, None)}
    grad = api.TemporalLeastSquares(solver, imaging_period=p).compute_gradient(
        shots, solver.ModelParameters(m, {"C": C0}), aux)
    gp = golden(f"period{p}_{name}")
    assert _rel(grad.data, gp["grad"]) < 1e-9
    assert aux["objective_value"][1] == pytest.approx(float(gp["objective"]), rel=1e-10)
    Ps = [problems.oracle_problem(solver, s) for s in shots]
    dobs = [s.receivers.interpolate_data(solver.ts()) for s in shots]
    ref, _ = pipeline.gradient(Ps, dobs, imaging_period=p)
    assert _rel(grad.data, ref) < 1e-9


@pytest.mark.parametrize("kw", [dict(checkpoint_every=1), dict(checkpoint_every=7), dict(checkpoint_every=10 ** 6),
                                dict(shots_per_launch=1), dict(use_graph=False)])
def test_schedule_variants_agree(kw, golden):
    g = golden("o8")
    m, shots, solver, C, C0 = _setup("o8", g, **kw)
    grad = api.TemporalLeastSquares(solver).compute_gradient(shots, solver.ModelParameters(m, {"C": C0}))
    assert _rel(grad.data, g["grad"]) < 1e-9


def test_migrate_batched_equals_plain(golden):
    """Both migration paths against each other and against the reference's migrate_shot of the
    same operand (tests/golden/mig_o6.npz)."""
    g = golden("o6")
    m, shots, solver, C, C0 = _setup("o6", g)
    m0 = solver.ModelParameters(m, {"C": C0})
    solver.model_parameters = m0
    f = golden("mig_o6")
    op = f["operand"]
    assert op.shape == (solver.nsteps, shots[0].receivers.receiver_count)
    a = api.TemporalModeling(solver, batched=True).migrate_shot(shots[0], m0, op, 1)
    b = api.TemporalModeling(solver, batched=False).migrate_shot(shots[0], m0, op, 1)
    assert _rel(a.data, b.data) < 1e-10
    assert _rel(a.data, f["image_p1"]) < 1e-9
    assert _rel(b.data, f["image_p1"]) < 1e-9


def test_forward_model_outputs_match_oracle(golden):
    g = golden("o2")
    m, shots, solver, C, C0 = problems.build(api, "o2")
    m1 = solver.ModelParameters(m, {"C": C})
    tm = api.TemporalModeling(solver)
    rv = tm.forward_model(shots[0], m1, 1, ["simdata", "dWaveOp", "wavefield"])
    P = problems.oracle_problem(solver, shots[0])
    sim, dws = pipeline.forward(P, want_dwaveop=True)
    assert _rel(rv["simdata"], sim) < 1e-11
    assert len(rv["dWaveOp"]) == len(dws)
    assert _rel(np.stack([d.reshape(-1) for d in rv["dWaveOp"]]), np.stack(dws)) < 1e-10
    assert len(rv["wavefield"]) == solver.nsteps
    fast = tm.forward_model(shots[0], m1, 1, ["simdata"])["simdata"]
    assert _rel(fast, sim) < 1e-11
    # the reference's own forward_model snapshots (unpadded wavefield, padded dWaveOp)
    f = golden("fwd_o2")
    ks = f["steps"]
    assert _rel(np.stack([np.ravel(rv["wavefield"][k]) for k in ks]), f["wavefield"]) < 1e-11
    assert _rel(np.stack([np.ravel(rv["dWaveOp"][k]) for k in ks]), f["dwaveop"]) < 1e-10


def test_time_step_on_host_solver_data_matches_oracle():
    """The reference-compatible per-step protocol (numpy SolverData) on the GPU kernel."""
    m, shots, solver, C, C0 = problems.build(api, "o6")
    solver.model_parameters = solver.ModelParameters(m, {"C": C})
    P = problems.oracle_problem(solver, shots[0])
    sd = solver.SolverData()
    rng = np.random.default_rng(9)
    dof = m.dof(include_bc=True)
    sd.k.data[:] = rng.standard_normal((sd.k.data.shape[0], 1)) * 1e-3
    sd.km1.u[:] = rng.standard_normal((dof, 1)) * 1e-3
    rhs = rng.standard_normal((dof, 1))
    solver.time_step(sd, rhs, None)
    aux = {"Phix": sd.k.Phix.reshape(-1), "Phiz": sd.k.Phiz.reshape(-1)}
    ref_u, ref_aux = pipeline.step("oracle", 2, P["order"], sd.km1.u.reshape(-1), aux, sd.k.u.reshape(-1), P["C"],
                                   rhs.reshape(-1), P["profiles"], P["dt"], P["deltas"], P["shape"])
    assert _rel(sd.kp1.u, ref_u) < 1e-13
    assert _rel(sd.kp1.Phix, ref_aux["Phix"]) < 1e-13
    dW = solver.compute_dWaveOp("time", sd)
    ref_dw = pipeline.dwaveop(P, sd.km1.u.reshape(-1), sd.k.u.reshape(-1), sd.kp1.u.reshape(-1), None)
    assert _rel(dW, ref_dw) < 1e-12


def test_plan_reports_its_kernel_launches(golden):
    g = golden("o6")
    m, shots, solver, C, C0 = _setup("o6", g)
    obj = api.TemporalLeastSquares(solver)
    obj.compute_gradient(shots, solver.ModelParameters(m, {"C": C0}))
    n = obj.last_plan.launches()
    assert n >= 3 * solver.nsteps


def test_status_word_clear_after_stable_run_and_flags_instability():
    from pysit_gb300.engine import WavePlan
    m, shots, solver, C, C0 = problems.build(api, "o6")
    solver.model_parameters = solver.ModelParameters(m, {"C": C})
    plan = WavePlan(solver, shots)
    plan.forward()
    assert plan.status() == 0
    # far beyond the leapfrog stability limit: after enough steps the wavefield
    # overflows and the forward sweep reports non-finite values
    m, shots, solver, C, C0 = problems.build(api, "o6")
    solver.cfl_safety = 3.0
    solver.trange = (0.0, 30.0)
    solver.t0, solver.tf = solver.trange
    solver.model_parameters = solver.ModelParameters(m, {"C": C})
    plan = WavePlan(solver, shots)
    plan.forward()
    assert plan.status() & 2
    assert plan.status() == 0  # reading clears the word


@pytest.mark.parametrize("name", ["o8", "3d"])
def test_autotuned_tiles_keep_the_gradient(name, golden):
    """The autotuner rebuilds the task table with the fastest (x length, interior z extent) pair;
    the gradient is unchanged, also with interior tasks 16 cells deep (several z-segments)."""
    from pysit_gb300.engine import WavePlan
    g = golden(name)
    m, shots, solver, C, C0 = _setup(name, g)
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    plan = WavePlan(solver, shots)
    plan.load_observed()
    res = plan.autotune(candidates=(8, 16, 48), nsteps=4, z_candidates=(0, 16))
    assert res["chosen"] in (8, 16, 48) and res["chosen_z"] in (0, 16)
    assert len(res["ms"]) == 6 and all(v > 0 for v in res["ms"].values())
    grad, rn = plan.gradient()
    assert plan.status() == 0
    assert _rel(grad.cpu().numpy(), g["grad"]) < 1e-9
    res = plan.autotune(candidates=(16,), nsteps=2, z_candidates=(16,))
    assert (res["chosen"], res["chosen_z"]) == (16, 16)
    grad, rn = plan.gradient()
    assert plan.status() == 0
    assert _rel(grad.cpu().numpy(), g["grad"]) < 1e-9
