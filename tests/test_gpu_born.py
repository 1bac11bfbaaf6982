"""GPU parity of Born modelling, the Hessian applications and Gauss-Newton against the
reference (fixtures tests/golden/born_<problem>.npz of the unmodified reference) and the
CPU oracle pinned to it.  Tolerances (relative L2):
  FP64  Born traces <= 1e-11, Hessian <= 1e-9
  FP32  Born traces <= 1e-4,  Hessian <= 1e-3 (against the FP64 reference)
"""
import numpy as np
import pytest

import pipeline
import problems
import pysit_gb300 as api
from pysit_gb300.engine import WavePlan

pytestmark = pytest.mark.gpu

BORN_PROBLEMS = ["o2", "o8", "1d", "3d"]


def _rel(a, b):
    a, b = np.ravel(np.asarray(a, float)), np.ravel(np.asarray(b, float))
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _setup(name, golden, precision="double", **solver_kw):
    g, b = golden(name), golden(f"born_{name}")
    m, shots, solver, C, C0 = problems.build(api, name, precision=precision, **solver_kw)
    ts_true = np.arange(int(g["nsteps_true"])) * float(g["dt_true"])
    for s, d in zip(shots, g["traces"]):
        s.reset_time_series(ts_true)
        s.receivers.data[:] = d
    m0 = solver.ModelParameters(m, {"C": C0})
    solver.model_parameters = m0
    m1 = m0.perturbation(data=b["m1"].reshape(-1, 1))
    return b, m, shots, solver, m0, m1


@pytest.mark.parametrize("precision,tol", [("double", 1e-11), ("single", 1e-4)])
@pytest.mark.parametrize("name", BORN_PROBLEMS)
def test_batched_born_matches_reference(name, precision, tol, golden):
    b, m, shots, solver, m0, m1 = _setup(name, golden, precision)
    plan = WavePlan(solver, shots)
    d1 = plan.born(m1).double().cpu().numpy()
    nrec = shots[0].receivers.receiver_count
    assert _rel(d1[:, :, :nrec], b["d1"]) < tol
    assert plan.status() == 0


@pytest.mark.parametrize("precision,tol", [("double", 1e-9), ("single", 1e-3)])
@pytest.mark.parametrize("name", BORN_PROBLEMS)
def test_batched_hessian_matches_reference(name, precision, tol, golden):
    b, m, shots, solver, m0, m1 = _setup(name, golden, precision)
    obj = api.TemporalLeastSquares(solver)
    h = obj.apply_hessian(shots, m0, m1, "approximate")
    assert _rel(h.data, b["hess_approximate"]) < tol
    mu = float(b["levenberg_mu"])
    hl = obj.apply_hessian(shots, m0, m1, "levenberg", levenberg_mu=mu)
    assert _rel(hl.data, b["hess_levenberg"]) < tol


@pytest.mark.parametrize("name", ["o2", "o8"])
def test_hessian_over_several_shot_groups(name, golden):
    """One shot per launch: every group runs its own Born sweep and migration."""
    b, m, shots, solver, m0, m1 = _setup(name, golden)
    assert len(shots) == 2
    plan = WavePlan(solver, shots, shots_per_launch=1, checkpoint_every=7)
    h, d1n = plan.hessian(m1)
    assert _rel(h.cpu().numpy(), b["hess_approximate"]) < 1e-9
    assert float(d1n.item()) == pytest.approx(float(np.sum(b["d1"] ** 2)), rel=1e-10)


@pytest.mark.parametrize("name", ["o2", "1d", "3d"])
def test_plain_path_hessian_modes_match_reference(name, golden):
    """apply_hessian step by step on the device (batched=False), all three modes."""
    b, m, shots, solver, m0, m1 = _setup(name, golden)
    obj = api.TemporalLeastSquares(solver, batched=False)
    mu = float(b["levenberg_mu"])
    for mode in ("approximate", "levenberg", "full"):
        h = obj.apply_hessian(shots, m0, m1, mode, levenberg_mu=mu)
        assert _rel(h.data, b[f"hess_{mode}"]) < 1e-9, mode


def test_full_hessian_batched_objective_falls_back_to_the_plain_loop(golden):
    b, m, shots, solver, m0, m1 = _setup("o8", golden)
    h = api.TemporalLeastSquares(solver).apply_hessian(shots, m0, m1, "full")
    assert _rel(h.data, b["hess_full"]) < 1e-9


@pytest.mark.parametrize("name", ["o2", "3d"])
def test_linear_forward_model_outputs(name, golden):
    """linear_forward_model: batched 'simdata', and the step-by-step path with dWaveOp0 given
    (from forward_model) and the dWaveOp outputs, against the reference and the oracle."""
    b, m, shots, solver, m0, m1 = _setup(name, golden)
    tm = api.TemporalModeling(solver)
    d1 = tm.linear_forward_model(shots[0], m0, m1, ["simdata"])["simdata"]
    assert _rel(d1, b["d1"][0]) < 1e-11
    dw0 = tm.forward_model(shots[0], m0, return_parameters=["dWaveOp"])["dWaveOp"]
    rv = tm.linear_forward_model(shots[0], m0, m1, ["simdata", "dWaveOp0", "dWaveOp1", "wavefield1"],
                                 dWaveOp0=dw0)
    assert _rel(rv["simdata"], b["d1"][0]) < 1e-11
    P = problems.oracle_problem(solver, shots[0])
    sim, dws, dw1 = pipeline.born(P, b["m1"], want_dwaveop1=True)
    assert _rel(np.stack(rv["dWaveOp0"]), np.stack(dws)) < 1e-11
    assert _rel(np.stack(rv["dWaveOp1"]), np.stack(dw1)) < 1e-10
    assert len(rv["wavefield1"]) == solver.nsteps
    rv2 = tm.linear_forward_model(shots[0], m0, m1, ["simdata", "dWaveOp0"])  # dWaveOp0 computed on the fly
    assert _rel(rv2["simdata"], b["d1"][0]) < 1e-11
    assert _rel(np.stack(rv2["dWaveOp0"]), np.stack(dws)) < 1e-11


def test_born_is_linear_and_adjoint_to_migration_at_size():
    """Size-independent properties on a 2D grid of 400 x 160 cells, 8 shots, FP64:
    F(2 m1) = 2 F(m1), and <F m1, d> = <m1, F* d> dV / dt with F* = migrate."""
    import torch
    mesh_spec = dict(n=(400, 160), L=(3990.0, 1590.0), pml=(20, 120.0), T=0.6, nsrc=8, nrec=200,
                     sdepth=20.0, rdepth=10.0, f=10.0, cfl=0.3, order=8)
    m, shots, solver, C, C0 = problems.build(api, "o8", spec_overrides=mesh_spec)
    m0 = solver.ModelParameters(m, {"C": C0})
    solver.model_parameters = m0
    plan = WavePlan(solver, shots, shots_per_launch=4)
    rng = np.random.default_rng(3)
    m1 = rng.standard_normal(m.dof()) * 1e-9
    d1 = plan.born(m1).double().cpu().numpy().copy()
    d1b = plan.born(2.0 * m1).double().cpu().numpy()
    assert _rel(d1b, 2.0 * d1) < 1e-13
    d = rng.standard_normal(d1.shape)
    img = plan.migrate(torch.as_tensor(d, device="cuda")).cpu().numpy()
    lhs = float(np.sum(d1 * d))
    rhs = float(np.dot(m1, img)) * float(np.prod(m.deltas)) / solver.dt
    assert lhs == pytest.approx(rhs, rel=1e-9)
    # the Hessian is symmetric: <H a, b> = <a, H b>
    a_, b_ = rng.standard_normal(m.dof()) * 1e-9, rng.standard_normal(m.dof()) * 1e-9
    ha = plan.hessian(a_)[0].cpu().numpy().copy()
    hb = plan.hessian(b_)[0].cpu().numpy()
    assert float(np.dot(ha, b_)) == pytest.approx(float(np.dot(a_, hb)), rel=1e-9)
    assert plan.status() == 0


def test_gauss_newton_step_matches_the_oracle():
    """One Gauss-Newton step (5 GMRES iterations, unit step) with the GPU gradient and the
    batched GPU Hessian equals the step built from the oracle's gradient and Hessian."""
    from pysit_gb300.optimization import krylov
    m, shots, solver, C, C0 = problems.build(api, "o2")
    api.generate_seismic_data(shots, solver, solver.ModelParameters(m, {"C": C}))
    m0 = solver.ModelParameters(m, {"C": C0})
    gn = api.GaussNewton(api.TemporalLeastSquares(solver), krylov_maxiter=5)
    out = gn(shots, m0, 1, line_search=("constant", 1.0))
    solver.model_parameters = m0
    Ps = [problems.oracle_problem(solver, s) for s in shots]
    dobs = [s.receivers.interpolate_data(solver.ts()) for s in shots]
    grad, _ = pipeline.gradient(Ps, dobs)
    d, info = krylov.gmres(lambda x: pipeline.hessian(Ps, x), -grad, maxiter=5)
    # the step is taken in m = C**-2 (linearize())
    m_start = np.asarray(m0.linearize()).reshape(-1)
    m_out = np.asarray(out.linearize()).reshape(-1)
    assert _rel(m_out - m_start, d) < 1e-7
    assert _rel(m_out, m_start + d) < 1e-12
    assert len(gn.krylov_residuals) == 6 and gn.krylov_residuals[-1] < gn.krylov_residuals[0]
