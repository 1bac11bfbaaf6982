"""Pins of the oracle's Born modelling and Hessian applications against the unmodified
reference (fixtures tests/golden/born_<problem>.npz made by make_golden.py born:<problem>):

* TemporalModeling.linear_forward_model 'simdata' of every shot
  (pysit/modeling/temporal_modeling.py:389-546);
* TemporalLeastSquares.apply_hessian in the modes approximate, levenberg and full
  (pysit/objective_functions/temporal_least_squares.py:200-249), at the starting model of
  each problem, for the seeded perturbation stored in the fixture.
"""
import numpy as np
import pytest

import pipeline
import problems
import pysit_gb300 as api

BORN_PROBLEMS = ["o2", "o8", "1d", "3d"]


def _rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300)


def _setup(name, golden):
    g, b = golden(name), golden(f"born_{name}")
    m, shots, solver, C, C0 = problems.build(api, name)
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    assert solver.nsteps == int(b["nsteps0"]) and solver.dt == pytest.approx(float(b["dt0"]), rel=1e-15)
    Ps = [problems.oracle_problem(solver, s) for s in shots]
    return g, b, Ps


@pytest.mark.parametrize("name", BORN_PROBLEMS)
def test_oracle_born_matches_reference(name, golden):
    g, b, Ps = _setup(name, golden)
    d1 = np.stack([pipeline.born(P, b["m1"])[0] for P in Ps])
    assert _rel(d1, b["d1"]) < 1e-11


@pytest.mark.parametrize("mode", ["approximate", "levenberg", "full"])
@pytest.mark.parametrize("name", BORN_PROBLEMS)
def test_oracle_hessian_matches_reference(name, mode, golden):
    g, b, Ps = _setup(name, golden)
    h = pipeline.hessian(Ps, b["m1"], mode, float(b["levenberg_mu"]), dobs=list(g["dobs0"]))
    assert _rel(h, b[f"hess_{mode}"]) < 1e-10


def test_oracle_born_is_linear_and_its_adjoint_is_migration():
    """<F m1, d> = <m1, F* d> with F* the unfolded migration: the dot-product test the
    reference's adjoint checks print (temporal_modeling.py:1086-1188), here asserted."""
    m, shots, solver, C, C0 = problems.build(api, "o6")
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    P = problems.oracle_problem(solver, shots[0])
    rng = np.random.default_rng(5)
    n_phys = m.dof(include_bc=False)
    m1 = rng.standard_normal(n_phys) * 1e-9
    d1, dws = pipeline.born(P, m1)
    d1b, _ = pipeline.born(P, 3.0 * m1)
    assert _rel(d1b, 3.0 * d1) < 1e-13
    d = rng.standard_normal(d1.shape)
    # migrate_shot = -dt * sum_k q_k dWaveOp0_k with the padding folded (the adjoint of the
    # edge padding).  The receivers sample with S = base * cell volume and inject with
    # S* = base^T (mesh_representation.py:211-212), so <F m1, d> = <m1, migrate(d)> * dV / dt
    # with the sign of the Born source -m1 dWaveOp0 cancelling the migration's minus.
    img = pipeline.fold(P, pipeline.adjoint_image(P, d, dws))
    lhs = float(np.sum(d1 * d))
    rhs = float(np.dot(m1, img)) * float(np.prod(P["deltas"])) / P["dt"]
    assert lhs == pytest.approx(rhs, rel=1e-6)
