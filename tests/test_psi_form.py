"""The two forms of the 3D PML psi term (oracle, CPU).

The reference's 3D step multiplies sigma_x sigma_y sigma_z psi by C^2
(pysit/solvers/constant_density_acoustic/time/scalar/constant_density_acoustic_time_scalar_3D.h:219),
which its matrix operator does not; with it, the step diverges at realistic PML
amplitudes.  The oracle's default reproduces the reference (pinned to its templates in
test_oracle_pin.py); the consistent form is the pml_psi='consistent' option of the
batched path."""
import os
import sys

import numpy as np
import pytest

import problems
import pysit_gb300 as api

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import pipeline  # noqa: E402

STRONG = dict(pml=(4, 160.0))  # the 3D problem with a realistic PML amplitude


def _forward(consistent):
    m, shots, solver, C, C0 = problems.build(api, "3d", spec_overrides=STRONG)
    solver.model_parameters = solver.ModelParameters(m, {"C": C})
    P = problems.oracle_problem(solver, shots[0])
    try:
        pipeline.set_psi_consistent(consistent)
        sim, _ = pipeline.forward(P)
    finally:
        pipeline.set_psi_consistent(False)
    return sim


def test_reference_form_diverges_where_the_consistent_form_stays_bounded():
    ref = _forward(False)
    con = _forward(True)
    assert np.all(np.isfinite(con))
    peak = np.abs(con).max()
    assert 0 < peak < 1.0  # the traces of a unit Ricker source
    # the reference form blows up within the record (or overflows)
    assert (not np.all(np.isfinite(ref))) or np.abs(ref).max() > 1e6 * peak


def test_forms_agree_while_the_psi_term_is_negligible():
    # weak PML: sigma_x sigma_y sigma_z psi is tiny next to the other terms
    m, shots, solver, C, C0 = problems.build(api, "3d")
    solver.model_parameters = solver.ModelParameters(m, {"C": C})
    P = problems.oracle_problem(solver, shots[0])
    try:
        pipeline.set_psi_consistent(True)
        con, _ = pipeline.forward(P)
    finally:
        pipeline.set_psi_consistent(False)
    ref, _ = pipeline.forward(P)
    assert np.linalg.norm(con - ref) / np.linalg.norm(ref) < 1e-3


def test_solver_rejects_an_unknown_psi_form():
    d = api.RectangularDomain((0.0, 100.0, api.PML(20.0, 10.0), api.PML(20.0, 10.0)),
                              (0.0, 100.0, api.PML(20.0, 10.0), api.PML(20.0, 10.0)),
                              (0.0, 100.0, api.PML(20.0, 10.0), api.PML(20.0, 10.0)))
    m = api.CartesianMesh(d, 11, 11, 11)
    with pytest.raises(ValueError):
        api.ConstantDensityAcousticWave(m, kernel_implementation="cuda", pml_psi="other")
