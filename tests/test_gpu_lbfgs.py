"""LBFGS driven by the GPU objective against PySIT's own LBFGS on its cpp FP64 solver
(tests/golden/lbfgs_o2.npz, made by make_golden.py): same objective history, step
lengths, number of misfit / gradient evaluations and final model."""
import os

import numpy as np
import pytest

import problems
import pysit_gb300 as api

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _run(precision, batched):
    g = np.load(os.path.join(HERE, "golden", "lbfgs_o2.npz"))
    m, shots, solver, C, C0 = problems.build(api, "o2", precision=precision)
    api.generate_seismic_data(shots, solver, solver.ModelParameters(m, {"C": C}))
    obj = api.TemporalLeastSquares(solver, batched=batched)
    calls = {"evaluate": 0, "gradient": 0}
    ev, gr = obj.evaluate, obj.compute_gradient

    def evaluate(*a, **k):
        calls["evaluate"] += 1
        return ev(*a, **k)

    def compute_gradient(*a, **k):
        calls["gradient"] += 1
        return gr(*a, **k)

    obj.evaluate, obj.compute_gradient = evaluate, compute_gradient
    opt = api.LBFGS(obj, memory_length=10)
    final = opt(shots, solver.ModelParameters(m, {"C": C0}), int(g["iterations"]), line_search="backtrack",
                status_configuration={"objective_frequency": 1, "gradient_length_frequency": 1})
    _, objective = opt.retrieve_history("objective")
    _, alpha = opt.retrieve_history("alpha")
    return g, np.array(objective), np.array(alpha), np.asarray(final.C).reshape(-1), calls


@pytest.mark.parametrize("batched", [True, False])
def test_lbfgs_fp64_follows_the_reference_run(batched):
    g, objective, alpha, final_C, calls = _run("double", batched)
    np.testing.assert_allclose(objective, g["objective"], rtol=1e-9)
    np.testing.assert_allclose(alpha, g["alpha"], rtol=1e-9)
    np.testing.assert_allclose(final_C, g["final_C"], rtol=1e-10)
    assert (calls["evaluate"], calls["gradient"]) == (int(g["n_evaluate"]), int(g["n_gradient"]))


def test_lbfgs_fp32_batched_tracks_the_reference_run():
    g, objective, alpha, final_C, calls = _run("single", True)
    # FP32 gradients carry ~1e-4 relative error; the misfit curve and the model follow closely
    np.testing.assert_allclose(objective, g["objective"], rtol=2e-2)
    assert np.linalg.norm(final_C - g["final_C"]) / np.linalg.norm(g["final_C"]) < 1e-4
