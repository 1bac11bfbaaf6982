"""Parity on grids whose z extent spans several task segments of the step kernels.

The step kernels cut the padded grid into warp / block tasks whose z-range is at most one
segment (32 lanes x the lane vector: 128 cells in the FP32 2D interior, 64 in FP64).  The
golden problems are small enough to fit one segment; the benchmark grid (464 cells in z)
is not.  These problems have 433 (2D) and 171 (3D) padded cells in z, with the sources at mid
depth so that the wavefields cross the segment boundaries:
  FP64 batched traces and gradient against the CPU oracle (<= 1e-11 / <= 1e-9),
  FP32 against that FP64 result (<= 1e-4 / <= 1e-3),
under both gradient schedules.
"""
import numpy as np
import pytest

import pipeline
import problems
import pysit_gb300 as api

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a, float).reshape(-1), np.asarray(b, float).reshape(-1)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _oracle(name):
    m, shots, solver, C, C0 = problems.build(api, name)
    solver.model_parameters = solver.ModelParameters(m, {"C": C})
    traces = [pipeline.forward(problems.oracle_problem(solver, s))[0] for s in shots]
    ts_true = solver.ts()
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    ts0 = solver.ts()
    # observed data on the start model's time axis (linear, zero outside: interp1d semantics)
    dobs = [np.stack([np.interp(ts0, ts_true, tr[:, r], left=0.0, right=0.0) for r in range(tr.shape[1])], axis=1)
            for tr in traces]
    grad, r2 = pipeline.gradient([problems.oracle_problem(solver, s) for s in shots], dobs)
    nz = m.shape(include_bc=True, as_grid=True)[-1]
    return dict(traces=np.stack(traces), dobs=np.stack(dobs), grad=grad, r2=r2, nz=nz)


@pytest.fixture(scope="module")
def deep2d():
    return _oracle("deep")


@pytest.fixture(scope="module")
def deep3d():
    return _oracle("deep3d")


@pytest.fixture(scope="module")
def manyrec():
    return _oracle("manyrec")


def _gpu(name, precision, schedule, dobs):
    import torch
    from pysit_gb300.engine import WavePlan
    m, shots, solver, C, C0 = problems.build(api, name, precision=precision)
    solver.model_parameters = solver.ModelParameters(m, {"C": C})
    fplan = WavePlan(solver, shots, forward_only=True)
    traces = fplan.forward().double().cpu().numpy()
    assert fplan.check_status() == 0
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    plan = WavePlan(solver, shots, gradient_schedule=schedule, checkpoint_every=23)
    plan.dobs.copy_(torch.as_tensor(dobs))
    g, rn = plan.gradient()
    assert plan.check_status() == 0
    return traces, g.cpu().numpy(), float(rn.item())


def _check(ref, name):
    out = {}
    for schedule in ("checkpoint", "store"):
        tr64, g64, r64 = _gpu(name, "double", schedule, ref["dobs"])
        assert _rel(tr64, ref["traces"]) < 1e-11
        assert _rel(g64, ref["grad"]) < 1e-9
        assert r64 == pytest.approx(ref["r2"], rel=1e-10)
        tr32, g32, r32 = _gpu(name, "single", schedule, ref["dobs"])
        assert _rel(tr32, tr64) < 1e-4
        assert _rel(g32, g64) < 1e-3
        assert r32 == pytest.approx(r64, rel=1e-3)
        out[schedule] = (g64, g32)
    return out


def test_deep_2d_grid_matches_the_oracle(deep2d):
    # the FP32 interior segment is 128 cells, the FP64 one 64: at least three and six of them
    assert deep2d["nz"] - 2 * (16 + 4) > 2 * 128
    _check(deep2d, "deep")


def test_deep_3d_grid_matches_the_oracle(deep3d):
    assert deep3d["nz"] - 2 * (5 + 4) > 128
    _check(deep3d, "deep3d")


def test_many_receivers_match_the_oracle(manyrec):
    # 12 x 501 receivers at 8 recorder threads each exceed the 128-thread recorder blocks of one
    # block per SM (152 on a GB300) several times over
    nshots, _, nrec = manyrec["traces"].shape
    assert nshots * nrec * 8 > 2 * 152 * 128
    _check(manyrec, "manyrec")
