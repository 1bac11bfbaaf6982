"""The allocation-free per-shot misfit entry point, checked against the plan's misfit.

pysit_misfit_per_shot_noalloc is for callers that cannot allocate device memory
(applications that reserve all device memory in their own pool up front, or
C/Fortran codes that link no allocator): it takes only its inputs and outputs and
keeps its reduction scratch in a fixed device array.  This file is collected
last so that a run stopping at the first failure has run every other test first;
it also passes when run alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import problems
import pysit_gb300 as api

pytestmark = pytest.mark.gpu


def _noalloc(plan, resid_out, out):
    from pysit_gb300 import _native
    torch = _native.require_cuda()
    code = _native.PYSIT_F64 if plan.tdtype == torch.float64 else _native.PYSIT_F32
    _native.check(_native.load().pysit_misfit_per_shot_noalloc(
        code, C.c_void_p(plan.dobs.data_ptr()), C.c_void_p(plan.traces.data_ptr()), plan.nshots,
        plan.nsteps * plan.nrec, C.c_void_p(resid_out.data_ptr()), C.c_void_p(out.data_ptr()),
        C.c_void_p(_native.stream_handle())))


@pytest.mark.parametrize("precision", ["double", "single"])
def test_noalloc_misfit_matches_plan_misfit_twice(precision):
    """Two calls in a row against the plan's misfit; the second allocates nothing, neither
    through torch's caching allocator nor on the device (free device memory unchanged)."""
    import torch
    from pysit_gb300.engine import WavePlan
    m, shots, solver, C_true, C0 = problems.build(api, "o8", precision=precision)
    api.generate_seismic_data(shots, solver, solver.ModelParameters(m, {"C": C_true}))
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    plan = WavePlan(solver, shots)
    plan.load_observed()
    rn_plan = float(plan.misfit(with_traces=True).item())
    resid = torch.empty_like(plan.traces)
    tol = 1e-12 if precision == "double" else 1e-5
    ref = (plan.dobs - plan.traces).double()
    expect = (ref.reshape(plan.nshots, -1) ** 2).sum(dim=1)
    out = torch.full((plan.nshots,), -1.0, dtype=torch.float64, device="cuda")
    for call in range(2):  # two calls in a row share the fixed scratch
        resid.fill_(float("nan"))
        out.fill_(-1.0)
        torch.cuda.synchronize()
        before = (torch.cuda.memory_allocated(), torch.cuda.mem_get_info()[0])
        _noalloc(plan, resid, out)
        torch.cuda.synchronize()
        if call == 1:  # the first call may load its kernels; the second allocates nothing at all
            assert (torch.cuda.memory_allocated(), torch.cuda.mem_get_info()[0]) == before
        assert float(out.sum().item()) == pytest.approx(rn_plan, rel=tol)
        assert torch.allclose(resid.double(), ref, rtol=0, atol=0)
        assert torch.allclose(out, expect, rtol=tol, atol=0)


def test_noalloc_in_place_residual():
    """resid may be the simulated-data array itself: the residual replaces it in place."""
    import torch
    from pysit_gb300.engine import WavePlan
    m, shots, solver, C_true, C0 = problems.build(api, "o2")
    api.generate_seismic_data(shots, solver, solver.ModelParameters(m, {"C": C_true}))
    solver.model_parameters = solver.ModelParameters(m, {"C": C0})
    plan = WavePlan(solver, shots)
    plan.load_observed()
    plan.misfit(with_traces=True)
    ref = (plan.dobs - plan.traces).clone()
    out = torch.empty(plan.nshots, dtype=torch.float64, device="cuda")
    _noalloc(plan, plan.traces, out)  # dsim and resid are one array
    torch.cuda.synchronize()
    assert torch.equal(plan.traces, ref)
    assert torch.allclose(out, (ref.reshape(plan.nshots, -1) ** 2).sum(dim=1), rtol=1e-12, atol=0)


def test_noalloc_rejects_too_many_shots():
    from pysit_gb300 import _native
    _native.require_cuda()
    rc = _native.load().pysit_misfit_per_shot_noalloc(_native.PYSIT_F32, C.c_void_p(16), C.c_void_p(16), 257, 10,
                                                      None, C.c_void_p(16), None)
    assert rc == _native.PYSIT_EINVAL
    assert b"256" in _native.load().pysit_cuda_last_error()
