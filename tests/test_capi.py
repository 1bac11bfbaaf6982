"""The C-ABI library loads and exports every entry point include/pysit_gb300.h
declares; argument validation and plan construction run on the host (no GPU)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from pysit_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    with open(os.path.join(ROOT, "include", "pysit_gb300.h")) as f:
        txt = f.read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(pysit_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from pysit_gb300 import build
    build.build()
    return _native.load()


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_native.exported_symbols())


def test_version_and_empty_error(lib):
    with open(os.path.join(ROOT, "include", "pysit_gb300.h")) as f:
        header = int(re.search(r"#define PYSIT_ABI_VERSION (\d+)", f.read()).group(1))
    assert lib.pysit_cuda_version() == header >= 1000
    assert isinstance(lib.pysit_cuda_last_error(), bytes)


@pytest.mark.parametrize("order", [0, 3, 10])
def test_step_rejects_bad_order_without_touching_the_device(lib, order):
    rc = lib.pysit_cda_step_2d(_native.PYSIT_F64, order, *([C.c_void_p(8)] * 6), None, 0, None, 0, None, 0,
                               None, 0, 1e-3, 1.0, 1.0, 10, 10, *([C.c_void_p(8)] * 3), None)
    assert rc == _native.PYSIT_EINVAL
    assert b"order" in lib.pysit_cuda_last_error()


def test_step_rejects_bad_dtype_and_null(lib):
    rc = lib.pysit_cda_step_1d(7, 4, *([C.c_void_p(8)] * 5), None, 0, None, 0, 1e-3, 1.0, 10,
                               C.c_void_p(8), C.c_void_p(8), None)
    assert rc == _native.PYSIT_EINVAL
    rc = lib.pysit_cda_step_1d(_native.PYSIT_F32, 4, None, *([C.c_void_p(8)] * 4), None, 0, None, 0, 1e-3,
                               1.0, 10, C.c_void_p(8), C.c_void_p(8), None)
    assert rc == _native.PYSIT_EINVAL
    with pytest.raises(_native.PysitCudaError):
        _native.check(rc)


def test_step_rejects_tiny_grid_and_long_profile(lib):
    rc = lib.pysit_cda_step_2d(_native.PYSIT_F64, 4, *([C.c_void_p(8)] * 6), None, 0, None, 0, None, 0,
                               None, 0, 1e-3, 1.0, 1.0, 2, 10, *([C.c_void_p(8)] * 3), None)
    assert rc == _native.PYSIT_EINVAL
    rc = lib.pysit_cda_step_2d(_native.PYSIT_F64, 4, *([C.c_void_p(8)] * 6), C.c_void_p(8), 11, None, 0,
                               None, 0, None, 0, 1e-3, 1.0, 1.0, 10, 10, *([C.c_void_p(8)] * 3), None)
    assert rc == _native.PYSIT_EINVAL


def _desc(nshots=2, nsteps=50, n=(30, 1, 24), order=4, dtype=_native.PYSIT_F32, keep=None):
    d = _native.PlanDesc()
    d.dim, d.order, d.dtype = 2, order, dtype
    for a in range(3):
        d.n[a] = n[a]
        d.delta[a] = 5.0
    d.pad_lo[0] = d.pad_hi[0] = d.pad_lo[2] = d.pad_hi[2] = 4
    d.dt, d.nsteps, d.imaging_period, d.checkpoint_every = 1e-4, nsteps, 1, 7
    d.shots_per_launch, d.nshots, d.use_graph = nshots, nshots, 1
    prof = np.linspace(50, 5, 4)
    keep.append(prof)
    for a in (0, 2):
        d.sig_l[a] = prof.ctypes.data_as(C.POINTER(C.c_double))
        d.sig_r[a] = prof.ctypes.data_as(C.POINTER(C.c_double))
        d.nsig_l[a] = d.nsig_r[a] = 4
    arrs = dict(src_tap_ptr=np.array([0, 1, 2], np.int64), src_tap_cell=np.array([100, 200], np.int64),
                src_tap_point=np.zeros(2, np.int32), src_tap_w=np.ones(2),
                src_amp=np.ones((nshots, nsteps, 1)),
                rec_tap_ptr=np.array([0, 2, 4], np.int64), rec_tap_cell=np.array([150, 151, 150, 152], np.int64),
                rec_tap_point=np.array([0, 1, 0, 1], np.int32), rec_tap_wsample=np.ones(4),
                rec_tap_winject=np.ones(4))
    ct = {np.int64: C.c_int64, np.int32: C.c_int32, np.float64: C.c_double}
    for k, v in arrs.items():
        keep.append(v)
        setattr(d, k, v.ctypes.data_as(C.POINTER(ct[v.dtype.type])))
    d.nsrc, d.nrec = 1, 2
    return d


def test_plan_create_reports_workspace_and_destroys(lib):
    keep = []
    d = _desc(keep=keep)
    h = C.c_void_p()
    _native.check(lib.pysit_plan_create(C.byref(d), C.byref(h)))
    nb = C.c_uint64()
    _native.check(lib.pysit_plan_workspace_bytes(h, C.byref(nb)))
    # fields: grid (30+8) x pitch 32, 2 shots, FP32; replay 7 + checkpoints 8x4 + states
    assert nb.value > (30 + 8) * 32 * 4 * 2 * (7 + 8 * 4)
    # running before binding a workspace is an error, not a crash
    rc = lib.pysit_plan_forward(h, None, None)
    assert rc == _native.PYSIT_EINVAL
    assert lib.pysit_plan_step_loop(h, 0, 4, None) == _native.PYSIT_EINVAL
    assert b"no workspace" in lib.pysit_cuda_last_error()
    cand = (C.c_int * 2)(16, 32)
    chosen = C.c_int()
    assert lib.pysit_plan_autotune(h, cand, 2, 4, C.byref(chosen), None, None) == _native.PYSIT_EINVAL
    assert b"no workspace" in lib.pysit_cuda_last_error()
    _native.check(lib.pysit_plan_destroy(h))


def test_plan_rejects_bad_taps(lib):
    keep = []
    d = _desc(keep=keep)
    bad = np.array([10 ** 9, 5], np.int64)
    keep.append(bad)
    d.src_tap_cell = bad.ctypes.data_as(C.POINTER(C.c_int64))
    h = C.c_void_p()
    assert lib.pysit_plan_create(C.byref(d), C.byref(h)) == _native.PYSIT_EINVAL
    assert b"out of the grid" in lib.pysit_cuda_last_error()


def test_plan_workspace_scales_with_checkpoint_interval(lib):
    sizes = []
    for S in (1, 7, 50, 10 ** 6):
        keep = []
        d = _desc(keep=keep)
        d.checkpoint_every = S
        h = C.c_void_p()
        _native.check(lib.pysit_plan_create(C.byref(d), C.byref(h)))
        nb = C.c_uint64()
        _native.check(lib.pysit_plan_workspace_bytes(h, C.byref(nb)))
        sizes.append(nb.value)
        lib.pysit_plan_destroy(h)
    # replay grows with S, checkpoints shrink with it: S=7 is the cheapest of the three
    assert sizes[1] < sizes[0] and sizes[1] < sizes[2]
    # an interval past the record (50 steps) is one segment of the whole record
    assert sizes[3] == sizes[2]


def test_workspace_of_the_schedules(lib):
    """store_dwaveop keeps one field per imaged step instead of checkpoints + a replay of S
    steps; forward_only drops every adjoint, imaging, replay and checkpoint buffer."""
    sizes = {}
    for name, store, fwd, period in (("ckpt", 0, 0, 1), ("store", 1, 0, 1), ("store_p2", 1, 0, 2),
                                     ("fwd", 0, 1, 1)):
        keep = []
        d = _desc(keep=keep, nsteps=50)
        d.store_dwaveop, d.forward_only, d.imaging_period = store, fwd, period
        h = C.c_void_p()
        _native.check(lib.pysit_plan_create(C.byref(d), C.byref(h)))
        nb = C.c_uint64()
        _native.check(lib.pysit_plan_workspace_bytes(h, C.byref(nb)))
        sizes[name] = nb.value
        lib.pysit_plan_destroy(h)
    field = (30 + 8) * 32 * 4 * 2  # one FP32 field of the 2 shots (rows x pitch), lower bound
    assert sizes["store"] - sizes["store_p2"] >= 24 * field  # 50 vs 25 kept steps
    assert sizes["store"] > sizes["ckpt"] > sizes["fwd"]


def test_lanes_plan_workspace(lib):
    """lanes = 2 builds one plan per shot range; its workspace holds both plus the lane sums."""
    sizes = {}
    for lanes in (1, 2):
        keep = []
        d = _desc(keep=keep, nshots=2)
        d.shots_per_launch = 1
        d.lanes = lanes
        h = C.c_void_p()
        _native.check(lib.pysit_plan_create(C.byref(d), C.byref(h)))
        nb = C.c_uint64()
        _native.check(lib.pysit_plan_workspace_bytes(h, C.byref(nb)))
        sizes[lanes] = nb.value
        tile = C.c_int()
        _native.check(lib.pysit_plan_get_tuning(h, C.byref(tile), None))
        lib.pysit_plan_destroy(h)
    assert sizes[2] > sizes[1]
