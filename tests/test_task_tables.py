"""Task tables of the 2D and 3D step kernels, read back through pysit_plan_task_table on the
host (no GPU): for grids with and without PML sides, orders 2-8, both precisions and the tile
choices the tuner may set, the tasks of a shot cover every cell of the padded grid exactly once;
interior tasks keep R cells clear of the padding and stay off the outer ring (the interior
kernels carry no PML terms and no masks); every task fits the lanes of its block (3D: a warp
takes 32 / vectors-of-z rows, 8 warps a block; 2D: at most 32 lane vectors of z)."""
import ctypes as C

import numpy as np
import pytest

from pysit_gb300 import _native


@pytest.fixture(scope="module")
def lib():
    from pysit_gb300 import build
    build.build()
    return _native.load()


def _desc(keep, dim, n, pml, order, dtype, tile_x=0, tile_z=0):
    """Plan description of one shot on the padded grid n (x, y, z), pml = (lo, hi) cells per axis
    (0: no PML on that side), one source and one receiver tap."""
    d = _native.PlanDesc()
    d.dim, d.order, d.dtype = dim, order, dtype
    axes = (0, 1, 2) if dim == 3 else (0, 2) if dim == 2 else (2,)
    for a in range(3):
        d.n[a] = n[a] if a in axes else 1
        d.delta[a] = 10.0
    for a in axes:
        lo, hi = pml[a]
        d.pad_lo[a], d.pad_hi[a] = lo, hi
        for side, cells in (("l", lo), ("r", hi)):
            if cells:
                prof = np.linspace(80.0, 5.0, cells)
                keep.append(prof)
                getattr(d, "sig_" + side)[a] = prof.ctypes.data_as(C.POINTER(C.c_double))
                getattr(d, "nsig_" + side)[a] = cells
    d.dt, d.nsteps, d.imaging_period, d.checkpoint_every = 1e-4, 8, 1, 4
    d.shots_per_launch = d.nshots = 1
    d.tile_x, d.tile_z = tile_x, tile_z
    ncell = int(np.prod([d.n[a] for a in range(3)]))
    arrs = dict(src_tap_ptr=np.array([0, 1], np.int64), src_tap_cell=np.array([ncell // 2], np.int64),
                src_tap_point=np.zeros(1, np.int32), src_tap_w=np.ones(1), src_amp=np.ones((1, 8, 1)),
                rec_tap_ptr=np.array([0, 1], np.int64), rec_tap_cell=np.array([ncell // 3], np.int64),
                rec_tap_point=np.zeros(1, np.int32), rec_tap_wsample=np.ones(1), rec_tap_winject=np.ones(1))
    ct = {np.int64: C.c_int64, np.int32: C.c_int32, np.float64: C.c_double}
    for k, v in arrs.items():
        keep.append(v)
        setattr(d, k, v.ctypes.data_as(C.POINTER(ct[v.dtype.type])))
    d.nsrc = d.nrec = 1
    return d


def _table(lib, d):
    h = C.c_void_p()
    _native.check(lib.pysit_plan_create(C.byref(d), C.byref(h)))
    try:
        n, ni = C.c_uint64(), C.c_int32()
        _native.check(lib.pysit_plan_task_table(h, None, 0, C.byref(n), C.byref(ni)))
        out = np.zeros(n.value, np.int32)
        _native.check(lib.pysit_plan_task_table(h, out.ctypes.data_as(C.POINTER(C.c_int32)), n.value, None, None))
    finally:
        lib.pysit_plan_destroy(h)
    return out, ni.value


def _interior_bounds(n, lo, hi, R):
    return (lo + R if lo > 0 else 1), (n - hi - R if hi > 0 else n - 1)


GRIDS3 = [((40, 36, 70), ((6, 6), (5, 7), (8, 8))),
          ((31, 29, 27), ((4, 4), (4, 4), (4, 4))),
          ((26, 30, 171), ((5, 5), (5, 5), (5, 5))),
          ((24, 22, 45), ((0, 6), (6, 0), (0, 7))),
          ((14, 12, 13), ((5, 5), (5, 5), (5, 5)))]   # too small for an interior


@pytest.mark.parametrize("grid", range(len(GRIDS3)))
@pytest.mark.parametrize("dtype", [_native.PYSIT_F32, _native.PYSIT_F64])
@pytest.mark.parametrize("order", [2, 8])
@pytest.mark.parametrize("tiles", [(0, 0), (8, 16), (16, 36), (64, 96)])
def test_3d_tasks_cover_the_grid_once(lib, grid, dtype, order, tiles):
    n, pml = GRIDS3[grid]
    keep = []
    tab, nint = _table(lib, _desc(keep, 3, n, pml, order, dtype, *tiles))
    tasks = tab.reshape(-1, 6)
    R, V = order // 2, 4 if dtype == _native.PYSIT_F32 else 2
    count = np.zeros(n, np.int16)
    box = [_interior_bounds(n[a], pml[a][0], pml[a][1], R) for a in range(3)]
    for t, (x0, x1, y0, y1, zs, ze) in enumerate(tasks):
        assert 0 <= x0 < x1 <= n[0] and 0 <= y0 < y1 <= n[1] and 0 <= zs < ze <= n[2]
        nzv = -(-(ze - zs) // V)
        assert zs % 4 == 0 and nzv <= 32
        assert y1 - y0 <= 8 * (32 // nzv)  # the block's warps reach every row
        if t < nint:
            assert ze % 4 == 0
            assert box[0][0] <= x0 and x1 <= box[0][1]
            assert box[1][0] <= y0 and y1 <= box[1][1]
            assert box[2][0] <= zs and ze <= box[2][1]
        count[x0:x1, y0:y1, zs:ze] += 1
    assert (count == 1).all()
    if grid < 3:
        assert nint > 0


GRIDS2 = [((70, 90), ((8, 8), (10, 10))),
          ((38, 32), ((4, 4), (4, 4))),
          ((41, 433), ((16, 16), (16, 16))),
          ((57, 47), ((0, 9), (9, 0))),
          ((12, 11), ((5, 5), (5, 5)))]


@pytest.mark.parametrize("grid", range(len(GRIDS2)))
@pytest.mark.parametrize("dtype", [_native.PYSIT_F32, _native.PYSIT_F64])
@pytest.mark.parametrize("order", [2, 4, 8])
@pytest.mark.parametrize("tiles", [(0, 0), (8, 16), (64, 96)])
def test_2d_tasks_cover_the_grid_once(lib, grid, dtype, order, tiles):
    (nx, nz), (px, pz) = GRIDS2[grid]
    keep = []
    tab, nint = _table(lib, _desc(keep, 2, (nx, 1, nz), (px, (0, 0), pz), order, dtype, *tiles))
    tasks = tab.reshape(-1, 5)
    R = order // 2
    count = np.zeros((nx, nz), np.int16)
    bx, bz = _interior_bounds(nx, px[0], px[1], R), _interior_bounds(nz, pz[0], pz[1], R)
    for t, (x0, x1, zs, ze, kind) in enumerate(tasks):
        assert 0 <= x0 < x1 <= nx and 0 <= zs < ze <= nz
        assert kind == (0 if t < nint else 1)
        V = 4 if (dtype == _native.PYSIT_F32 and kind == 0) else 2
        assert zs % 4 == 0 and ze - zs <= 32 * V
        if kind == 0:
            assert ze % 4 == 0
            assert bx[0] <= x0 and x1 <= bx[1] and bz[0] <= zs and ze <= bz[1]
        count[x0:x1, zs:ze] += 1
    assert (count == 1).all()


def test_task_table_of_a_1d_plan_is_empty(lib):
    keep = []
    tab, nint = _table(lib, _desc(keep, 1, (1, 1, 120), ((0, 0), (0, 0), (10, 10)), 4, _native.PYSIT_F64))
    assert tab.size == 0 and nint == 0


def test_3d_plan_refuses_x_planes_beyond_32_bit_tap_offsets(lib):
    keep = []
    d = _desc(keep, 3, (12, 24000, 24000), ((2, 2), (2, 2), (2, 2)), 4, _native.PYSIT_F32)
    h = C.c_void_p()
    assert lib.pysit_plan_create(C.byref(d), C.byref(h)) == _native.PYSIT_EINVAL
    assert b"x-plane" in lib.pysit_cuda_last_error()
