"""The C oracle step against a plain-Python statement of the same arithmetic, bit for bit (FP64).

The oracle restates the reference templates (pysit/solvers/constant_density_acoustic/time/
scalar/constant_density_acoustic_time_scalar_{1D.h:44-131, 2D.h:43-180, 3D.h:46-236}); its cells
with every tap inside the grid take an unrolled path.  The loops here sum the same terms in the
same order with Python floats (IEEE doubles, no fused multiply-add), so any change of the
oracle's order of operations, on either path, shows up as a difference in the last bit.
"""
import ctypes as C

import numpy as np
import pytest

import pipeline

D1W = {1: [0, 1.0 / 2.0], 2: [0, 2.0 / 3.0, -1.0 / 12.0], 3: [0, 3.0 / 4.0, -3.0 / 20.0, 1.0 / 60.0],
       4: [0, 4.0 / 5.0, -1.0 / 5.0, 4.0 / 105.0, -1.0 / 280.0]}
D2W = {1: [-2.0, 1.0], 2: [-5.0 / 2.0, 4.0 / 3.0, -1.0 / 12.0], 3: [-49.0 / 18.0, 3.0 / 2.0, -3.0 / 20.0, 1.0 / 90.0],
       4: [-205.0 / 72.0, 8.0 / 5.0, -1.0 / 5.0, 8.0 / 315.0, -1.0 / 560.0]}


def _d1(v, idx, s, pos, n, R, d):
    acc = 0.0
    for m in range(-R, R + 1):
        if m == 0 or not 0 <= pos + m < n:
            continue
        w = D1W[R][m] if m > 0 else -D1W[R][-m]
        acc += w * v[idx + m * s]
    return acc / d


def _d2(v, idx, s, pos, n, R, d2):
    acc = 0.0
    for m in range(-R, R + 1):
        if not 0 <= pos + m < n:
            continue
        acc += D2W[R][abs(m)] * v[idx + m * s]
    return acc / d2


def _sig(l, r, i, n):
    if len(l) and i < len(l):
        return float(l[i])
    if len(r) and i >= n - len(r):
        return float(r[len(r) - ((n - 1) - i)])
    return 0.0


def _step2d(order, um_, px, pz, u, Cv, rhs, prof, dt, dx, dz, nx, nz):
    R = order // 2
    dt2, dx2, dz2 = dt * dt, dx * dx, dz * dz
    o_px, o_pz, o_u = np.zeros(nx * nz), np.zeros(nx * nz), np.zeros(nx * nz)
    for i in range(1, nx - 1):
        for k in range(1, nz - 1):
            idx = i * nz + k
            dudx = _d1(u, idx, nz, i, nx, R, dx)
            dphixdx = _d1(px, idx, nz, i, nx, R, dx)
            lap = _d2(u, idx, nz, i, nx, R, dx2)
            dudz = _d1(u, idx, 1, k, nz, R, dz)
            dphizdz = _d1(pz, idx, 1, k, nz, R, dz)
            lap += _d2(u, idx, 1, k, nz, R, dz2)
            sx, sz = _sig(*prof[0], i, nx), _sig(*prof[1], k, nz)
            c2 = Cv[idx] * Cv[idx]
            um, uc = um_[idx], u[idx]
            if sz != 0 or sx != 0:
                o_px[idx] = px[idx] - dt * sx * px[idx] + dt * (sz - sx) * dudx
                o_pz[idx] = pz[idx] - dt * sz * pz[idx] + dt * (sx - sz) * dudz
                fac1 = 2.0 * dt2 / (2.0 + dt * (sx + sz))
                fac2 = (c2 * (rhs[idx] + lap + dphixdx + dphizdz) - (um - 2.0 * uc) / dt2
                        + (sx + sz) * um / (2.0 * dt) - (sx * sz) * uc)
                o_u[idx] = fac1 * fac2
            else:
                o_px[idx], o_pz[idx] = px[idx], pz[idx]
                o_u[idx] = dt2 * c2 * (rhs[idx] + lap + dphixdx + dphizdz) - (um - 2.0 * uc)
    return o_u, o_px, o_pz


def _step3d(order, um_, px, py, pz, psi, u, Cv, rhs, prof, dt, dd, n, consistent):
    R = order // 2
    nx, ny, nz = n
    dx, dy, dz = dd
    dt2, dx2, dy2, dz2 = dt * dt, dx * dx, dy * dy, dz * dz
    ys, xs = nz, ny * nz
    N = nx * ny * nz
    o = [np.zeros(N) for _ in range(5)]  # u, phix, phiy, phiz, psi
    for i in range(1, nx - 1):
        for j in range(1, ny - 1):
            for k in range(1, nz - 1):
                idx = i * xs + j * ys + k
                dudx = _d1(u, idx, xs, i, nx, R, dx)
                dphixdx = _d1(px, idx, xs, i, nx, R, dx)
                dpsidx = _d1(psi, idx, xs, i, nx, R, dx)
                lap = _d2(u, idx, xs, i, nx, R, dx2)
                dudy = _d1(u, idx, ys, j, ny, R, dy)
                dphiydy = _d1(py, idx, ys, j, ny, R, dy)
                dpsidy = _d1(psi, idx, ys, j, ny, R, dy)
                lap += _d2(u, idx, ys, j, ny, R, dy2)
                dudz = _d1(u, idx, 1, k, nz, R, dz)
                dphizdz = _d1(pz, idx, 1, k, nz, R, dz)
                dpsidz = _d1(psi, idx, 1, k, nz, R, dz)
                lap += _d2(u, idx, 1, k, nz, R, dz2)
                sx, sy, sz = _sig(*prof[0], i, nx), _sig(*prof[1], j, ny), _sig(*prof[2], k, nz)
                c2 = Cv[idx] * Cv[idx]
                um, uc = um_[idx], u[idx]
                o[4][idx] = psi[idx] + dt * uc
                if sz != 0 or sy != 0 or sx != 0:
                    o[1][idx] = px[idx] - dt * sx * px[idx] + dt * (sy + sz - sx) * dudx + dt * (sy * sz * dpsidx)
                    o[2][idx] = py[idx] - dt * sy * py[idx] + dt * (sz + sx - sy) * dudy + dt * (sz * sx * dpsidy)
                    o[3][idx] = pz[idx] - dt * sz * pz[idx] + dt * (sx + sy - sz) * dudz + dt * (sx * sy * dpsidz)
                    fac1 = 2.0 * dt2 / (2.0 + dt * (sx + sy + sz))
                    if consistent:
                        src = c2 * (rhs[idx] + lap + dphixdx + dphiydy + dphizdz) - (sx * sy * sz) * psi[idx]
                    else:
                        src = c2 * (rhs[idx] + lap + dphixdx + dphiydy + dphizdz - (sx * sy * sz) * psi[idx])
                    fac2 = (src - (um - 2.0 * uc) / dt2 + (sx + sy + sz) * um / (2.0 * dt)
                            - (sx * sy + sy * sz + sz * sx) * uc)
                    o[0][idx] = fac1 * fac2
                else:
                    o[1][idx], o[2][idx], o[3][idx] = px[idx], py[idx], pz[idx]
                    o[0][idx] = dt2 * c2 * (rhs[idx] + lap + dphixdx + dphiydy + dphizdz) - (um - 2.0 * uc)
    return o


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


@pytest.mark.parametrize("order", [2, 4, 6, 8])
def test_2d_step_bit_for_bit(order):
    rng = np.random.default_rng(order)
    nx, nz = 14, 17
    f = [rng.standard_normal(nx * nz) for _ in range(6)]
    f[4] = 1500.0 + 100.0 * rng.random(nx * nz)
    prof = [(rng.random(3) * 60, rng.random(4) * 60), (rng.random(5) * 60, np.zeros(0))]
    dt, dx, dz = 1e-3, 5.0, 4.0
    outs = [np.empty(nx * nz) for _ in range(3)]
    rc = pipeline.lib("oracle").oracle_cda2d_step_f64(
        C.c_int(order), *[_p(a) for a in f],
        _p(prof[0][0]), C.c_int(3), _p(prof[0][1]), C.c_int(4), _p(prof[1][0]), C.c_int(5), _p(prof[1][1]), C.c_int(0),
        C.c_double(dt), C.c_double(dx), C.c_double(dz), C.c_int(nx), C.c_int(nz), *[_p(a) for a in outs])
    assert rc == 0
    o_u, o_px, o_pz = _step2d(order, f[0], f[1], f[2], f[3], f[4], f[5], prof, dt, dx, dz, nx, nz)
    np.testing.assert_array_equal(outs[2], o_u)
    np.testing.assert_array_equal(outs[0], o_px)
    np.testing.assert_array_equal(outs[1], o_pz)


@pytest.mark.parametrize("order", [2, 8])
@pytest.mark.parametrize("consistent", [0, 1])
def test_3d_step_bit_for_bit(order, consistent):
    rng = np.random.default_rng(10 * order + consistent)
    n = (11, 10, 12)
    N = int(np.prod(n))
    f = [rng.standard_normal(N) for _ in range(8)]   # um, phix, phiy, phiz, psi, u, C, rhs
    f[6] = 1500.0 + 100.0 * rng.random(N)
    prof = [(rng.random(2) * 40, rng.random(3) * 40), (np.zeros(0), rng.random(2) * 40),
            (rng.random(4) * 40, rng.random(2) * 40)]
    dt, dd = 1e-3, (5.0, 6.0, 4.0)
    outs = [np.empty(N) for _ in range(5)]   # phix, phiy, phiz, psi, u
    lib = pipeline.lib("oracle")
    lib.oracle_set_psi_consistent(C.c_int(consistent))
    try:
        args = []
        for lo, hi in prof:
            args += [_p(lo), C.c_int(len(lo)), _p(hi), C.c_int(len(hi))]
        rc = lib.oracle_cda3d_step_f64(C.c_int(order), *[_p(a) for a in f], *args, C.c_double(dt),
                                       *[C.c_double(x) for x in dd], *[C.c_int(x) for x in n],
                                       *[_p(a) for a in outs])
    finally:
        lib.oracle_set_psi_consistent(C.c_int(0))
    assert rc == 0
    o = _step3d(order, f[0], f[1], f[2], f[3], f[4], f[5], f[6], f[7], prof, dt, dd, n, consistent)
    for got, want in zip((outs[4], outs[0], outs[1], outs[2], outs[3]), o):
        np.testing.assert_array_equal(got, want)
