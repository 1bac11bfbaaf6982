"""GPU parity of the per-step C-ABI kernels against the CPU oracle
(which is pinned to the reference's templates in test_oracle_pin.py)."""
import ctypes as C

import numpy as np
import pytest

import pipeline

pytestmark = pytest.mark.gpu


def _inputs(dim, shape, dtype, rng, npml=(3, 4)):
    n = int(np.prod(shape))
    km1, k = rng.standard_normal(n).astype(dtype), rng.standard_normal(n).astype(dtype)
    aux = {a: rng.standard_normal(n).astype(dtype) for a in pipeline.AUX[dim]}
    Cm = (1500 + 1000 * rng.random(n)).astype(dtype)
    rhs = rng.standard_normal(n).astype(dtype)
    prof = [(np.linspace(80, 5, npml[0]).astype(dtype), np.linspace(5, 80, npml[1]).astype(dtype))
            for _ in range(dim)]
    return km1, aux, k, Cm, rhs, prof


def _gpu_step(dim, order, km1, aux, k, Cm, rhs, prof, dt, deltas, shape):
    import torch
    from pysit_gb300 import _native
    lib = _native.load()
    t = lambda a: torch.as_tensor(a, device="cuda")  # noqa: E731
    dt_code = _native.PYSIT_F64 if km1.dtype == np.float64 else _native.PYSIT_F32
    d = {k_: t(v) for k_, v in aux.items()}
    out = {k_: torch.zeros_like(v) for k_, v in d.items()}
    u = torch.zeros_like(t(k))
    ins = [t(x) for x in (km1, k, Cm, rhs)]
    pr = [(t(l), len(l), t(r), len(r)) for l, r in prof]
    P = lambda x: C.c_void_p(x.data_ptr()) if x.numel() else None  # noqa: E731
    s = _native.stream_handle()
    if dim == 1:
        rc = lib.pysit_cda_step_1d(dt_code, order, P(ins[0]), P(d["Phiz"]), P(ins[1]), P(ins[2]), P(ins[3]),
                                   P(pr[0][0]), pr[0][1], P(pr[0][2]), pr[0][3], dt, deltas[0], shape[0],
                                   P(out["Phiz"]), P(u), s)
    elif dim == 2:
        rc = lib.pysit_cda_step_2d(dt_code, order, P(ins[0]), P(d["Phix"]), P(d["Phiz"]), P(ins[1]), P(ins[2]),
                                   P(ins[3]), P(pr[0][0]), pr[0][1], P(pr[0][2]), pr[0][3], P(pr[1][0]), pr[1][1],
                                   P(pr[1][2]), pr[1][3], dt, deltas[0], deltas[1], shape[0], shape[1],
                                   P(out["Phix"]), P(out["Phiz"]), P(u), s)
    else:
        rc = lib.pysit_cda_step_3d(dt_code, order, P(ins[0]), P(d["Phix"]), P(d["Phiy"]), P(d["Phiz"]),
                                   P(d["psi"]), P(ins[1]), P(ins[2]), P(ins[3]),
                                   P(pr[0][0]), pr[0][1], P(pr[0][2]), pr[0][3], P(pr[1][0]), pr[1][1],
                                   P(pr[1][2]), pr[1][3], P(pr[2][0]), pr[2][1], P(pr[2][2]), pr[2][3],
                                   dt, deltas[0], deltas[1], deltas[2], shape[0], shape[1], shape[2],
                                   P(out["Phix"]), P(out["Phiy"]), P(out["Phiz"]), P(out["psi"]), P(u), s)
    _native.check(rc)
    torch.cuda.synchronize()
    return u.cpu().numpy(), {k_: v.cpu().numpy() for k_, v in out.items()}


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("order", [2, 4, 6, 8])
@pytest.mark.parametrize("dim,shape", [(1, [53]), (2, [37, 45]), (3, [17, 19, 21])])
def test_step_matches_oracle(dim, shape, order, dtype):
    rng = np.random.default_rng(11 * dim + order)
    km1, aux, k, Cm, rhs, prof = _inputs(dim, shape, dtype, rng)
    deltas = [7.0, 9.0, 11.0][:dim]
    ref_u, ref_aux = pipeline.step("oracle", dim, order, km1, aux, k, Cm, rhs, prof, 1e-3, deltas, shape)
    u, a = _gpu_step(dim, order, km1, aux, k, Cm, rhs, prof, 1e-3, deltas, shape)
    tol = 1e-13 if dtype == np.float64 else 3e-5
    assert np.abs(u - ref_u).max() <= tol * np.abs(ref_u).max()
    for name in pipeline.AUX[dim]:
        assert np.abs(a[name] - ref_aux[name]).max() <= tol * max(np.abs(ref_aux[name]).max(), 1e-30), name


@pytest.mark.parametrize("sides", [(0, 5), (5, 0), (0, 0)])
def test_step_dirichlet_sides(sides):
    rng = np.random.default_rng(2)
    shape = [23, 29]
    km1, aux, k, Cm, rhs, prof = _inputs(2, shape, np.float64, rng, npml=sides)
    ref_u, _ = pipeline.step("oracle", 2, 8, km1, aux, k, Cm, rhs, prof, 1e-3, [8.0, 8.0], shape)
    u, _ = _gpu_step(2, 8, km1, aux, k, Cm, rhs, prof, 1e-3, [8.0, 8.0], shape)
    assert np.abs(u - ref_u).max() <= 1e-13 * np.abs(ref_u).max()


@pytest.mark.parametrize("dim,shape", [(1, [40]), (2, [21, 26]), (3, [9, 10, 11])])
def test_dwaveop_matches_oracle(dim, shape):
    import torch
    from pysit_gb300 import _native
    rng = np.random.default_rng(4)
    n = int(np.prod(shape))
    um, uc, up, psi = (rng.standard_normal(n) for _ in range(4))
    maps = [np.abs(rng.standard_normal(s)) * 10 for s in shape]
    P = dict(dim=dim, dt=1e-3, shape=shape, sigmaps=maps)
    ref = pipeline.dwaveop(P, um, uc, up, psi if dim == 3 else None)
    t = lambda a: torch.as_tensor(a, device="cuda")  # noqa: E731
    out = torch.zeros(n, dtype=torch.float64, device="cuda")
    if dim == 1:
        dims, sg = (1, 1, shape[0]), (None, None, t(maps[0]))
    elif dim == 2:
        dims, sg = (shape[0], 1, shape[1]), (t(maps[0]), None, t(maps[1]))
    else:
        dims, sg = tuple(shape), tuple(t(m) for m in maps)
    ptr = lambda x: None if x is None else C.c_void_p(x.data_ptr())  # noqa: E731
    tensors = [t(um), t(uc), t(up), t(psi)]
    _native.check(_native.load().pysit_cda_dwaveop(_native.PYSIT_F64, dim, *[ptr(x) for x in tensors[:3]],
                                                   ptr(tensors[3]) if dim == 3 else None, *[ptr(x) for x in sg],
                                                   *dims, 1e-3, ptr(out), _native.stream_handle()))
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
