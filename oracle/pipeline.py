"""TEST INFRASTRUCTURE: CPU restatement of PySIT's time-domain modelling and gradient.

Used only as the checker (tests/, __graft_entry__.smoke(), bench.py's CPU
baseline); the product never imports it.  Pinned against the reference by
tests/test_oracle_pin.py (step kernel versus the reference's own templates
compiled into oracle/_ref) and by the golden fixtures of tests/golden/.

A problem is given as plain arrays (padded grid, z fastest):
    dim, order, shape (padded), deltas, C (padded, flat), dt, nsteps,
    profiles[a] = (left, right)    step-kernel PML profiles per axis,
    sigmaps[a]                     full-length mesh sigma map per axis,
    pads[a] = (lo, hi)             padding widths per axis,
    src = (cells, points, weights, amps[nsteps, npts])   padded cells,
    rec = (cells, recs, w_sample, w_inject, nrec)       padded cells.
Restated reference functions (paths inside the pysit project):
    forward  TemporalModeling.forward_model      modeling/temporal_modeling.py:60-169
    dWaveOp  _compute_dWaveOp_time               solvers/constant_density_acoustic/
                                                 constant_density_acoustic_base.py:24-40
    adjoint  TemporalModeling.adjoint_model      modeling/temporal_modeling.py:228-387
    fold     ModelPerturbationBase.add_padding   solvers/model_parameter.py:537-594
    gradient TemporalLeastSquares.compute_gradient objective_functions/temporal_least_squares.py:141-198
    born     TemporalModeling.linear_forward_model modeling/temporal_modeling.py:389-546
    hessian  TemporalLeastSquares.apply_hessian   objective_functions/temporal_least_squares.py:200-249
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS = {}


def lib(kind="oracle"):
    """'oracle' = my C restatement (liboracle.so); 'ref' = the reference templates (_ref/libcda_ref.so)."""
    if kind not in _LIBS:
        path = os.path.join(_HERE, "liboracle.so" if kind == "oracle" else os.path.join("_ref", "libcda_ref.so"))
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} is not built (make -C oracle)")
        _LIBS[kind] = C.CDLL(path)
    return _LIBS[kind]


def ref_available():
    return os.path.exists(os.path.join(_HERE, "_ref", "libcda_ref.so"))


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def step(kind, dim, order, km1_u, k_aux, k_u, Cpad, rhs, profiles, dt, deltas, shape, omp=False):
    """One leapfrog step.  k_aux is a dict of the aux fields ('Phiz' | 'Phix','Phiz' |
    'Phix','Phiy','Phiz','psi').  Returns (kp1_u, kp1_aux).  dtype follows km1_u."""
    L = lib(kind)
    dt_ = km1_u.dtype
    suf = "f64" if dt_ == np.float64 else "f32"
    pfx = "ref" if kind == "ref" else "oracle"
    cast = lambda a: np.ascontiguousarray(a, dtype=dt_)  # noqa: E731
    km1_u, k_u, Cpad, rhs = cast(km1_u), cast(k_u), cast(Cpad), cast(rhs)
    prof = [(cast(l), cast(r)) for l, r in profiles]
    # the oracle's steps write every output cell; the reference's OpenMP variants get zeroed outputs
    new = np.empty_like if kind == "oracle" else np.zeros_like
    out_u = new(k_u)
    extra = [C.c_int(1 if omp else 0)] if kind == "ref" else []
    if dim == 1:
        phz = cast(k_aux["Phiz"])
        o_phz = new(phz)
        f = getattr(L, f"{pfx}_cda1d_step_{suf}")
        rc = f(C.c_int(order), _p(km1_u), _p(phz), _p(k_u), _p(Cpad), _p(rhs),
               _p(prof[0][0]), C.c_int(len(prof[0][0])), _p(prof[0][1]), C.c_int(len(prof[0][1])),
               C.c_double(dt), C.c_double(deltas[0]), C.c_int(shape[0]), _p(o_phz), _p(out_u), *extra)
        aux = {"Phiz": o_phz}
    elif dim == 2:
        phx, phz = cast(k_aux["Phix"]), cast(k_aux["Phiz"])
        o_phx, o_phz = new(phx), new(phz)
        f = getattr(L, f"{pfx}_cda2d_step_{suf}")
        rc = f(C.c_int(order), _p(km1_u), _p(phx), _p(phz), _p(k_u), _p(Cpad), _p(rhs),
               _p(prof[0][0]), C.c_int(len(prof[0][0])), _p(prof[0][1]), C.c_int(len(prof[0][1])),
               _p(prof[1][0]), C.c_int(len(prof[1][0])), _p(prof[1][1]), C.c_int(len(prof[1][1])),
               C.c_double(dt), C.c_double(deltas[0]), C.c_double(deltas[1]), C.c_int(shape[0]),
               C.c_int(shape[1]), _p(o_phx), _p(o_phz), _p(out_u), *extra)
        aux = {"Phix": o_phx, "Phiz": o_phz}
    else:
        phx, phy, phz, psi = (cast(k_aux[n]) for n in ("Phix", "Phiy", "Phiz", "psi"))
        outs = [new(phx) for _ in range(4)]
        f = getattr(L, f"{pfx}_cda3d_step_{suf}")
        rc = f(C.c_int(order), _p(km1_u), _p(phx), _p(phy), _p(phz), _p(psi), _p(k_u), _p(Cpad), _p(rhs),
               _p(prof[0][0]), C.c_int(len(prof[0][0])), _p(prof[0][1]), C.c_int(len(prof[0][1])),
               _p(prof[1][0]), C.c_int(len(prof[1][0])), _p(prof[1][1]), C.c_int(len(prof[1][1])),
               _p(prof[2][0]), C.c_int(len(prof[2][0])), _p(prof[2][1]), C.c_int(len(prof[2][1])),
               C.c_double(dt), C.c_double(deltas[0]), C.c_double(deltas[1]), C.c_double(deltas[2]),
               C.c_int(shape[0]), C.c_int(shape[1]), C.c_int(shape[2]),
               _p(outs[0]), _p(outs[1]), _p(outs[2]), _p(outs[3]), _p(out_u), *extra)
        aux = {"Phix": outs[0], "Phiy": outs[1], "Phiz": outs[2], "psi": outs[3]}
    if rc != 0:
        raise ValueError(f"oracle step rejected its arguments (rc={rc})")
    return out_u, aux


AUX = {1: ("Phiz",), 2: ("Phix", "Phiz"), 3: ("Phix", "Phiy", "Phiz", "psi")}


def set_psi_consistent(on):
    """3D oracle step: False (default) multiplies sigma_x sigma_y sigma_z psi by C^2 as the
    reference's _3D.h:219 does; True leaves C^2 out (the reference's matrix operator)."""
    lib("oracle").oracle_set_psi_consistent(C.c_int(1 if on else 0))


def _dwaveop_sigma(P):
    """S1, S2, S3 of dwaveop on the full grid, built once per problem: the reference keeps the
    same sums and products as the solver's operator_components (sxPsz, sxsz, ...;
    pysit/solvers/constant_density_acoustic/time/scalar/constant_density_acoustic_time_scalar_2D.py:51-65)."""
    c = P.get("_dwaveop_sigma")
    if c is not None and c[0] is P["sigmaps"]:
        return c[1:]
    dim = P["dim"]
    g = [np.asarray(s, float) for s in P["sigmaps"]]
    shape = P["shape"]
    if dim == 1:
        s1 = g[0]
        s2 = np.zeros_like(s1)
        s3 = None
    elif dim == 2:
        sx, sz = g[0][:, None], g[1][None, :]
        s1 = (sx + sz).reshape(-1)
        s2 = (sx * sz).reshape(-1)
        s3 = None
    else:
        sx, sy, sz = g[0][:, None, None], g[1][None, :, None], g[2][None, None, :]
        full = np.ones(tuple(shape))
        s1 = (full * (sx + sy + sz)).reshape(-1)
        s2 = (full * (sx * sy + sx * sz + sy * sz)).reshape(-1)
        s3 = (full * (sx * sy * sz)).reshape(-1)
    P["_dwaveop_sigma"] = (P["sigmaps"], s1, s2, s3)
    return s1, s2, s3


def dwaveop(P, um, uc, up, psi):
    """(u+ - 2u + u-)/dt^2 + S1 (u+ - u-)/(2dt) + S2 u (+ S3 psi in 3D), mesh sigma maps."""
    dt = P["dt"]
    s1, s2, s3 = _dwaveop_sigma(P)
    out = (up - 2 * uc + um) / dt ** 2 + s1 * (up - um) / (2.0 * dt) + s2 * uc
    if s3 is not None:
        out = out + s3 * psi
    return out


def forward(P, want_dwaveop=False, imaging_period=1, kind="oracle", dtype=np.float64):
    """Traces [nsteps, nrec] (recorded from u_k before step k) and optionally dWaveOp list."""
    dim, n = P["dim"], int(np.prod(P["shape"]))
    um = np.zeros(n, dtype)
    uc = np.zeros(n, dtype)
    aux = {a: np.zeros(n, dtype) for a in AUX[dim]}
    scells, spts, sw, amps = P["src"]
    rcells, rrecs, rws, rwi, nrec = P["rec"]
    sim = np.zeros((P["nsteps"], nrec))
    dws = []
    for k in range(P["nsteps"]):
        np.add.at(sim[k], rrecs, rws * uc[rcells])
        rhs = np.zeros(n)
        np.add.at(rhs, scells, sw * amps[k, spts])
        up, aux_n = step(kind, dim, P["order"], um, aux, uc, P["C"], rhs, P["profiles"], P["dt"], P["deltas"],
                         P["shape"])
        if want_dwaveop and k % imaging_period == 0:
            dws.append(dwaveop(P, um.astype(float, copy=False), uc.astype(float, copy=False), up.astype(float, copy=False),
                               aux["psi"].astype(float, copy=False) if dim == 3 else None))
        if k == P["nsteps"] - 1:
            break
        um, uc, aux = uc, up, aux_n
    return sim, dws


def adjoint_image(P, resid, dws, imaging_period=1, kind="oracle", dtype=np.float64, extra_rhs=None,
                  want_dwaveop=False):
    """Padded imaging condition -dt*p*sum_k q_k dWaveOp[k//p] of one shot.

    extra_rhs[k] (padded) is added to the adjoint source of step k (the Hessian's
    operand_model * operand_dWaveOpAdj[k], _setup_adjoint_rhs :216-226); with
    want_dwaveop the dWaveOp of the adjoint field after each step is returned too,
    in forward time order (adjoint_model's 'dWaveOpAdj', :342-345 and :383-385)."""
    dim, n = P["dim"], int(np.prod(P["shape"]))
    qm = np.zeros(n, dtype)
    qc = np.zeros(n, dtype)
    aux = {a: np.zeros(n, dtype) for a in AUX[dim]}
    rcells, rrecs, rws, rwi, nrec = P["rec"]
    ic = np.zeros(n)
    dwa = []
    for k in range(P["nsteps"] - 1, -1, -1):
        if k % imaging_period == 0:
            ic += qc * dws[k // imaging_period]
        rhs = np.zeros(n)
        np.add.at(rhs, rcells, rwi * resid[k, rrecs])
        if extra_rhs is not None:
            rhs += extra_rhs[k]
        qp, aux_n = step(kind, dim, P["order"], qm, aux, qc, P["C"], rhs, P["profiles"], P["dt"], P["deltas"],
                         P["shape"])
        if want_dwaveop and k % imaging_period == 0:
            dwa.append(dwaveop(P, qm.astype(float, copy=False), qc.astype(float, copy=False), qp.astype(float, copy=False),
                               aux["psi"].astype(float, copy=False) if dim == 3 else None))
        if k == 0:
            break
        qm, qc, aux = qc, qp, aux_n
    ic = ic * (-1 * P["dt"]) * imaging_period
    if want_dwaveop:
        return ic, dwa[::-1]
    return ic


def pad(P, m, mode=None):
    """Unpadded grid array -> padded grid: zeros (CartesianMesh.pad_array default, mesh.py:446-533)
    or numpy.pad's `mode` ('edge' for linear_forward_model's m1, temporal_modeling.py:434)."""
    pads = [tuple(p) for p in P["pads"]]
    inner = [s - lo - hi for s, (lo, hi) in zip(P["shape"], pads)]
    a = np.asarray(m, float).reshape(inner)
    return np.pad(a, pads, mode=mode or "constant").reshape(-1)


def born(P, m1, kind="oracle", dtype=np.float64, want_dwaveop1=False):
    """linear_forward_model (temporal_modeling.py:389-546) of one shot about the model of P:
    u1 driven by rhs_k = -m1_edge_padded * dWaveOp0_k, traces of u1_k recorded before step k.
    Returns (traces [nsteps, nrec], dWaveOp0 list[, dWaveOp1 list])."""
    dim, n = P["dim"], int(np.prod(P["shape"]))
    _, dws = forward(P, True, 1, kind, dtype)
    m1p = pad(P, m1, "edge")
    um = np.zeros(n, dtype)
    uc = np.zeros(n, dtype)
    aux = {a: np.zeros(n, dtype) for a in AUX[dim]}
    rcells, rrecs, rws, rwi, nrec = P["rec"]
    sim = np.zeros((P["nsteps"], nrec))
    dw1 = []
    for k in range(P["nsteps"]):
        np.add.at(sim[k], rrecs, rws * uc[rcells])
        rhs = m1p * (-1 * dws[k])
        up, aux_n = step(kind, dim, P["order"], um, aux, uc, P["C"], rhs, P["profiles"], P["dt"], P["deltas"],
                         P["shape"])
        if want_dwaveop1:
            dw1.append(dwaveop(P, um.astype(float, copy=False), uc.astype(float, copy=False), up.astype(float, copy=False),
                               aux["psi"].astype(float, copy=False) if dim == 3 else None))
        if k == P["nsteps"] - 1:
            break
        um, uc, aux = uc, up, aux_n
    if want_dwaveop1:
        return sim, dws, dw1
    return sim, dws


def hessian(Ps, m1, hessian_mode="approximate", levenberg_mu=0.0, dobs=None, kind="oracle"):
    """apply_hessian (temporal_least_squares.py:200-249) summed over shots, unpadded m-space.

    approximate / levenberg: sum_s F_s* F_s m1 (+ mu m1); full: adds the second-order terms
    driven by the residual r0 = dobs - F(m0) (needs dobs).  Every migration images at every
    step (imaging_period 1, the step of the dWaveOp0 lists)."""
    if hessian_mode not in ("approximate", "full", "levenberg"):
        raise ValueError(hessian_mode)
    out = np.zeros(np.asarray(m1).size)
    for i, P in enumerate(Ps):
        if hessian_mode in ("approximate", "levenberg"):
            d1, dws = born(P, m1, kind)
            out += fold(P, adjoint_image(P, d1, dws, 1, kind))
        else:
            sim0, _ = forward(P, False, 1, kind)
            r0 = dobs[i] - sim0
            d1, dws, dw1 = born(P, m1, kind, want_dwaveop1=True)
            ic1, dwa1 = adjoint_image(P, r0, dw1, 1, kind, want_dwaveop=True)
            m1z = pad(P, m1)
            ic2 = adjoint_image(P, d1, dws, 1, kind, extra_rhs=[m1z * d for d in dwa1])
            out += fold(P, ic1) + fold(P, ic2)
    if hessian_mode == "levenberg":
        out = out + levenberg_mu * np.asarray(m1, float).reshape(-1)
    return out


def fold(P, padded):
    """add_padding: every PML strip summed onto the adjacent boundary row/column."""
    a = np.array(padded, dtype=float).reshape(tuple(P["shape"]))
    sl = []
    for ax, (lo, hi) in enumerate(P["pads"]):
        nin = a.shape[ax] - lo - hi
        def s(x):
            idx = [slice(None)] * a.ndim
            idx[ax] = x
            return tuple(idx)
        a[s(lo)] += a[s(slice(0, lo))].sum(axis=ax)
        a[s(lo + nin - 1)] += a[s(slice(lo + nin, a.shape[ax]))].sum(axis=ax)
        sl.append(slice(lo, lo + nin))
    return a[tuple(sl)].reshape(-1)


def gradient(Ps, dobs, imaging_period=1, kind="oracle"):
    """compute_gradient over shots: (grad (unpadded, m-space), r_norm2 = sum ||r||^2)."""
    grad = None
    r2 = 0.0
    for P, d in zip(Ps, dobs):
        sim, dws = forward(P, True, imaging_period, kind)
        r = d - sim
        g = fold(P, adjoint_image(P, r, dws, imaging_period, kind))
        grad = -g if grad is None else grad - g
        r2 += float(np.linalg.norm(r) ** 2)
    return grad, r2
