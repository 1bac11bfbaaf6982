"""Generate the golden fixtures of tests/golden/ by running the unmodified reference.

Run where the reference tree exists, after ``make -C oracle`` built its SWIG module into
oracle/_ref (the tree is PYSIT_REFERENCE_ROOT or the one oracle/Makefile used):

    python tests/golden/make_golden.py            # all problems of tests/problems.py
    python tests/golden/make_golden.py lbfgs:o2   # the reference's LBFGS run on problem o2
    python tests/golden/make_golden.py born:o2    # Born modelling and Hessian applications on o2
    python tests/golden/make_golden.py period:o6:2  # the gradient with imaging every 2 steps
    python tests/golden/make_golden.py fwd:o2     # forward_model's wavefield and dWaveOp snapshots
    python tests/golden/make_golden.py mig:o6     # migrate_shot of a seeded operand

For every problem it stores (compressed .npz): the traces of every shot
modelled on the true model by the reference's own ``generate_seismic_data``
with ``kernel_implementation='cpp'`` (FP64), the gradient and objective of
``TemporalLeastSquares.compute_gradient`` at the starting model, dt/nsteps of
both models, and snapshots of host-side operators (source / receiver
smearing weights, PML profiles, resampled observed data) that the product's
host code must reproduce.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import pysit_live  # noqa: E402
import problems  # noqa: E402


def _sparse_nz(op):
    import scipy.sparse as spsp
    op = op.tocsr() if hasattr(op, "tocsr") else spsp.csr_matrix(np.asarray(op))
    coo = op.tocoo()
    order = np.lexsort((coo.col, coo.row))
    return np.asarray(coo.row)[order], np.asarray(coo.col)[order], np.asarray(coo.data)[order]


def run(name):
    pysit = pysit_live.import_pysit()
    m, shots, solver, C, C0 = problems.build(pysit, name, kernel="cpp")
    truth = solver.ModelParameters(m, {"C": C})
    pysit.generate_seismic_data(shots, solver, truth)
    dt_true, nsteps_true = solver.dt, solver.nsteps
    traces = np.stack([s.receivers.data.copy() for s in shots])
    obj = pysit.TemporalLeastSquares(solver)
    start = solver.ModelParameters(m, {"C": C0})
    aux = {"objective_value": (True, None), "residual_norm": (True, None)}
    grad = obj.compute_gradient(shots, start, aux)
    dt0, nsteps0 = solver.dt, solver.nsteps
    dobs0 = np.stack([s.receivers.interpolate_data(solver.ts()) for s in shots])
    out = dict(traces=traces, dt_true=dt_true, nsteps_true=nsteps_true, grad=grad.data.reshape(-1),
               objective=aux["objective_value"][1], residual_norm=aux["residual_norm"][1],
               dt0=dt0, nsteps0=nsteps0, dobs0=dobs0)
    s0 = shots[0]
    r, c, v = _sparse_nz(s0.sources.adjoint_sampling_operator)
    out.update(src_rows=r, src_vals=v)
    r, c, v = _sparse_nz(s0.receivers.sampling_operator)
    out.update(rec_rows=r, rec_cols=c, rec_vals=v)
    for a in range(m.dim):
        p = m.parameters[a]
        for side, bc in (("l", p.lbc), ("r", p.rbc)):
            if bc.type == "pml":
                out[f"sigma_{a}{side}"] = np.asarray(bc.sigma)
        axis = {1: "z", 2: "xz", 3: "xyz"}[m.dim][a]
        out[f"sigmap_{a}"] = np.asarray(solver.operator_components["s" + axis])
    out["ricker"] = np.array([pysit.RickerWavelet(problems.SPECS[name]["f"])(t) for t in (0.0, 0.01, 0.05, 0.1)])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}: shots={len(shots)} nsteps_true={nsteps_true} nsteps0={nsteps0} "
          f"|grad|={np.linalg.norm(out['grad']):.6e} objective={out['objective']:.6e}")


def run_period(name, period):
    """compute_gradient with imaging every `period` steps (temporal_least_squares.py:16-25,
    forward_model / migrate_shot with imaging_period, temporal_modeling.py:146-148, 313-365)."""
    pysit = pysit_live.import_pysit()
    m, shots, solver, C, C0 = problems.build(pysit, name, kernel="cpp")
    pysit.generate_seismic_data(shots, solver, solver.ModelParameters(m, {"C": C}))
    obj = pysit.TemporalLeastSquares(solver, imaging_period=period)
    aux = {"objective_value": (True, None)}
    grad = obj.compute_gradient(shots, solver.ModelParameters(m, {"C": C0}), aux)
    out = dict(grad=grad.data.reshape(-1), objective=aux["objective_value"][1], period=period,
               nsteps0=solver.nsteps)
    np.savez_compressed(os.path.join(HERE, f"period{period}_{name}.npz"), **out)
    print(f"period{period}_{name}: |grad|={np.linalg.norm(out['grad']):.6e} objective={out['objective']:.6e}")


def run_fwd(name):
    """forward_model(shot 0, true model, imaging_period 1, ['simdata', 'wavefield', 'dWaveOp'])
    (temporal_modeling.py:60-169): the wavefield (unpadded, before the step) and dWaveOp (padded,
    after it) at four steps."""
    pysit = pysit_live.import_pysit()
    m, shots, solver, C, C0 = problems.build(pysit, name, kernel="cpp")
    tm = pysit.TemporalModeling(solver)
    rv = tm.forward_model(shots[0], solver.ModelParameters(m, {"C": C}), 1, ["simdata", "wavefield", "dWaveOp"])
    n = solver.nsteps
    ks = np.array([1, n // 3, 2 * n // 3, n - 1])
    out = dict(steps=ks, simdata=rv["simdata"], nsteps=n, dt=solver.dt,
               wavefield=np.stack([np.ravel(rv["wavefield"][k]) for k in ks]),
               dwaveop=np.stack([np.ravel(rv["dWaveOp"][k]) for k in ks]))
    np.savez_compressed(os.path.join(HERE, f"fwd_{name}.npz"), **out)
    print(f"fwd_{name}: nsteps={n} |dWaveOp snapshots|={np.linalg.norm(out['dwaveop']):.6e}")


def run_mig(name):
    """migrate_shot (temporal_modeling.py:171-214) of shot 0 at the starting model for a seeded
    data-space operand, imaging every step and every second step."""
    pysit = pysit_live.import_pysit()
    m, shots, solver, C, C0 = problems.build(pysit, name, kernel="cpp")
    m0 = solver.ModelParameters(m, {"C": C0})
    solver.model_parameters = m0
    tm = pysit.TemporalModeling(solver)
    op = np.random.default_rng(0).standard_normal((solver.nsteps, shots[0].receivers.receiver_count))
    out = dict(operand=op, nsteps=solver.nsteps)
    for p in (1, 2):
        out[f"image_p{p}"] = np.ravel(tm.migrate_shot(shots[0], m0, op, p).data)
    np.savez_compressed(os.path.join(HERE, f"mig_{name}.npz"), **out)
    print(f"mig_{name}: nsteps={solver.nsteps} |image|={np.linalg.norm(out['image_p1']):.6e}")


LBFGS_ITERS = 5


def run_lbfgs(name):
    """PySIT's own LBFGS (memory 10, backtracking line search) for LBFGS_ITERS
    iterations on the problem's data, with the cpp FP64 solver: objective and
    alpha histories, the function/gradient call counts and the final model."""
    pysit = pysit_live.import_pysit()
    m, shots, solver, C, C0 = problems.build(pysit, name, kernel="cpp")
    pysit.generate_seismic_data(shots, solver, solver.ModelParameters(m, {"C": C}))
    obj = pysit.TemporalLeastSquares(solver)
    calls = {"evaluate": 0, "gradient": 0}
    ev, gr = obj.evaluate, obj.compute_gradient

    def evaluate(*a, **k):
        calls["evaluate"] += 1
        return ev(*a, **k)

    def compute_gradient(*a, **k):
        calls["gradient"] += 1
        return gr(*a, **k)

    obj.evaluate, obj.compute_gradient = evaluate, compute_gradient
    opt = pysit.LBFGS(obj, memory_length=10)
    final = opt(shots, solver.ModelParameters(m, {"C": C0}), LBFGS_ITERS, line_search="backtrack",
                status_configuration={"objective_frequency": 1, "gradient_length_frequency": 1})
    _, objective = opt.retrieve_history("objective")
    _, alpha = opt.retrieve_history("alpha")
    _, gnorm = opt.retrieve_history("gradient_length")
    out = dict(objective=np.array(objective), alpha=np.array(alpha), gradient_length=np.array(gnorm),
               final_C=np.asarray(final.C).reshape(-1), n_evaluate=calls["evaluate"],
               n_gradient=calls["gradient"], iterations=LBFGS_ITERS)
    np.savez_compressed(os.path.join(HERE, f"lbfgs_{name}.npz"), **out)
    print(f"lbfgs_{name}: objective {out['objective']} alpha {out['alpha']} "
          f"evaluate {calls['evaluate']} gradient {calls['gradient']}")


BORN_SEED = 11
LEVENBERG_MU = 1e5


def born_perturbation(C0, seed=BORN_SEED):
    """The model perturbation of the Born / Hessian fixtures: 1 % of m0 = C0**-2, seeded noise."""
    rng = np.random.default_rng(seed)
    c0 = np.asarray(C0, float).reshape(-1)
    return 0.01 * rng.standard_normal(c0.size) / c0 ** 2


def run_born(name):
    """The reference's linear forward model (simdata of every shot, dWaveOp0 computed on the
    fly) and its Hessian applications (approximate, levenberg with LEVENBERG_MU, full) at the
    starting model, for the perturbation born_perturbation(C0).

    apply_hessian calls migrate_shot without its positional imaging_period
    (temporal_least_squares.py:217 against temporal_modeling.py:171), a TypeError; the
    migrate_shot used here supplies imaging_period = 1, the period of the dWaveOp0 lists."""
    pysit = pysit_live.import_pysit()
    m, shots, solver, C, C0 = problems.build(pysit, name, kernel="cpp")
    pysit.generate_seismic_data(shots, solver, solver.ModelParameters(m, {"C": C}))
    m0 = solver.ModelParameters(m, {"C": C0})
    m1v = born_perturbation(C0)
    m1 = m0.perturbation(data=m1v.reshape(-1, 1))
    obj = pysit.TemporalLeastSquares(solver)
    tm = obj.modeling_tools
    d1 = np.stack([tm.linear_forward_model(s, m0, m1, ["simdata"])["simdata"] for s in shots])
    mig = tm.migrate_shot

    def migrate_shot(shot, m0_, operand_simdata, imaging_period=1, *a, **k):
        return mig(shot, m0_, operand_simdata, imaging_period, *a, **k)

    tm.migrate_shot = migrate_shot
    out = dict(m1=m1v, d1=d1, dt0=solver.dt, nsteps0=solver.nsteps, levenberg_mu=LEVENBERG_MU)
    for mode in ("approximate", "levenberg", "full"):
        h = obj.apply_hessian(shots, m0, m1, hessian_mode=mode, levenberg_mu=LEVENBERG_MU)
        out[f"hess_{mode}"] = np.asarray(h.data).reshape(-1)
    np.savez_compressed(os.path.join(HERE, f"born_{name}.npz"), **out)
    print(f"born_{name}: |d1|={np.linalg.norm(d1):.6e} |H m1|={np.linalg.norm(out['hess_approximate']):.6e} "
          f"|H_full m1|={np.linalg.norm(out['hess_full']):.6e}")


if __name__ == "__main__":
    names = sys.argv[1:] or list(problems.SPECS)
    for n in names:
        if n.startswith("lbfgs:"):
            run_lbfgs(n.split(":", 1)[1])
        elif n.startswith("born:"):
            run_born(n.split(":", 1)[1])
        elif n.startswith("mig:"):
            run_mig(n.split(":", 1)[1])
        elif n.startswith("fwd:"):
            run_fwd(n.split(":", 1)[1])
        elif n.startswith("period:"):
            _, prob, per = n.split(":")
            run_period(prob, int(per))
        else:
            run(n)
