"""Optimizers (LBFGS, GradientDescent): the host logic against the reference's own
classes on a synthetic objective (runs where the reference tree is present), and the
history / iteration-parameter behaviour on its own."""
import os
import sys

import numpy as np
import pytest

import pysit_gb300 as api

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))


class _Solver:
    """Just what an optimizer touches: mesh, ModelParameters, model_parameters."""

    def __init__(self, mesh):
        self.mesh = mesh
        self.ModelParameters = api.ConstantDensityAcousticParameters
        self.model_parameters = None


class _Objective:
    """Synthetic misfit in m = C**-2: J = sum_i dV (a/2 d_i^2 + b/4 d_i^4), d = m - m_true.
    Its gradient for the cell-volume inner product is a d + b d^3, like the wave misfit's."""

    def __init__(self, mesh, m_true, a, b):
        self.solver = _Solver(mesh)
        self.m_true = m_true
        self.a, self.b = a, b
        self.dV = float(np.prod(mesh.deltas))
        self.n_eval = self.n_grad = 0

    def use_parallel(self):
        return False

    def _d(self, model):
        return model.linearize() - self.m_true

    def evaluate(self, shots, m0, **kwargs):
        self.n_eval += 1
        d = self._d(m0)
        return float(self.dV * np.sum(0.5 * self.a * d ** 2 + 0.25 * self.b * d ** 4))

    def compute_gradient(self, shots, m0, aux_info={}, **kwargs):
        self.n_grad += 1
        d = self._d(m0)
        if "objective_value" in aux_info:
            aux_info["objective_value"] = (True, self.evaluate(shots, m0))
        if "residual_norm" in aux_info:
            aux_info["residual_norm"] = (True, float(np.linalg.norm(d)))
        return m0.perturbation(data=self.a * d + self.b * d ** 3)


def _problem():
    d = api.RectangularDomain((0.0, 300.0, api.PML(40.0, 100.0), api.PML(40.0, 100.0)),
                              (0.0, 200.0, api.PML(40.0, 100.0), api.PML(40.0, 100.0)))
    m = api.CartesianMesh(d, 31, 21)
    x, z = m.mesh_coords()
    C_true = 2000.0 + 300.0 * np.sin(x / 60.0) * np.cos(z / 45.0)
    C0 = np.full_like(C_true, 2000.0)
    m_true = C_true ** -2
    # curvature of the quartic term comparable with the quadratic one at the start
    a = 1.0
    b = a / float(np.mean((C0 ** -2 - m_true) ** 2))
    return m, C0, m_true, a, b


def _run(cls, obj, m, C0, iters, line_search="backtrack", **kw):
    opt = cls(obj, **kw)
    start = api.ConstantDensityAcousticParameters(m, {"C": C0})
    final = opt([], start, iters, line_search=line_search,
                status_configuration={"value_frequency": 1, "objective_frequency": 1,
                                      "gradient_length_frequency": 1})
    return opt, final


def test_lbfgs_decreases_the_objective_and_keeps_histories():
    m, C0, m_true, a, b = _problem()
    obj = _Objective(m, m_true, a, b)
    opt, final = _run(api.LBFGS, obj, m, C0, 8, memory_length=4)
    it, vals = opt.retrieve_history("objective")
    assert list(it) == list(range(8))
    assert all(v1 < v0 for v0, v1 in zip(vals, vals[1:]))
    assert vals[-1] < 1e-3 * vals[0]
    it, alphas = opt.retrieve_history("alpha")
    assert len(alphas) == 8 and all(al > 0 for al in alphas)
    assert opt.retrieve_history("step") == (None, None)  # frequency 0: not kept
    assert len(opt.memory) == 4


def test_iteration_parameters_list_runs_each_entry():
    m, C0, m_true, a, b = _problem()
    obj = _Objective(m, m_true, a, b)
    opt, _ = _run(api.GradientDescent, obj, m, C0, [2, (3, {})])
    assert opt.iteration == 5 and obj.n_grad == 5
    with pytest.raises(ValueError):
        _run(api.GradientDescent, obj, m, C0, [2.5])


@pytest.fixture(scope="module")
def ref_optimization():
    import pysit_live
    if not pysit_live.available():
        pytest.skip("reference tree absent")
    return pysit_live.import_pysit()


@pytest.mark.parametrize("which,kw,ls", [("LBFGS", dict(memory_length=3), "backtrack"),
                                         ("LBFGS", dict(memory_length=None), "backtrack"),
                                         ("GradientDescent", {}, "backtrack"),
                                         ("LBFGS", dict(memory_length=5), ("constant", 0.5))])
def test_optimizer_matches_the_reference_class(ref_optimization, which, kw, ls):
    m, C0, m_true, a, b = _problem()
    o_ref = _Objective(m, m_true, a, b)
    opt_ref, fin_ref = _run(getattr(ref_optimization, which), o_ref, m, C0, 7, line_search=ls, **kw)
    o_new = _Objective(m, m_true, a, b)
    opt_new, fin_new = _run(getattr(api, which), o_new, m, C0, 7, line_search=ls, **kw)
    _, v_ref = opt_ref.retrieve_history("objective")
    _, v_new = opt_new.retrieve_history("objective")
    np.testing.assert_allclose(v_new, v_ref, rtol=1e-12, atol=0)
    _, a_ref = opt_ref.retrieve_history("alpha")
    _, a_new = opt_new.retrieve_history("alpha")
    np.testing.assert_allclose(a_new, a_ref, rtol=1e-12, atol=0)
    assert np.all(np.isfinite(fin_new.C)) and v_new[-1] < v_new[0]
    np.testing.assert_allclose(fin_new.C, fin_ref.C, rtol=1e-12, atol=0)
    assert (o_new.n_eval, o_new.n_grad) == (o_ref.n_eval, o_ref.n_grad)


# ---- Gauss-Newton and its Krylov solvers ------------------------------------------------

class _ObjectiveGN(_Objective):
    """_Objective with its Gauss-Newton Hessian H v = (a + 3 b d^2) v (same inner product)."""

    def __init__(self, *args):
        super().__init__(*args)
        self.n_hess = 0

    def apply_hessian(self, shots, m0, m1, hessian_mode="approximate", levenberg_mu=0.0, **kwargs):
        self.n_hess += 1
        d = self._d(m0)
        v = np.asarray(getattr(m1, "data", m1), dtype=float).reshape(d.shape)
        return m0.perturbation(data=(self.a + 3 * self.b * d ** 2) * v)


def test_gmres_and_cg_solve_small_systems():
    from pysit_gb300.optimization import krylov
    rng = np.random.default_rng(4)
    n = 40
    A = np.eye(n) * 4 + rng.standard_normal((n, n)) * 0.3
    b = rng.standard_normal(n)
    x_true = np.linalg.solve(A, b)
    res = []
    x, info = krylov.gmres(lambda v: A @ v, b, tol=1e-12, maxiter=n, residuals=res)
    assert info == 0 and np.linalg.norm(x - x_true) < 1e-9 * np.linalg.norm(x_true)
    assert res[0] == pytest.approx(np.linalg.norm(b)) and res[-1] <= 1e-12 * np.linalg.norm(b) * 1.0001
    # restarted: 10 cycles of 8
    x, info = krylov.gmres(A, b, tol=1e-10, restrt=8, maxiter=10)
    assert info == 0 and np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b) * 1.0001
    # too few iterations: info = iterations run, residual still decreasing
    res = []
    x, info = krylov.gmres(A, b, tol=1e-14, maxiter=3, residuals=res)
    assert info == 3 and len(res) == 4 and res[-1] < res[0]
    assert res[-1] == pytest.approx(np.linalg.norm(A @ x - b), rel=1e-8)
    # SPD system with cg
    S = A @ A.T + np.eye(n)
    x, info = krylov.cg(lambda v: S @ v, b, tol=1e-12, maxiter=200)
    assert info == 0 and np.linalg.norm(S @ x - b) <= 1e-11 * np.linalg.norm(b)
    x, info = krylov.gmres(A, np.zeros(n))
    assert info == 0 and not x.any()


def test_gauss_newton_converges_fast_and_keeps_histories():
    m, C0, m_true, a, b = _problem()
    obj = _ObjectiveGN(m, m_true, a, b)
    opt, final = _run(api.GaussNewton, obj, m, C0, 6, krylov_maxiter=10)
    _, vals = opt.retrieve_history("objective")
    assert all(v1 < v0 for v0, v1 in zip(vals, vals[1:]))
    assert vals[-1] < 1e-6 * vals[0]  # Newton: linear far out on the quartic, then quadratic
    assert vals[-1] / vals[-2] < 1e-3
    _, alphas = opt.retrieve_history("alpha")
    assert len(alphas) == 6 and alphas[0] <= 1.0
    assert obj.n_hess >= 6
    assert opt.krylov_residuals[-1] < opt.krylov_residuals[0]


def test_gauss_newton_matches_the_reference_class(ref_optimization, monkeypatch):
    """The reference's GaussNewton takes pyamg.krylov.gmres (absent here); with this package's
    gmres in its place both classes take the same steps on the same objective."""
    from pysit_gb300.optimization import krylov
    ref_gn = sys.modules[ref_optimization.GaussNewton.__module__]
    monkeypatch.setattr(ref_gn, "gmres", krylov.gmres)
    m, C0, m_true, a, b = _problem()
    o_ref = _ObjectiveGN(m, m_true, a, b)
    opt_ref, fin_ref = _run(ref_optimization.GaussNewton, o_ref, m, C0, 3, krylov_maxiter=6)
    o_new = _ObjectiveGN(m, m_true, a, b)
    opt_new, fin_new = _run(api.GaussNewton, o_new, m, C0, 3, krylov_maxiter=6)
    _, v_ref = opt_ref.retrieve_history("objective")
    _, v_new = opt_new.retrieve_history("objective")
    np.testing.assert_allclose(v_new, v_ref, rtol=1e-12, atol=0)
    _, a_ref = opt_ref.retrieve_history("alpha")
    _, a_new = opt_new.retrieve_history("alpha")
    np.testing.assert_allclose(a_new, a_ref, rtol=1e-12, atol=0)
    np.testing.assert_allclose(fin_new.C, fin_ref.C, rtol=1e-12, atol=0)
    assert (o_new.n_eval, o_new.n_grad, o_new.n_hess) == (o_ref.n_eval, o_ref.n_grad, o_ref.n_hess)
