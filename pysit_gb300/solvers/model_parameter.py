"""Model parameters and perturbations (mirror of pysit.solvers.model_parameter).

Semantics followed (pysit/solvers/model_parameter.py):
  * a model stores the nonlinear wave speed C as a (dof, 1) column; arithmetic
    acts on the linear form m = C**-2 (WaveSpeed.linearize, :80-92;
    ModelParameterBase.__add__/__sub__/__mul__, :306-420);
  * model - model and model - perturbation give a perturbation in linear form;
  * ``with_padding(padding_mode='edge')`` pads with numpy.pad (:262-276) as the
    solver does on assignment (solver_base.py:107-117);
  * a perturbation's ``add_padding`` sums every PML strip onto the adjacent
    boundary row/column and drops the padding (:537-594);
  * ``inner_product`` is the mesh inner product (sum * prod(deltas)).
"""
from __future__ import annotations

import numpy as np

__all__ = ["ConstantDensityAcousticParameters", "WaveSpeed", "fold_padding"]


class WaveSpeed:
    name = "C"

    @staticmethod
    def linearize(data):
        return data ** -2

    @staticmethod
    def unlinearize(data):
        return np.sqrt(1.0 / data)

    @staticmethod
    def validate(data):
        if not np.all(np.isfinite(data)):
            return False, "finite"
        if not np.all(data > 0):
            return False, "positivity"
        return True, None


def fold_padding(mesh, padded):
    """Fold the PML strips of a padded grid array onto the physical boundary and
    return the unpadded array (ModelPerturbationBase.add_padding semantics)."""
    full = mesh.shape(include_bc=True, as_grid=True)
    a = np.array(padded, dtype=float).reshape(full)
    sl = []
    for ax in range(mesh.dim):
        lo, hi = mesh.parameters[ax].lbc.n, mesh.parameters[ax].rbc.n
        n_in = full[ax] - lo - hi
        idx = [slice(None)] * mesh.dim
        first = list(idx); first[ax] = lo
        last = list(idx); last[ax] = lo + n_in - 1
        left = list(idx); left[ax] = slice(0, lo)
        right = list(idx); right[ax] = slice(lo + n_in, full[ax])
        a[tuple(first)] += a[tuple(left)].sum(axis=ax)
        a[tuple(last)] += a[tuple(right)].sum(axis=ax)
        sl.append(slice(lo, lo + n_in))
    return a[tuple(sl)].reshape(-1, 1)


class _Perturbation:
    """Linear model perturbation (m-space), (dof, 1) column."""

    parameter_list = [WaveSpeed]

    def __init__(self, mesh, padded=False, inputs=None, dtype=np.double, **kwargs):
        self.mesh = mesh
        self.padded = padded
        self.dtype = dtype
        dof = mesh.dof(include_bc=padded)
        self.data = np.zeros((dof, 1), dtype=dtype)
        if inputs is not None:
            if isinstance(inputs, dict):
                inputs = inputs.get("C", 0.0)
            if isinstance(inputs, (list, tuple)):
                inputs = inputs[0]
            arr = np.asarray(inputs, dtype=dtype)
            if arr.size not in (1, dof):
                raise ValueError("Improper dimensions for input array.")
            self.data[:] = arr.reshape(-1, 1) if arr.size == dof else arr

    parameter_count = property(lambda self: 1)

    @property
    def C(self):
        return self.data

    @C.setter
    def C(self, v):
        self.data[:] = v

    def _new(self, data):
        return type(self)(self.mesh, padded=self.padded, inputs=data, dtype=self.dtype)

    @staticmethod
    def _val(rhs):
        return rhs.data if isinstance(rhs, _Perturbation) else rhs

    def __add__(self, rhs):
        if isinstance(rhs, ConstantDensityAcousticParameters):
            return rhs.__add__(self)
        return self._new(self.data + self._val(rhs))

    __radd__ = __add__

    def __iadd__(self, rhs):
        self.data += self._val(rhs)
        return self

    def __sub__(self, rhs):
        return self._new(self.data - self._val(rhs))

    def __rsub__(self, lhs):
        return self._new(self._val(lhs) - self.data)

    def __isub__(self, rhs):
        self.data -= self._val(rhs)
        return self

    def __mul__(self, rhs):
        if isinstance(rhs, _Perturbation):
            return self.data * rhs.data
        if isinstance(rhs, np.ndarray) and rhs.shape == self.data.shape:
            return self.data * rhs
        return self._new(rhs * self.data)

    __rmul__ = __mul__

    def __imul__(self, rhs):
        self.data *= self._val(rhs)
        return self

    def __neg__(self):
        return self._new(-self.data)

    def __truediv__(self, rhs):
        return self._new(self.data / rhs)

    def asarray(self):
        return self.data

    def norm(self, ord=None):
        return np.linalg.norm(self.data, ord=ord)

    @property
    def T(self):
        return self.data.T

    def inner_product(self, other):
        if not isinstance(other, _Perturbation):
            raise ValueError("Perturbation inner product is only defined for perturbations.")
        return float(self.mesh.inner_product(self.data, other.data))

    def without_padding(self):
        if not self.padded:
            return self
        return type(self)(self.mesh, padded=False, inputs=self.mesh.unpad_array(self.data, copy=True),
                          dtype=self.dtype)

    def with_padding(self, **kwargs):
        if self.padded:
            return self
        return type(self)(self.mesh, padded=True, inputs=self.mesh.pad_array(self.data, **kwargs),
                          dtype=self.dtype)

    def add_padding(self):
        return type(self)(self.mesh, padded=False, inputs=fold_padding(self.mesh, self.data), dtype=self.dtype)

    def __deepcopy__(self, memo):
        return type(self)(self.mesh, padded=self.padded, inputs=self.data.copy(), dtype=self.dtype)

    def __repr__(self):
        return repr(self.data)


class ConstantDensityAcousticParameters:
    """Wave-speed model C of the constant-density acoustic equation."""

    parameter_list = [WaveSpeed]

    class Perturbation(_Perturbation):
        pass

    def __init__(self, mesh, inputs=None, linear_inputs=None, padded=False, **kwargs):
        self.mesh = mesh
        self.padded = padded
        dof = mesh.dof(include_bc=padded)
        self.data = np.ones((dof, 1)) * np.inf
        if inputs is not None:
            if isinstance(inputs, dict):
                if "C" in inputs:
                    self.data[:] = np.asarray(inputs["C"], dtype=float).reshape(-1, 1) \
                        if np.size(inputs["C"]) == dof else inputs["C"]
            elif isinstance(inputs, (list, tuple)):
                self.data[:] = np.asarray(inputs[0], dtype=float).reshape(-1, 1)
            elif isinstance(inputs, np.ndarray):
                if inputs.size != dof:
                    raise ValueError("Improper dimensions for input array.")
                self.data = inputs.reshape(-1, 1)
            else:
                raise ValueError("Invalid format for collection of input parameters.")
        if linear_inputs is not None:
            self.data[:] = WaveSpeed.unlinearize(np.asarray(linear_inputs, dtype=float).reshape(-1, 1))

    parameter_count = property(lambda self: 1)

    @property
    def C(self):
        return self.data

    @C.setter
    def C(self, v):
        self.data[:] = v

    def perturbation(self, data=None, *args, **kwargs):
        return self.Perturbation(self.mesh, padded=self.padded, inputs=data, **kwargs)

    def linearize(self, asperturbation=False):
        out = WaveSpeed.linearize(self.data)
        return self.perturbation(out) if asperturbation else out

    def validate(self, raise_exception=False):
        ok, why = WaveSpeed.validate(self.data)
        if not ok and raise_exception:
            raise Exception(f"Validation of model failed: {why}")
        return ok

    def with_padding(self, **kwargs):
        if self.padded:
            return self
        return type(self)(self.mesh, inputs=self.mesh.pad_array(self.data, **kwargs), padded=True)

    def without_padding(self):
        if not self.padded:
            return self
        return type(self)(self.mesh, inputs=self.mesh.unpad_array(self.data, copy=True), padded=False)

    def _lin(self, rhs):
        if isinstance(rhs, ConstantDensityAcousticParameters):
            return WaveSpeed.linearize(rhs.data)
        if isinstance(rhs, _Perturbation):
            return rhs.data
        return rhs

    def __add__(self, rhs):
        return type(self)(self.mesh, padded=self.padded,
                          inputs=WaveSpeed.unlinearize(WaveSpeed.linearize(self.data) + self._lin(rhs)))

    __radd__ = __add__

    def __sub__(self, rhs):
        if isinstance(rhs, (ConstantDensityAcousticParameters, _Perturbation)):
            return self.perturbation(WaveSpeed.linearize(self.data) - self._lin(rhs))
        return self.perturbation(WaveSpeed.linearize(self.data) - rhs)

    def __mul__(self, rhs):
        if isinstance(rhs, _Perturbation):
            return WaveSpeed.linearize(self.data) * rhs.data
        if isinstance(rhs, np.ndarray) and rhs.shape == self.data.shape:
            return WaveSpeed.linearize(self.data) * rhs
        return type(self)(self.mesh, padded=self.padded,
                          inputs=WaveSpeed.unlinearize(rhs * WaveSpeed.linearize(self.data)))

    __rmul__ = __mul__

    def asarray(self):
        return self.data

    def norm(self, ord=None):
        return np.linalg.norm(self.data, ord=ord)

    @property
    def T(self):
        return self.data.T

    def __deepcopy__(self, memo):
        return type(self)(self.mesh, padded=self.padded, inputs=self.data.copy())

    def __repr__(self):
        return repr(self.data)
