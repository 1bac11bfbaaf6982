"""Cartesian mesh with PML / Dirichlet padding (mirror of pysit.core.mesh).

Semantics followed (pysit/core/mesh.py):
  * ``CartesianMesh(domain, *n)``: ``delta = length / (n - 1)`` per axis (:171-206);
  * the padded shape adds ``lbc.n + rbc.n`` nodes per axis (:307-339); arrays are
    C-ordered with z fastest, vectors are column vectors ``(dof, 1)``;
  * a PML side pads ``n = ceil(width / delta)`` nodes and stores the profile
    ``sigma``: the PML profile evaluated on ``n + 1`` points of [0, 1] without the
    node on the physical boundary (:749-782); a Dirichlet side pads nothing;
  * ``eval_on_mesh`` spreads one side's profile over the padded grid (:784-831);
  * ``pad_array`` / ``unpad_array`` (:385-533).
"""
from __future__ import annotations

import math

import numpy as np

from .domain import Bunch

__all__ = ["CartesianMesh", "StructuredPML", "StructuredDirichlet"]

_AXES = {1: ["z"], 2: ["x", "z"], 3: ["x", "y", "z"]}


class StructuredBC:
    type = None
    boundary_type = None

    def __init__(self, mesh, domain_bc, dim, side, delta):
        self.mesh = mesh
        self.domain_bc = domain_bc
        self.dim = dim
        self.side = side
        self._n = 0
        self.solver_padding = 1

    @property
    def n(self):
        return self._n


class StructuredDirichlet(StructuredBC):
    type = "dirichlet"
    boundary_type = "dirichlet"


class StructuredPML(StructuredBC):
    type = "pml"

    def __init__(self, mesh, domain_bc, dim, side, delta):
        super().__init__(mesh, domain_bc, dim, side, delta)
        self._n = int(np.ceil(domain_bc.length / delta))
        s = domain_bc.evaluate(self._n + 1, side)
        # the extra evaluation point is the physical boundary node itself
        self.sigma = s[1:] if side == "right" else s[:-1]
        self.boundary_type = domain_bc.boundary_type

    def eval_on_mesh(self):
        """Profile of this side broadcast over the padded grid, as a (dof, 1) column."""
        shape = self.mesh.shape(include_bc=True, as_grid=True)
        out = np.zeros(shape)
        sl = [slice(None)] * self.mesh.dim
        view_shape = [1] * self.mesh.dim
        view_shape[self.dim] = -1
        if self.side == "left":
            sl[self.dim] = slice(0, self._n)
        else:
            sl[self.dim] = slice(shape[self.dim] - self._n, None)
        out[tuple(sl)] = self.sigma.reshape(view_shape)
        return out.reshape(self.mesh.shape(include_bc=True, as_grid=False))


def _mesh_bc(mesh, domain_bc, dim, side, delta):
    if domain_bc.type == "pml":
        return StructuredPML(mesh, domain_bc, dim, side, delta)
    if domain_bc.type == "dirichlet":
        return StructuredDirichlet(mesh, domain_bc, dim, side, delta)
    raise NotImplementedError(f"boundary condition '{domain_bc.type}' is not supported by the time solvers")


class CartesianMesh:
    """Structured Cartesian mesh over a RectangularDomain."""
    type = "structured-cartesian"

    def __init__(self, domain, *axis_nodes):
        if not 1 <= len(axis_nodes) <= 3:
            raise ValueError("Mesh dimension must be between 1 and 3.")
        if len(axis_nodes) != domain.dim:
            raise ValueError("Mesh dimension must match domain dimension.")
        self.domain = domain
        self.dim = domain.dim
        self.parameters = {}
        for i, key in enumerate(_AXES[self.dim]):
            n = int(axis_nodes[i])
            delta = domain.parameters[i].length / (n - 1)
            p = Bunch(n=n, delta=delta)
            p.lbc = _mesh_bc(self, domain.parameters[i].lbc, i, "left", delta)
            p.rbc = _mesh_bc(self, domain.parameters[i].rbc, i, "right", delta)
            self.parameters[i] = p
            self.parameters[key] = p
            setattr(self, key, p)
        self._shapes = {}
        self._dofs = {}

    @property
    def deltas(self):
        return tuple(self.parameters[i].delta for i in range(self.dim))

    def _compute_shape(self, include_bc):
        sh = []
        for i in range(self.dim):
            p = self.parameters[i]
            n = p.n + (p.lbc.n + p.rbc.n if include_bc else 0)
            sh.append(n)
        self._shapes[(include_bc, True)] = sh
        self._shapes[(include_bc, False)] = (int(np.prod(sh)), 1)
        self._dofs[include_bc] = int(np.prod(sh))

    def shape(self, include_bc=False, as_grid=False):
        if (include_bc, as_grid) not in self._shapes:
            self._compute_shape(include_bc)
        return self._shapes[(include_bc, as_grid)]

    def dof(self, include_bc=False):
        if include_bc not in self._dofs:
            self._compute_shape(include_bc)
        return self._dofs[include_bc]

    def pad_widths(self):
        """[(left, right)] padding nodes per axis."""
        return [(self.parameters[i].lbc.n, self.parameters[i].rbc.n) for i in range(self.dim)]

    def mesh_coords(self, sparse=False, include_bc=False):
        rows = []
        for i in range(self.dim):
            p = self.parameters[i]
            d = self.domain.parameters[i]
            if include_bc:
                rows.append(np.linspace(d.lbound - p.lbc.n * p.delta, d.rbound + p.rbc.n * p.delta,
                                        p.n + p.lbc.n + p.rbc.n))
            else:
                rows.append(np.linspace(d.lbound, d.rbound, p.n))
        if self.dim == 1:
            tup = (rows[0],)
        else:
            tup = np.meshgrid(*rows, sparse=sparse, indexing="ij")
        if not sparse:
            tup = tuple(x.reshape(self.shape(include_bc)) for x in tup)
        return tup

    def nodes(self, include_bc=False):
        return np.hstack(self.mesh_coords(include_bc=include_bc))

    def unpad_array(self, in_array, copy=False):
        sh_g = self.shape(include_bc=False, as_grid=True)
        sh_v = self.shape(include_bc=False, as_grid=False)
        if tuple(in_array.shape) in (tuple(sh_g), tuple(sh_v)):
            out = in_array
        else:
            full = self.shape(include_bc=True, as_grid=True)
            sl = tuple(slice(self.parameters[i].lbc.n, full[i] - self.parameters[i].rbc.n)
                       for i in range(self.dim))
            out = in_array.reshape(full)[sl]
        if in_array.ndim == 2 and in_array.shape[1] == 1:
            out = out.reshape(-1, 1)
        return out.copy() if copy else out

    def pad_array(self, in_array, out_array=None, padding_mode=None):
        sh_in_v = tuple(self.shape(include_bc=False, as_grid=False))
        sh_in_g = self.shape(include_bc=False, as_grid=True)
        sh_out_v = self.shape(include_bc=True, as_grid=False)
        sh_out_g = self.shape(include_bc=True, as_grid=True)
        # a caller's out_array is filled through a grid-shaped view of it (the reference
        # reshapes it in place; the returned array has the reference's shape either way)
        if out_array is not None:
            grid = out_array.reshape(sh_out_g)
            if not np.shares_memory(grid, out_array):
                raise ValueError("out_array must be contiguous")
        if padding_mode is not None:
            pads = tuple((self.parameters[i].lbc.n, self.parameters[i].rbc.n) for i in range(self.dim))
            padded = np.pad(np.asarray(in_array).reshape(sh_in_g), pads, mode=padding_mode)
            if out_array is not None:
                grid[:] = padded
            else:
                grid = padded
        else:
            if out_array is None:
                grid = np.zeros(sh_out_g, dtype=in_array.dtype)
            sl = tuple(slice(self.parameters[i].lbc.n, sh_out_g[i] - self.parameters[i].rbc.n)
                       for i in range(self.dim))
            grid[sl] = np.asarray(in_array).reshape(sh_in_g)
        return grid.reshape(sh_out_v if tuple(in_array.shape) == sh_in_v else sh_out_g)

    def inner_product(self, a, b):
        return np.dot(np.ravel(a), np.ravel(b)) * math.prod(self.deltas)
