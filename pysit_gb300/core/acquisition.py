"""Sources, receivers, wavelets and shots (mirror of pysit.core acquisition classes).

Semantics followed (paths inside the reference project):
  * point representation, pysit/core/mesh_representation.py:115-212: a point is
    smeared by a Gaussian of standard deviation ``max(deltas) * approximation_width``
    evaluated on the unpadded grid nodes within
    ``ceil(round(deviations*sigma/delta, 3))`` nodes of the nearest node
    (``int(round((pos - lbound)/delta))``), normalised by
    ``1/((sqrt(2 pi) sigma)**dim)``; or a single 'delta' node of weight 1/prod(deltas).
    The sampling operator is ``base * prod(deltas)``, its adjoint ``base.T``;
  * ``PointSource.f(t) = adjoint_sampling_operator * (intensity * w(t))``
    (pysit/core/sources.py:106-129);
  * ``DerivativeGaussianPulse`` / ``RickerWavelet`` (pysit/core/wave_source.py:100-203):
    ``x = (t - t_shift)/(sqrt(2) sigma)``, ``sigma = 1/(pi nu sqrt(2))``,
    ``t_shift = 6 sigma``, value ``(-1/sqrt2)**n H_n(x) exp(-x^2)`` dropped below
    ``threshold``; the Ricker wavelet is minus the n = 2 pulse;
  * ``ReceiverSet`` (pysit/core/receivers.py:362-564): stacked sampling operator,
    ``interpolate_data`` = linear interpolation with zero fill outside the
    recorded time axis (scipy interp1d, receivers.py:56-105);
  * ``equispaced_acquisition`` (pysit/core/acquisition.py:14-103).
Taps are exposed as plain arrays for the GPU pipeline (``taps()``).
"""
from __future__ import annotations

import copy
import math
from functools import reduce

import numpy as np
import scipy.sparse as spsp

__all__ = ["DerivativeGaussianPulse", "RickerWavelet", "GaussianPulse", "PointSource", "SourceSet",
           "PointReceiver", "ReceiverSet", "Shot", "SourceEncodedSupershot", "equispaced_acquisition",
           "linear_interpolate"]

_SQRT2 = math.sqrt(2.0)


# ---------------------------------------------------------------------------
# wavelets
# ---------------------------------------------------------------------------
class DerivativeGaussianPulse:
    """n-th derivative of a Gaussian pulse, time domain."""

    time_source = True
    frequency_source = True

    def __init__(self, peak_frequency, order=0, threshold=1e-6, shift_deviations=6, t_shift=None):
        self._order = order
        self.peak_frequency = peak_frequency
        self.threshold = threshold
        self.shift_deviations = shift_deviations
        self.sigma = 1 / (math.pi * peak_frequency * _SQRT2)
        self.t_shift = shift_deviations * self.sigma if t_shift is None else t_shift
        self._hermite = np.polynomial.Hermite([0.0] * order + [1.0])

    @property
    def order(self):
        return self._order

    def _pulse(self, ts):
        ts = np.atleast_1d(np.asarray(ts, dtype=float))
        n = self.order
        x = (ts - self.t_shift) / (_SQRT2 * self.sigma)
        v = ((-1 / _SQRT2) ** n) * self._hermite(x) * np.exp(-(x ** 2))
        v[np.abs(v) < self.threshold] = 0.0
        return v

    def _evaluate_time(self, ts):
        return self._pulse(ts)

    def _evaluate_frequency(self, nus):
        nus = np.atleast_1d(np.asarray(nus, dtype=float))
        w = 2 * np.pi * nus
        n = self.order
        v = (math.sqrt(2 * np.pi) * (-1) ** n * (1j * w) ** n * self.sigma ** (n + 1)
             * np.exp(-0.5 * self.sigma ** 2 * w ** 2) * np.exp(-1j * 2 * np.pi * nus * self.t_shift))
        v[np.abs(v) < self.threshold] = 0.0
        return v

    def __call__(self, t=None, nu=None, **kwargs):
        scalar = t is not None and not np.iterable(t)
        if t is not None:
            v = self._evaluate_time(t)
        elif nu is not None:
            scalar = not np.iterable(nu)
            v = self._evaluate_frequency(nu)
        else:
            raise ValueError("Either a time or frequency must be provided.")
        return v[0] if scalar else v


class RickerWavelet(DerivativeGaussianPulse):
    """Negative second derivative of a Gaussian (Ricker 1953)."""

    def __init__(self, nu, **kwargs):
        kwargs.pop("order", None)
        super().__init__(nu, order=2, **kwargs)

    def _evaluate_time(self, ts):
        return -1 * self._pulse(ts)

    def _evaluate_frequency(self, nus):
        return -1 * super()._evaluate_frequency(nus)


class GaussianPulse(DerivativeGaussianPulse):
    def __init__(self, nu, **kwargs):
        kwargs.pop("order", None)
        super().__init__(nu, order=0, **kwargs)


# ---------------------------------------------------------------------------
# point representation
# ---------------------------------------------------------------------------
class _PointRepresentation:
    def __init__(self, mesh, pos, approximation="gaussian", approximation_width=1,
                 approximation_deviations=3, **kwargs):
        self.mesh = mesh
        self.domain = mesh.domain
        self.deltas = mesh.deltas
        self._prod_deltas = float(np.prod(self.deltas))
        dim = self.domain.dim
        if dim == 1 and not isinstance(pos, tuple):
            pos = (pos,)
        self.position = tuple(pos)
        self.approximation = approximation
        self.approximation_width = approximation_width
        self.approximation_deviations = approximation_deviations
        shape = mesh.shape(as_grid=True)
        mins = self.domain.collect("lbound")
        if approximation == "gaussian":
            grid = mesh.mesh_coords(sparse=True)
            sigma = max(self.deltas) * approximation_width
            width = np.ceil(np.around(approximation_deviations * sigma / np.array(self.deltas), 3)).astype(int)
            gc = [int(round((p - m) / d)) for m, d, p in zip(mins, self.deltas, self.position)]
            ranges = [list(range(max(0, c - w), min(g.size, c + w + 1))) for g, w, c in zip(grid, width, gc)]
            windows = [np.asarray(g).flatten()[r] for g, r in zip(grid, ranges)]
            if dim == 1:
                idx_grids = (np.array(ranges[0]),)
                sub = (np.array(windows[0]),)
            else:
                idx_grids = np.meshgrid(*ranges)
                sub = np.meshgrid(*windows)
            norm = 1.0 / ((np.sqrt(2 * np.pi) ** dim) * (sigma ** dim))
            data = norm * np.exp((-0.5 / sigma ** 2) * reduce(lambda a, b: a + b,
                                                              [(s - p) ** 2 for s, p in zip(sub, self.position)]))
            idx = np.ravel_multi_index(np.array([g.flatten() for g in idx_grids]).astype(int), shape)
            self._indices = idx.astype(np.int64)
            self._base = data.flatten().astype(float)
        elif approximation == "delta":
            gc = tuple(int(round((p - m) / d)) for m, d, p in zip(mins, self.deltas, self.position))
            self._indices = np.array([np.ravel_multi_index(gc, shape)], dtype=np.int64)
            self._base = np.array([1.0 / self._prod_deltas])
        else:
            raise ValueError("Only 'delta' and 'gaussian' are valid approximations for a point source or receiver.")

    @property
    def sampling_operator(self):
        dof = self.mesh.dof()
        return spsp.csr_matrix((self._base * self._prod_deltas, self._indices,
                                np.array([0, len(self._indices)])), shape=(1, dof))

    @property
    def adjoint_sampling_operator(self):
        dof = self.mesh.dof()
        return spsp.csr_matrix((self._base, self._indices, np.array([0, len(self._indices)])),
                               shape=(1, dof)).T.tocsr()


# ---------------------------------------------------------------------------
# sources
# ---------------------------------------------------------------------------
class PointSource(_PointRepresentation):
    """Point source ``intensity * w(t)`` smeared on the grid."""

    def __init__(self, mesh, pos, src_func, intensity=1.0, **kwargs):
        super().__init__(mesh, pos, **kwargs)
        self.w = src_func
        self.intensity = intensity
        self.shot = None

    source_count = property(lambda self: 1)

    def set_shot(self, shot):
        self.shot = shot

    def reset_time_series(self, ts):
        pass

    def f(self, t=0.0, nu=None, **kwargs):
        """Source term on the unpadded grid as a (dof, 1) column (sources.py:106-129)."""
        out = np.zeros((self.mesh.dof(), 1))
        amp = self.intensity * (self.w(t, **kwargs) if nu is None else self.w(nu=nu, **kwargs))
        np.add.at(out[:, 0], self._indices, self._base * amp)
        return out

    def taps(self):
        """(unpadded cell, point, weight) of the injection operator S*."""
        return self._indices, np.zeros(len(self._indices), np.int32), self._base

    def amplitudes(self, ts):
        """[nsteps, 1] amplitudes intensity * w(t_k) of the single source point."""
        return (self.intensity * np.asarray(self.w(np.asarray(ts)), dtype=float)).reshape(-1, 1)


class SourceSet:
    """Several point sources fired together (one shot, several injection points)."""

    def __init__(self, mesh, sources):
        self.mesh = mesh
        self.source_list = list(sources)
        self.shot = None

    source_count = property(lambda self: len(self.source_list))

    def set_shot(self, shot):
        self.shot = shot

    def reset_time_series(self, ts):
        pass

    def f(self, t=0.0, **kwargs):
        return sum(s.f(t, **kwargs) for s in self.source_list)

    def taps(self):
        cells, pts, ws = [], [], []
        for i, s in enumerate(self.source_list):
            c, _, w = s.taps()
            cells.append(c); pts.append(np.full(len(c), i, np.int32)); ws.append(w)
        return np.concatenate(cells), np.concatenate(pts), np.concatenate(ws)

    def amplitudes(self, ts):
        return np.hstack([s.amplitudes(ts) for s in self.source_list])


# ---------------------------------------------------------------------------
# receivers
# ---------------------------------------------------------------------------
def linear_interpolate(ts_src, data, ts_new):
    """Linear interpolation along axis 0 with zero fill outside [ts_src[0], ts_src[-1]].

    Restates scipy.interpolate.interp1d(kind='linear', bounds_error=False,
    fill_value=0) as used by ReceiverBase.interpolate_data (receivers.py:56-105):
    the interval is found with searchsorted(side='left') clipped to [1, n-1] and
    the value is ``slope * (t - t_lo) + y_lo``.
    """
    ts_src = np.asarray(ts_src, dtype=float)
    ts_new = np.atleast_1d(np.asarray(ts_new, dtype=float))
    y = np.asarray(data, dtype=float)
    n = len(ts_src)
    out = np.zeros((len(ts_new),) + y.shape[1:])
    if n == 0:
        return out
    if n == 1:
        hit = ts_new == ts_src[0]
        out[hit] = y[0]
        return out
    idx = np.clip(np.searchsorted(ts_src, ts_new, side="left"), 1, n - 1)
    lo = idx - 1
    x_lo, x_hi = ts_src[lo], ts_src[idx]
    slope = (y[idx] - y[lo]) / (x_hi - x_lo).reshape((-1,) + (1,) * (y.ndim - 1))
    val = slope * (ts_new - x_lo).reshape((-1,) + (1,) * (y.ndim - 1)) + y[lo]
    inside = (ts_new >= ts_src[0]) & (ts_new <= ts_src[-1])
    out[inside] = val[inside]
    return out


class _ReceiverBase:
    def __init__(self):
        self.ts = None
        self._data = None
        self.shot = None

    def set_shot(self, shot):
        self.shot = shot

    def reset_time_series(self, ts):
        self.ts = np.asarray(ts, dtype=float)
        self.clear_data(len(ts))

    def interpolate_data(self, ts):
        if self.ts is None:
            raise TypeError("Interpolator has not been defined for the current receiver.")
        return linear_interpolate(self.ts, self.data, ts)

    data = property(lambda self: self._data, lambda self, v: setattr(self, "_data", v))


class PointReceiver(_PointRepresentation, _ReceiverBase):
    """Single receiver (samples u at a smeared point)."""

    def __init__(self, mesh, pos, **kwargs):
        _PointRepresentation.__init__(self, mesh, pos, **kwargs)
        _ReceiverBase.__init__(self)

    receiver_count = property(lambda self: 1)

    def clear_data(self, n):
        self.data = np.zeros((n, 1))

    def taps(self):
        """(unpadded cell, receiver, sampling weight, injection weight)."""
        return (self._indices, np.zeros(len(self._indices), np.int32), self._base * self._prod_deltas,
                self._base)

    def sample_data_from_array(self, arr, k=None, data=None):
        v = float(np.dot(self._base * self._prod_deltas, np.ravel(arr)[self._indices]))
        if k is None:
            return v
        (self.data if data is None else data)[k] = v

    def extend_data_to_array(self, k=None, data=None):
        d = (self.data if data is None else data)
        val = d[k] if k is not None else d
        out = np.zeros((self.mesh.dof(), 1))
        np.add.at(out[:, 0], self._indices, self._base * float(np.ravel(val)[0]))
        return out


class ReceiverSet(_ReceiverBase):
    """Set of point receivers recorded together."""

    def __init__(self, mesh, receivers, **kwargs):
        super().__init__()
        self.mesh = mesh
        self.receiver_list = list(receivers)
        self._prod_deltas = float(np.prod(mesh.deltas))

    receiver_count = property(lambda self: sum(r.receiver_count for r in self.receiver_list))

    def set_shot(self, shot):
        self.shot = shot
        for r in self.receiver_list:
            r.set_shot(shot)

    def clear_data(self, n):
        self.data = np.zeros((n, self.receiver_count))

    def taps(self):
        cells, recs, ws, wi = [], [], [], []
        for i, r in enumerate(self.receiver_list):
            c, _, s, a = r.taps()
            cells.append(c); recs.append(np.full(len(c), i, np.int32)); ws.append(s); wi.append(a)
        return np.concatenate(cells), np.concatenate(recs), np.concatenate(ws), np.concatenate(wi)

    @property
    def sampling_operator(self):
        return spsp.vstack([r.sampling_operator for r in self.receiver_list]).tocsr()

    @property
    def adjoint_sampling_operator(self):
        return spsp.hstack([r.adjoint_sampling_operator for r in self.receiver_list]).tocsr()

    def sample_data_from_array(self, arr, k=None, data=None):
        v = np.asarray(self.sampling_operator @ np.ravel(arr)).reshape(1, -1)
        if k is None:
            return v
        (self.data if data is None else data)[k, :] = v

    def extend_data_to_array(self, k=None, data=None):
        d = (self.data if data is None else data)
        val = np.asarray(d[k, :] if k is not None else d, dtype=float).reshape(-1)
        return np.asarray(self.adjoint_sampling_operator @ val).reshape(-1, 1)


class Shot:
    """A seismic shot: sources fired together and the receivers recording them."""

    def __init__(self, sources, receivers):
        self.receivers = receivers
        receivers.set_shot(self)
        self.sources = sources
        sources.set_shot(self)

    def initialize(self, data_length):
        self.receivers.clear_data(data_length)

    def reset_time_series(self, ts):
        self.sources.reset_time_series(ts)
        self.receivers.reset_time_series(ts)

    def gather(self, as_array=False, offset=None):
        if offset is not None:
            raise NotImplementedError("Gather by offset not yet implemented.")
        return self.receivers.data if as_array else self.receivers


class SourceEncodedSupershot(Shot):
    """Source-encoded supershot (pysit/core/shot.py:148-345), time domain.

    The member shots' point sources fire together, source i with intensity code_i; the
    observed data are encoded the same way, sum_i code_i d_i.  Codes are i.i.d. standard
    normal ('gaussian') or +-1 with equal odds ('krebs'); ``encode()`` draws new ones.
    The members must have point sources, the same receivers (fixed spread: identical
    sampling operators) and recorded time data.  On the GPU a supershot is one shot of
    the batched plan with one injection point per member source.

    The reference class cannot be constructed: its encoded source set calls
    ``super().__init__(self, ...)`` (shot.py:196), a TypeError, and its 'krebs' codes use
    ``np.random.random_integers``, removed from numpy.  Here the set is a SourceSet of
    copies of the member sources and 'krebs' draws ``randint(0, 2)`` (the same draw).
    Codes come from numpy's global generator as in the reference, or from ``rng`` (a
    numpy Generator) when given.  The frequency-domain branch is outside this path.
    """

    def __init__(self, shots, weight_type="gaussian", rng=None):
        self.weight_type = weight_type
        self._rng = rng
        self.encoding = 0  # bumped by every encode(); plans built for an older encoding are not reused
        self.sequential_shots = shots

    def generate_weight_vector(self):
        n = self._nshots
        if self.weight_type == "gaussian":
            return self._rng.standard_normal(n) if self._rng is not None else np.random.randn(n)
        if self.weight_type == "krebs":
            draw = self._rng.integers(0, 2, n) if self._rng is not None else np.random.randint(0, 2, n)
            return 2 * draw - 1
        raise Exception("Incorrect weight type supplied.")

    def encode(self, codes=None):
        """Draw new codes (or take `codes`), rebuild the encoded sources and data."""
        import copy
        shots = self._sequential_shots
        codes = self.generate_weight_vector() if codes is None else np.asarray(codes, dtype=float)
        if len(codes) != self._nshots:
            raise ValueError("one code per member shot is needed")
        sources = []
        for shot, c in zip(shots, codes):
            src = copy.copy(shot.sources)
            src.intensity = float(c) * shot.sources.intensity
            sources.append(src)
        enc = SourceSet(shots[0].sources.mesh, sources)
        receivers = copy.deepcopy(shots[0].receivers)
        receivers.data = sum(float(c) * np.asarray(s.receivers.data, dtype=float) for s, c in zip(shots, codes))
        self.codes = np.asarray(codes, dtype=float)
        self.sources = enc
        enc.set_shot(self)
        self.receivers = receivers
        receivers.set_shot(self)
        self.encoding += 1

    @property
    def sequential_shots(self):
        return self._sequential_shots

    @sequential_shots.setter
    def sequential_shots(self, shots):
        shots = list(shots)
        if not shots:
            raise ValueError("a supershot needs at least one shot")
        for shot in shots:
            if type(shot.sources) is not PointSource:
                raise Exception("The shots have to have a PointSource as source.")
        ref_op = shots[0].receivers.sampling_operator
        for shot in shots:
            op = shot.receivers.sampling_operator
            if op.shape != ref_op.shape or abs(op - ref_op).nnz != 0:
                raise Exception("The receiver acquisition has to be the same for each shot in order to "
                                "construct a supershot.")
        if getattr(shots[0].receivers, "data", None) is None:
            raise Exception("No time data recorded yet.")
        self._sequential_shots = shots
        self._nshots = len(shots)
        self.is_time_simulation = True
        self.encode()


def equispaced_acquisition(mesh, wavelet, sources=1, receivers="max", source_depth=None,
                           source_kwargs={}, receiver_depth=None, receiver_kwargs={},
                           parallel_shot_wrap=None):
    """Surface acquisition with equispaced sources and receivers (acquisition.py:14-103)."""
    m, d = mesh, mesh.domain
    size, rank = (1, 0) if parallel_shot_wrap is None else (parallel_shot_wrap.size, parallel_shot_wrap.rank)
    xmin, xmax = d.x.lbound, d.x.rbound
    zmin = d.z.lbound
    source_depth = zmin if source_depth is None else source_depth
    receiver_depth = zmin if receiver_depth is None else receiver_depth
    shots = []
    if m.dim == 2:
        receivers = m.x.n if receivers == "max" else receivers
        sources = m.x.n if sources == "max" else sources
        if receivers > m.x.n:
            raise ValueError("Number of receivers exceeds mesh nodes.")
        if sources > m.x.n:
            raise ValueError("Number of sources exceeds mesh nodes.")
        xpos = np.linspace(xmin, xmax, receivers)
        base = ReceiverSet(m, [PointReceiver(m, (x, receiver_depth), **receiver_kwargs) for x in xpos])
        local = (sources // size, 1)
    elif m.dim == 3:
        ymin, ymax = d.y.lbound, d.y.rbound
        receivers = (m.x.n, m.y.n) if receivers == "max" else receivers
        sources = (m.x.n, m.y.n) if sources == "max" else sources
        if receivers[0] > m.x.n or receivers[1] > m.y.n:
            raise ValueError("Number of receivers exceeds mesh nodes.")
        if sources[0] > m.x.n or sources[1] > m.y.n:
            raise ValueError("Number of sources exceeds mesh nodes.")
        xpos = np.linspace(xmin, xmax, receivers[0])
        ypos = np.linspace(ymin, ymax, receivers[1])
        base = ReceiverSet(m, [PointReceiver(m, (x, y, receiver_depth), **receiver_kwargs)
                               for x in xpos for y in ypos])
        local = (sources[0] // size, sources[1] // size)
    else:
        raise ValueError("equispaced_acquisition needs a 2D or 3D mesh")
    for i in range(int(local[0])):
        for j in range(int(local[1])):
            idx = i + local[0] * rank
            jdx = j + local[1] * rank
            if m.dim == 2:
                pos = (xmin + (xmax - xmin) * (idx + 1.0) / (sources + 1.0), source_depth)
            else:
                pos = (xmin + (xmax - xmin) * (idx + 1.0) / (sources[0] + 1.0),
                       ymin + (ymax - ymin) * (jdx + 1.0) / (sources[1] + 1.0), source_depth)
            # receivers are copied per shot, sharing the mesh object
            shots.append(Shot(PointSource(m, pos, wavelet, **source_kwargs),
                              copy.deepcopy(base, {id(m): m, id(d): d})))
    return shots
