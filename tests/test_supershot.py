"""Source-encoded supershots (pysit/core/shot.py:148-345) on the host: codes, encoded
sources and data, validation; and the oracle's linearity over the encoding.  The
reference's class cannot be constructed (its encoded source set calls
super().__init__(self, ...), a TypeError), so the definition is the check: a supershot
is the member shots fired together with intensities code_i, its data sum_i code_i d_i."""
import numpy as np
import pytest

import pipeline
import problems
import pysit_gb300 as api


def _shots_with_data(name="o2"):
    m, shots, solver, C, C0 = problems.build(api, name)
    solver.model_parameters = solver.ModelParameters(m, {"C": C})
    ts = solver.ts()
    rng = np.random.default_rng(8)
    for s in shots:
        s.reset_time_series(ts)
        s.receivers.data[:] = rng.standard_normal(s.receivers.data.shape)
    return m, shots, solver, C, C0


def test_codes_and_encoded_data():
    m, shots, solver, C, C0 = _shots_with_data()
    ss = api.SourceEncodedSupershot(shots, rng=np.random.default_rng(3))
    codes = ss.codes
    assert codes.shape == (len(shots),)
    np.testing.assert_allclose(ss.receivers.data, sum(c * s.receivers.data for c, s in zip(codes, shots)))
    assert ss.sources.source_count == len(shots)
    ts = solver.ts()
    amp = ss.sources.amplitudes(ts)
    for i, (c, s) in enumerate(zip(codes, shots)):
        np.testing.assert_allclose(amp[:, i], c * s.sources.amplitudes(ts)[:, 0])
    # the member shots are untouched
    assert all(s.sources.intensity == 1.0 for s in shots)
    cells, pts, w = ss.sources.taps()
    assert set(pts.tolist()) == set(range(len(shots)))
    old = ss.encoding
    ss.encode()
    assert ss.encoding == old + 1 and not np.array_equal(ss.codes, codes)
    ss.encode(codes=[1.0, -1.0])
    np.testing.assert_allclose(ss.receivers.data, shots[0].receivers.data - shots[1].receivers.data)


def test_krebs_codes_are_signs_and_global_generator_matches_the_reference_draw():
    m, shots, solver, C, C0 = _shots_with_data()
    ss = api.SourceEncodedSupershot(shots, weight_type="krebs", rng=np.random.default_rng(1))
    for _ in range(5):
        ss.encode()
        assert set(np.unique(ss.codes)) <= {-1.0, 1.0}
    np.random.seed(123)
    ss = api.SourceEncodedSupershot(shots)  # numpy's global generator, as the reference draws
    np.random.seed(123)
    np.testing.assert_array_equal(ss.codes, np.random.randn(len(shots)))
    with pytest.raises(Exception):
        api.SourceEncodedSupershot(shots, weight_type="uniform")


def test_supershot_validation():
    m, shots, solver, C, C0 = _shots_with_data()
    other = problems.build(api, "o2", spec_overrides=dict(nrec=12))[1]
    for s in other:
        s.reset_time_series(solver.ts())
    with pytest.raises(Exception, match="receiver acquisition"):
        api.SourceEncodedSupershot([shots[0], other[1]])
    fresh = problems.build(api, "o2")[1]
    with pytest.raises(Exception, match="No time data"):
        api.SourceEncodedSupershot(fresh)
    ss = api.SourceEncodedSupershot(shots, rng=np.random.default_rng(0))
    with pytest.raises(Exception, match="PointSource"):
        api.SourceEncodedSupershot([ss])


def test_oracle_supershot_traces_are_the_encoded_sum():
    m, shots, solver, C, C0 = _shots_with_data()
    ss = api.SourceEncodedSupershot(shots, rng=np.random.default_rng(9))
    sim = pipeline.forward(problems.oracle_problem(solver, ss))[0]
    parts = [pipeline.forward(problems.oracle_problem(solver, s))[0] for s in shots]
    ref = sum(c * p for c, p in zip(ss.codes, parts))
    assert np.linalg.norm(sim - ref) <= 1e-12 * np.linalg.norm(ref)
