"""Observed-data files: generate_seismic_data(save_method=...) and
generate_seismic_data_from_file (pysit/modeling/data_modeling.py:59-173, 180-333).

Round trips of pysit_gb300's writer and reader ('pickle', 'savemat'; 'h5py' where h5py is
installed), and the file format against the reference itself: a 'savemat' directory
written by the reference's generate_seismic_data is read by pysit_gb300, and one written
here is read by the reference's generate_seismic_data_from_file (tests run where the
reference tree is present).  Data are set on the host, so no GPU is needed.
"""
import numpy as np
import pytest

import problems
import pysit_gb300 as api
from pysit_gb300.modeling.data_modeling import load_shot_data, save_shot_data

METHODS = ["pickle", "savemat", pytest.param("h5py", marks=pytest.mark.skipif(
    not __import__("importlib").util.find_spec("h5py"), reason="h5py not installed"))]


def _shots(seed=1):
    m, shots, solver, C, C0 = problems.build(api, "o2")
    solver.model_parameters = solver.ModelParameters(m, {"C": C})
    ts = solver.ts()
    rng = np.random.default_rng(seed)
    for s in shots:
        s.reset_time_series(ts)
        s.receivers.data[:] = rng.standard_normal(s.receivers.data.shape)
    return m, shots, solver


@pytest.mark.parametrize("method", METHODS)
def test_round_trip(method, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    m, shots, solver = _shots()
    save_shot_data(shots, method)
    assert (tmp_path / "shots_time" / f"shot_2.{ {'pickle': 'save', 'savemat': 'mat', 'h5py': 'hdf5'}[method]}").exists()
    _, fresh, _ = _shots(seed=2)
    api.generate_seismic_data_from_file(fresh, solver, save_method=method)
    for a, b in zip(shots, fresh):
        np.testing.assert_array_equal(b.receivers.data, a.receivers.data)
        np.testing.assert_array_equal(b.receivers.ts, a.receivers.ts)
        np.testing.assert_allclose(b.receivers.interpolate_data(solver.ts()), a.receivers.data, rtol=1e-12,
                                   atol=1e-15)


def test_errors(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    m, shots, solver = _shots()
    with pytest.raises(TypeError):
        save_shot_data(shots, "segy")
    with pytest.raises(ImportError, match="no shot directory"):
        load_shot_data(shots, "savemat")
    save_shot_data(shots, "pickle")
    with pytest.raises(IOError):
        load_shot_data(shots, "savemat")  # files of another method


@pytest.fixture(scope="module")
def ref():
    import pysit_live
    if not pysit_live.available():
        pytest.skip("reference tree absent")
    return pysit_live.import_pysit()


def test_savemat_files_are_exchangeable_with_the_reference(ref, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    # reference writes (its cpp solver models the data), pysit_gb300 reads
    rm, rshots, rsolver, C, C0 = problems.build(ref, "o2", kernel="cpp")
    ref.generate_seismic_data(rshots, rsolver, rsolver.ModelParameters(rm, {"C": C}), save_method="savemat")
    m, shots, solver = _shots()
    api.generate_seismic_data_from_file(shots, solver, save_method="savemat")
    for a, b in zip(rshots, shots):
        np.testing.assert_array_equal(b.receivers.data, a.receivers.data)
        np.testing.assert_array_equal(b.receivers.ts, a.receivers.ts)
    # pysit_gb300 writes, the reference reads
    m, mine, solver = _shots(seed=5)
    save_shot_data(mine, "savemat")
    ref.generate_seismic_data_from_file(rshots, rsolver, save_method="savemat")
    for a, b in zip(mine, rshots):
        np.testing.assert_array_equal(b.receivers.data, a.receivers.data)
        np.testing.assert_array_equal(np.ravel(b.receivers.ts), a.receivers.ts)
