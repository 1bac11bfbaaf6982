"""Synthetic data generation and observed-data files (mirror of pysit.modeling.data_modeling).

``generate_seismic_data(shots, solver, model)`` assigns the model, resets every
shot's time axis to ``solver.ts()`` and stores the simulated traces in
``shot.receivers.data`` (generate_seismic_data / generate_shot_data_time,
pysit/modeling/data_modeling.py:17-178, 335-429).  All shots are modelled by one
batched device call; ``wavefields=[]`` (per-step wavefields of a single shot)
takes the plain per-step device loop instead.

``save_method`` ('pickle', 'savemat', 'h5py') then writes every shot's traces and time
axis to ``./shots_time/shot_<i>.<ext>`` and ``ts_<i>.<ext>`` (i from 1), and
``generate_seismic_data_from_file`` reads them back into the shots (:59-173, :180-333):
  pickle   one pickled ndarray per file (the reference opens the files with Python 2's
           ``file()``, a NameError under Python 3; ``open()`` here);
  savemat  one MATLAB variable per file, named by the file's own path as the reference
           names it, so either side reads the other's files;
  h5py     one dataset per file, named by the file's path (needs h5py).
The directory is replaced on every save, as the reference does.  ``path`` (a keyword the
reference does not have) moves it.
"""
from __future__ import annotations

import os
import shutil
import time

import numpy as np

from ..engine import plan_for

__all__ = ["generate_seismic_data", "generate_shot_data_time", "generate_seismic_data_from_file",
           "save_shot_data", "load_shot_data"]

_EXT = {"pickle": "save", "savemat": "mat", "h5py": "hdf5"}
_DEFAULT_PATH = "./shots_time"


def _files(path, i, method):
    ext = _EXT[method]
    return path + "/shot_" + str(i + 1) + "." + ext, path + "/ts_" + str(i + 1) + "." + ext


def _h5py():
    try:
        import h5py
    except ImportError:
        raise ImportError("h5py is not installed please install it and try again")
    return h5py


def save_shot_data(shots, save_method, path=_DEFAULT_PATH):
    """Write every shot's receivers.data and receivers.ts (data_modeling.py:59-121)."""
    if save_method not in _EXT:
        raise TypeError("Unknown save_method")
    h5 = _h5py() if save_method == "h5py" else None
    if os.path.exists(path):
        shutil.rmtree(path)
    os.makedirs(path)
    for i, shot in enumerate(shots):
        fshot, fts = _files(path, i, save_method)
        data = np.asarray(shot.receivers.data)
        ts = np.asarray(shot.receivers.ts)
        for fname, arr in ((fshot, data), (fts, ts)):
            if save_method == "pickle":
                import pickle
                with open(fname, "wb") as f:
                    pickle.dump(arr, f, protocol=pickle.HIGHEST_PROTOCOL)
            elif save_method == "savemat":
                import scipy.io as sio
                sio.savemat(fname, mdict={fname: arr})
            else:
                with h5.File(fname, "w") as f:
                    dts = f.create_dataset(fname, arr.shape, arr.dtype)
                    dts[...] = arr


def load_shot_data(shots, save_method, path=_DEFAULT_PATH):
    """Read the files of save_shot_data back into the shots (data_modeling.py:180-262)."""
    if save_method not in _EXT:
        raise TypeError("Unknown save_method")
    h5 = _h5py() if save_method == "h5py" else None
    if not os.path.exists(path):
        raise ImportError("There is no shot directory, please relaunch generate_seismic_data with save_method "
                          "argument")
    try:
        for i, shot in enumerate(shots):
            fshot, fts = _files(path, i, save_method)
            if save_method == "pickle":
                import pickle
                with open(fts, "rb") as f:
                    ts = pickle.load(f)
                with open(fshot, "rb") as f:
                    data = pickle.load(f)
            elif save_method == "savemat":
                import scipy.io as sio
                ts = sio.loadmat(fts)[fts].flatten()
                data = sio.loadmat(fshot)[fshot]
            else:
                with h5.File(fts, "r") as f:
                    ts = f[fts][...]
                with h5.File(fshot, "r") as f:
                    data = f[fshot][...]
            shot.receivers.clear_data(len(ts))
            shot.receivers.ts = np.asarray(ts, dtype=float)
            shot.receivers.data = np.asarray(data)
    except (IOError, KeyError):
        raise IOError("Files are corrupted or generated with different save_method argument")


def generate_seismic_data_from_file(shots, solver, verbose=False, save_method=None, path=_DEFAULT_PATH, **kwargs):
    """Load observed data written by generate_seismic_data(save_method=...) into the shots."""
    if solver.supports["equation_dynamics"] != "time":
        raise TypeError("A time solver must be specified.")
    t0 = time.time()
    if save_method is not None:
        load_shot_data(shots, save_method, path)
    if verbose:
        dt = time.time() - t0
        print(f"Data loading: {dt}s")


def generate_seismic_data(shots, solver, model, verbose=False, frequencies=None, save_method=None,
                          wavefields=None, path=_DEFAULT_PATH, **kwargs):
    if solver.supports["equation_dynamics"] != "time":
        raise TypeError("A time solver must be specified.")
    if save_method is not None and save_method not in _EXT:
        raise TypeError("Unknown save_method")
    t0 = time.time()
    if wavefields is not None:
        for shot in shots:
            generate_shot_data_time(shot, solver, model, wavefields=wavefields, **kwargs)
    else:
        solver.model_parameters = model
        ts = solver.ts()
        plan = plan_for(solver, shots, forward_only=True)
        traces = plan.forward().double().cpu().numpy()
        plan.check_status()
        for i, shot in enumerate(shots):
            shot.reset_time_series(ts)
            shot.dt = solver.dt
            shot.trange = solver.trange
            shot.receivers.data[:] = traces[i, :, :shot.receivers.receiver_count]
    if verbose:
        dt = time.time() - t0
        print(f"Data generation: {dt}s")
        print(f"Data generation: {dt / max(1, len(shots))}s/shot")
    if save_method is not None:
        save_shot_data(shots, save_method, path)


def generate_shot_data_time(shot, solver, model, wavefields=None, wavefields_padded=None, verbose=False,
                            **kwargs):
    """One shot, per-step device loop; optionally keeps every wavefield (unpadded)."""
    from .temporal_modeling import TemporalModeling
    solver.model_parameters = model
    ts = solver.ts()
    shot.reset_time_series(ts)
    shot.dt = solver.dt
    shot.trange = solver.trange
    rp = {"simdata"}
    if wavefields is not None:
        rp.add("wavefield")
    rv = TemporalModeling(solver)._forward_plain(shot, 1, rp)
    shot.receivers.data[:] = rv["simdata"]
    if wavefields is not None:
        wavefields[:] = rv["wavefield"]
