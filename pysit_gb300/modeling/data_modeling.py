"""Synthetic data generation (mirror of pysit.modeling.data_modeling).

``generate_seismic_data(shots, solver, model)`` assigns the model, resets every
shot's time axis to ``solver.ts()`` and stores the simulated traces in
``shot.receivers.data`` (generate_seismic_data / generate_shot_data_time,
pysit/modeling/data_modeling.py:17-178, 335-429).  All shots are modelled by one
batched device call; ``wavefields=[]`` (per-step wavefields of a single shot)
takes the plain per-step device loop instead.
"""
from __future__ import annotations

import time

import numpy as np

from ..engine import plan_for

__all__ = ["generate_seismic_data", "generate_shot_data_time"]


def generate_seismic_data(shots, solver, model, verbose=False, frequencies=None, save_method=None,
                          wavefields=None, **kwargs):
    if solver.supports["equation_dynamics"] != "time":
        raise TypeError("A time solver must be specified.")
    if save_method is not None:
        raise NotImplementedError("saving generated data to disk is not supported by pysit_gb300")
    t0 = time.time()
    if wavefields is not None:
        for shot in shots:
            generate_shot_data_time(shot, solver, model, wavefields=wavefields, **kwargs)
    else:
        solver.model_parameters = model
        ts = solver.ts()
        plan = plan_for(solver, shots)
        traces = plan.forward().double().cpu().numpy()
        for i, shot in enumerate(shots):
            shot.reset_time_series(ts)
            shot.dt = solver.dt
            shot.trange = solver.trange
            shot.receivers.data[:] = traces[i, :, :shot.receivers.receiver_count]
    if verbose:
        dt = time.time() - t0
        print(f"Data generation: {dt}s")
        print(f"Data generation: {dt / max(1, len(shots))}s/shot")


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
