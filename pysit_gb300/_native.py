"""ctypes binding of libpysit_gb300.so (declared in include/pysit_gb300.h).

The library must exist: every product entry point raises if it is missing or
if no CUDA device is visible.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libpysit_gb300.so")

PYSIT_OK = 0
PYSIT_EINVAL = -1
PYSIT_ECUDA = -2
PYSIT_ENONFINITE = -3
PYSIT_ESTATE = -4
PYSIT_EHOST = -5
PYSIT_ETIMEOUT = -6
PYSIT_F32 = 0
PYSIT_F64 = 1

_vp = C.c_void_p
_i = C.c_int
_d = C.c_double


class PysitCudaError(RuntimeError):
    """Error returned by the CUDA library (carries the C status code)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[pysit_gb300 status {code}] {msg}")
        self.code = code


class PlanDesc(C.Structure):
    """Mirror of pysit_plan_desc."""
    _fields_ = [
        ("dim", _i), ("order", _i), ("dtype", _i),
        ("n", _i * 3), ("delta", _d * 3), ("pad_lo", _i * 3), ("pad_hi", _i * 3),
        ("dt", _d), ("nsteps", _i), ("imaging_period", _i), ("checkpoint_every", _i),
        ("shots_per_launch", _i), ("nshots", _i),
        ("sig_l", C.POINTER(_d) * 3), ("nsig_l", _i * 3),
        ("sig_r", C.POINTER(_d) * 3), ("nsig_r", _i * 3),
        ("sigmap", C.POINTER(_d) * 3),
        ("nsrc", _i),
        ("src_tap_ptr", C.POINTER(C.c_int64)), ("src_tap_cell", C.POINTER(C.c_int64)),
        ("src_tap_point", C.POINTER(C.c_int32)), ("src_tap_w", C.POINTER(_d)),
        ("src_amp", C.POINTER(_d)),
        ("nrec", _i),
        ("rec_tap_ptr", C.POINTER(C.c_int64)), ("rec_tap_cell", C.POINTER(C.c_int64)),
        ("rec_tap_point", C.POINTER(C.c_int32)), ("rec_tap_wsample", C.POINTER(_d)),
        ("rec_tap_winject", C.POINTER(_d)),
        ("use_graph", _i),
        ("psi_consistent", _i),
        ("tile_x", _i),
        ("shot_nsteps", C.POINTER(C.c_int32)),
        ("store_dwaveop", _i),
        ("forward_only", _i),
        ("shell_share", _d * 3),
        ("lanes", _i),
        ("wait_polls", C.c_uint32),
        ("wait_fault", _i),
        ("tile_z", _i),
    ]


_PROTOS = {
    "pysit_cuda_last_error": (C.c_char_p, []),
    "pysit_cuda_version": (_i, []),
    "pysit_cda_step_1d": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp, _i, _d, _d, _i,
                               _vp, _vp, _vp]),
    "pysit_cda_step_2d": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp, _i, _vp, _i,
                               _vp, _i, _d, _d, _d, _i, _i, _vp, _vp, _vp, _vp]),
    "pysit_cda_step_3d": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                               _vp, _i, _vp, _i, _vp, _i, _vp, _i, _vp, _i, _vp, _i,
                               _d, _d, _d, _d, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp]),
    "pysit_cda_dwaveop": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _d, _vp,
                               _vp]),
    "pysit_plan_create": (_i, [C.POINTER(PlanDesc), C.POINTER(_vp)]),
    "pysit_plan_destroy": (_i, [_vp]),
    "pysit_plan_workspace_bytes": (_i, [_vp, C.POINTER(C.c_uint64)]),
    "pysit_plan_bind_workspace": (_i, [_vp, _vp, C.c_uint64, _vp]),
    "pysit_plan_set_model": (_i, [_vp, _vp, _vp]),
    "pysit_plan_forward": (_i, [_vp, _vp, _vp]),
    "pysit_plan_gradient": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "pysit_plan_misfit": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "pysit_plan_migrate": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "pysit_plan_get_tuning": (_i, [_vp, C.POINTER(_i), C.POINTER(_d)]),
    "pysit_plan_born": (_i, [_vp, _vp, _vp, _vp]),
    "pysit_plan_hessian": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "pysit_plan_status": (_i, [_vp, C.POINTER(_i), _vp]),
    "pysit_misfit_per_shot_noalloc": (_i, [_i, _vp, _vp, _i, C.c_int64, _vp, _vp, _vp]),
    "pysit_plan_last_launch_count": (_i, [_vp, C.POINTER(C.c_int64)]),
    "pysit_plan_step_loop": (_i, [_vp, _i, _i, _vp]),
    "pysit_plan_autotune": (_i, [_vp, C.POINTER(_i), _i, _i, C.POINTER(_i), C.POINTER(C.c_double), _vp]),
    "pysit_plan_autotune_tiles": (_i, [_vp, C.POINTER(_i), _i, C.POINTER(_i), _i, _i, C.POINTER(_i), C.POINTER(_i),
                                       C.POINTER(C.c_double), _vp]),
    "pysit_plan_get_tiles": (_i, [_vp, C.POINTER(_i), C.POINTER(_i)]),
    "pysit_plan_task_table": (_i, [_vp, C.POINTER(C.c_int32), C.c_uint64, C.POINTER(C.c_uint64),
                                   C.POINTER(C.c_int32)]),
    "pysit_group_create": (_i, [C.POINTER(_vp), _i, C.POINTER(_vp)]),
    "pysit_group_destroy": (_i, [_vp]),
    "pysit_group_gradient": (_i, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), _vp]),
}

_lib = None
_lock = threading.Lock()


def exported_symbols() -> list[str]:
    """Names of every entry point this binding expects the library to export."""
    return list(_PROTOS)


def load(path: str | None = None):
    """Load (once) and return the CUDA library; raises if it is missing."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or os.environ.get("PYSIT_GB300_LIB", LIB_PATH)
        if not os.path.exists(p):
            raise PysitCudaError(PYSIT_ESTATE,
                                 f"CUDA library {p} is missing: run `python -m pysit_gb300.build` "
                                 "(pysit_gb300 has no CPU fallback)")
        lib = C.CDLL(p)
        for name, (res, args) in _PROTOS.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
        return lib


def check(rc: int) -> None:
    """Raise PysitCudaError for a non-zero status of a library call."""
    if rc != PYSIT_OK:
        msg = load().pysit_cuda_last_error().decode(errors="replace")
        raise PysitCudaError(rc, msg)


def require_cuda():
    """Return torch after checking a CUDA device is usable (no CPU fallback)."""
    import torch
    if not torch.cuda.is_available():
        raise PysitCudaError(PYSIT_ESTATE, "no CUDA device is visible: pysit_gb300 runs on the GPU only")
    load()
    return torch


def stream_handle(stream=None) -> int:
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)
