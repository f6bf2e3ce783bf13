"""ctypes binding of ``libgbnufft.so`` (declared in ``include/gbnufft.h``).

The library is loaded lazily on first use.  There is no fallback: if the
library has not been built, or cannot be loaded, every operator call raises.
"""

from __future__ import annotations

import ctypes
import threading
from pathlib import Path

from . import _build

_c_int = ctypes.c_int
_c_i64 = ctypes.c_int64
_c_dbl = ctypes.c_double
_c_flt = ctypes.c_float
_vp = ctypes.c_void_p

GBN_OK = 0
GBN_ERR_ARG = 1
GBN_ERR_CUDA = 2
GBN_ERR_CUFFT = 3
GBN_ERR_NOMEM = 4
GBN_ERR_STATE = 5

STAGES = {"pad": 0, "fft": 1, "interp": 2, "spread": 3, "crop": 4, "zero": 5, "grad": 6,
          "kmul": 7}

# name -> (restype, argtypes); must match include/gbnufft.h
SIGNATURES = {
    "gbn_version": (_c_int, []),
    "gbn_last_error": (ctypes.c_char_p, []),
    "gbn_plan_create": (
        _c_int,
        [_c_int, ctypes.POINTER(_c_i64), _c_dbl, _c_dbl, _c_int, _c_int, _c_int, ctypes.POINTER(_vp)],
    ),
    "gbn_plan_destroy": (_c_int, [_vp]),
    "gbn_plan_info": (
        _c_int,
        [_vp, ctypes.POINTER(_c_int), ctypes.POINTER(_c_dbl), ctypes.POINTER(_c_i64), ctypes.POINTER(_c_int)],
    ),
    "gbn_plan_device_bytes": (_c_int, [_vp, ctypes.POINTER(_c_i64)]),
    "gbn_plan_tune": (_c_int, [_vp, ctypes.POINTER(_c_int), _c_int, _c_int]),
    "gbn_setpts": (_c_int, [_vp, _c_i64, _vp, _vp, _vp, _vp]),
    "gbn_op": (_c_int, [_vp, _vp, _vp, _vp, _c_int, _c_int, _c_flt, _c_int, _vp]),
    "gbn_adj": (_c_int, [_vp, _vp, _vp, _vp, _vp, _c_int, _c_int, _c_flt, _c_int, _vp]),
    "gbn_dc": (_c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _c_int, _c_int, _c_flt, _vp]),
    "gbn_pipe": (_c_int, [_vp, _vp, _c_int, _c_flt, _vp]),
    "gbn_grad_traj_op": (_c_int, [_vp, _vp, _vp, _vp, _vp, _c_int, _c_int, _c_flt, _vp]),
    "gbn_grad_traj_adj": (_c_int, [_vp, _vp, _vp, _vp, _vp, _c_int, _c_int, _c_flt, _vp]),
    "gbn_batch_create": (_c_int, [_c_int, ctypes.POINTER(_vp), ctypes.POINTER(_vp)]),
    "gbn_batch_bind": (
        _c_int,
        [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp),
         ctypes.POINTER(_c_flt), ctypes.POINTER(_c_int)],
    ),
    "gbn_batch_op": (_c_int, [_vp, _vp]),
    "gbn_batch_adj": (_c_int, [_vp, _vp]),
    "gbn_batch_destroy": (_c_int, [_vp]),
    "gbn_toep_create": (_c_int, [_vp, _c_i64, _vp, _vp, _vp, _vp, ctypes.POINTER(_vp), _vp]),
    "gbn_toep_info": (_c_int, [_vp, ctypes.POINTER(_c_i64)]),
    "gbn_toep_kernel": (_c_int, [_vp, _vp, _vp]),
    "gbn_toep_apply": (_c_int, [_vp, _vp, _vp, _vp, _c_int, _c_int, _c_flt, _vp]),
    "gbn_toep_destroy": (_c_int, [_vp]),
    "gbn_toep_plan": (_c_int, [_vp, ctypes.POINTER(_vp)]),
    "gbn_toep_cg_iter": (
        _c_int,
        [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _c_int, _c_int, _c_flt, _c_flt, _vp],
    ),
    "gbn_toep_power_iter": (_c_int, [_vp, _vp, _vp, _vp, _vp, _c_flt, _vp]),
    "gbn_stack_create": (_c_int, [ctypes.POINTER(_c_i64), ctypes.POINTER(_c_int), _c_int, _c_int,
                                  ctypes.POINTER(_vp)]),
    "gbn_stack_fwd": (_c_int, [_vp, _vp, _vp, _vp, _c_int, _vp]),
    "gbn_stack_adj": (_c_int, [_vp, _vp, _vp, _vp, _c_int, _c_int, _vp]),
    "gbn_stack_destroy": (_c_int, [_vp]),
    "gbn_orc_reduce": (_c_int, [_vp, _vp, _vp, _c_int, _c_int, _c_int, _c_i64, _c_i64, _vp]),
    "gbn_orc_expand": (_c_int, [_vp, _vp, _vp, _c_int, _c_int, _c_int, _c_i64, _c_i64, _vp]),
    "gbn_profile": (_c_int, [_vp, _c_int]),
    "gbn_profile_read": (_c_int, [_vp, _c_int, ctypes.POINTER(_c_dbl), ctypes.POINTER(_c_i64)]),
    "gbn_norm2_f64": (_c_int, [_vp, _c_i64, _vp, _vp]),
    "gbn_dotu_f64": (_c_int, [_vp, _vp, _c_i64, _c_int, _vp, _vp]),
    "gbn_cg_update": (_c_int, [_c_i64, _vp, _vp, _vp, _vp, _vp, _vp, _c_flt, _vp]),
    "gbn_power_step": (_c_int, [_c_i64, _vp, _vp, _vp, _vp, _vp]),
    "gbn_scale_ratio": (_c_int, [_c_i64, _vp, _vp, _vp, _vp]),
    "gbn_pipe_static": (
        _c_int,
        [_c_int, ctypes.POINTER(_c_i64), _c_dbl, _c_dbl, _c_i64, _vp, _vp, _vp, _vp, _c_int, _c_flt, _vp],
    ),
}

_lock = threading.Lock()
_lib = None


class GB300Error(RuntimeError):
    """A CUDA-side failure reported by the GB300 NUFFT library."""


def library_path() -> Path:
    return _build.LIB


def _preload_cuda():
    # torch brings libcudart / libcufft into the process; importing it first
    # lets the dynamic loader resolve the library's CUDA dependencies.
    try:
        import torch  # noqa: F401
    except ImportError:
        pass


def load(path: str | Path | None = None):
    """Load the library (once) and declare every entry point's signature."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path is not None else _build.LIB
        if not p.exists():
            raise RuntimeError(
                f"GB300 NUFFT library not built ({p} missing): run "
                "`python -c 'import __graft_entry__ as g; g.build()'`"
            )
        _preload_cuda()
        lib = ctypes.CDLL(str(p))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


def last_error() -> str:
    msg = load().gbn_last_error()
    return msg.decode() if msg else ""


def check(status: int, what: str):
    """Raise the exception matching a non-zero status code."""
    if status == GBN_OK:
        return
    msg = f"{what}: {last_error()}"
    if status == GBN_ERR_ARG:
        raise ValueError(msg)
    if status == GBN_ERR_NOMEM:
        raise MemoryError(msg)
    raise GB300Error(f"{msg} (status {status})")


def call(name: str, *args):
    """Call an entry point and raise on a non-zero status."""
    check(getattr(load(), name)(*args), name)
