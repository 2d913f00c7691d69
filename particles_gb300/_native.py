"""ctypes binding of ``libparticles_gb300.so`` (the C ABI in include/particles_gb300.h).

The library is built in-tree by ``particles_gb300.build`` (nvcc, sm_103a).  If
it is missing it is built on first use; if that fails, import fails loudly.
There is no CPU fallback anywhere in the package.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

from . import build as _build

PT_METHOD_RK5, PT_METHOD_DOP853 = 1, 2
PT_PREC_FP64, PT_PREC_FP64_FMA, PT_PREC_FP32, PT_PREC_BF16 = 0, 1, 2, 3
PT_OK, PT_ERR_ARG, PT_ERR_CUDA, PT_ERR_NOMEM = 0, -1, -2, -3
PT_ERR_TIMEOUT, PT_ERR_UNSUPPORTED, PT_ERR_PARTICLE, PT_ERR_BOUNDS = -4, -5, -6, -7
PT_ST_DONE, PT_ST_RUNNING, PT_ST_ESCAPED, PT_ST_NOT_RUN = 0, 1, 2, -1
PT_ST_STEP_LIMIT, PT_ST_DT_UNDERFLOW, PT_ST_NONFINITE, PT_ST_TIMEOUT = -2, -3, -4, -5

PRECISIONS = {"fp64": PT_PREC_FP64, "fp64_fma": PT_PREC_FP64_FMA,
              "fp32": PT_PREC_FP32, "bf16": PT_PREC_BF16}

# Every symbol include/particles_gb300.h declares (checked by the CPU tests).
EXPORTS = [
    "pt_integrate", "pt_method_from_name", "pt_fields_create", "pt_fields_create_device",
    "pt_fields_destroy", "pt_fields_bytes", "pt_integrate_fields", "pt_carry_bytes",
    "pt_run_device", "pt_run_check", "pt_last_error", "pt_abi_version", "pt_tableau",
    "pt_debug_pow", "pt_debug_accel", "pt_probe_peak", "pt_debug_unpack", "pt_debug_echo",
    "pt_integrate_device_noalloc", "pt_integrate_device_noalloc_check", "pt_mlp_nparam", "pt_mlp_create", "pt_mlp_destroy",
    "pt_mlp_infer", "pt_mlp_loss_grad", "pt_mlp_adam", "pt_autotune",
    "pt_ensemble_create", "pt_ensemble_destroy", "pt_ensemble_run", "pt_ensemble_capture",
    "pt_ensemble_replay", "pt_ensemble_counts", "pt_ensemble_escaped", "pt_ensemble_check",
    "pt_copy_rows", "pt_debug_ctl_pow", "pt_debug_qdiv", "pt_debug_smul", "pt_last_transfer_bytes", "pt_debug_intpipe",
    "pt_initial_state", "pt_moments", "pt_debug_face_params", "pt_debug_face_cap",
]

PT_INIT_SPEED, PT_INIT_GAMMA, PT_INIT_MAXWELLIAN = 0, 1, 2
PT_CTL_CLASSICAL, PT_CTL_LEARNED, PT_CTL_FACE, PT_CTL_NOISE = 0, 1, 2, 4


class PtOptions(C.Structure):
    _fields_ = [
        ("struct_size", C.c_int32), ("precision", C.c_int32), ("open_x", C.c_int32),
        ("controller", C.c_int32), ("max_steps", C.c_int64), ("eta", C.c_double),
        ("jj", C.c_void_p), ("t_stop", C.c_double), ("time_budget_s", C.c_double),
        ("status", C.c_void_p), ("carry", C.c_void_p), ("model", C.c_void_p),
        ("records", C.c_void_p), ("record_capacity", C.c_int64), ("order", C.c_void_p),
        ("blocks_per_sm", C.c_int32), ("interpolation", C.c_int32),
        ("threads_per_block", C.c_int32), ("open_x_margin", C.c_double),
    ]


class PtMember(C.Structure):
    _fields_ = [
        ("fields", C.c_void_p), ("params", C.c_void_p), ("np", C.c_int64), ("m", C.c_int32),
        ("open_x", C.c_int32), ("eta", C.c_double), ("max_steps", C.c_int64),
        ("time", C.c_void_p), ("state", C.c_void_p), ("cnt", C.c_void_p),
        ("status", C.c_void_p), ("carry", C.c_void_p), ("open_x_margin", C.c_double),
    ]


# Accepted-step records (pt_options.records): a 4-float header, then records
# of the nine controller features, log(dt) and log(error ratio).
REC_HEADER_FLOATS, REC_FLOATS = 4, 11


class PtError(RuntimeError):
    def __init__(self, code: int, where: str, message: str):
        super().__init__(f"{where}: code {code}: {message}")
        self.code = code


_lib = None


def checked() -> bool:
    """PT_CHECKED=1 in the environment selects the bounds-checked library."""
    return os.environ.get("PT_CHECKED", "0") not in ("", "0")


def lib_path() -> Path:
    return _build.LIB_CHECKED if checked() else _build.LIB


def load():
    """Load (building first if needed) the native library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build(checked=checked())
    L = C.CDLL(str(path))
    vp, i32, i64, d = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    L.pt_integrate.argtypes = [i32, i64, i32, vp, vp, vp, vp, vp, vp, vp, vp]
    L.pt_method_from_name.argtypes = [C.c_char_p]
    L.pt_method_from_name.restype = i32
    L.pt_fields_create.argtypes = [vp, vp, vp, vp, i32, C.POINTER(vp)]
    L.pt_fields_create_device.argtypes = [vp, vp, vp, vp, i32, vp, C.POINTER(vp)]
    L.pt_fields_destroy.argtypes = [vp]
    L.pt_fields_bytes.argtypes = [vp]
    L.pt_fields_bytes.restype = i64
    L.pt_integrate_fields.argtypes = [i32, i64, i32, vp, vp, vp, vp, vp, vp]
    L.pt_carry_bytes.argtypes = [i64]
    L.pt_carry_bytes.restype = i64
    L.pt_run_device.argtypes = [i32, i64, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    L.pt_run_check.argtypes = [vp]
    L.pt_autotune.argtypes = [i32, i64, i32, vp, vp, vp, vp, vp, i64, vp, vp, vp]
    L.pt_ensemble_create.argtypes = [i32, i32, vp, vp, C.POINTER(vp)]
    L.pt_ensemble_destroy.argtypes = [vp]
    L.pt_ensemble_run.argtypes = [vp, d, vp]
    L.pt_ensemble_capture.argtypes = [vp, i32, d, vp]
    L.pt_ensemble_replay.argtypes = [vp, vp]
    L.pt_ensemble_counts.argtypes = [vp, vp, vp]
    L.pt_ensemble_escaped.argtypes = [vp, i32, vp, i64, C.POINTER(i64)]
    L.pt_ensemble_check.argtypes = [vp]
    L.pt_copy_rows.argtypes = [vp, i64, i32, i32, i32, vp, vp]
    L.pt_last_transfer_bytes.argtypes = [vp]
    L.pt_last_error.restype = C.c_char_p
    L.pt_abi_version.restype = i32
    L.pt_tableau.argtypes = [i32, vp]
    L.pt_tableau.restype = i32
    L.pt_debug_pow.argtypes = [i64, vp, vp, vp, vp]
    L.pt_debug_ctl_pow.argtypes = [i64, vp, vp, vp, vp]
    L.pt_debug_qdiv.argtypes = [i64, vp, vp, vp, vp]
    L.pt_debug_smul.argtypes = [i64, vp, vp, vp, vp]
    L.pt_debug_intpipe.argtypes = [i64, vp, i32, vp, vp, vp]
    L.pt_debug_accel.argtypes = [vp, i64, vp, vp, vp, vp]
    L.pt_probe_peak.argtypes = [i32, i32, C.POINTER(d)]
    L.pt_debug_unpack.argtypes = [i32, i64, i32, vp, i32, i32, vp, vp, vp]
    L.pt_debug_echo.argtypes = [i32, i64, i32, vp, i32, i32, vp, vp, vp, vp]
    L.pt_integrate_device_noalloc.argtypes = [i32, i64, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    L.pt_integrate_device_noalloc_check.argtypes = [vp]
    L.pt_initial_state.argtypes = [i32, i64, i32, C.c_uint64, i64, vp, vp, vp]
    L.pt_moments.argtypes = [i64, vp, i64, vp, vp]
    L.pt_debug_face_params.argtypes = [i32, C.c_float, C.c_float]
    L.pt_debug_face_cap.argtypes = [vp, i32, i64, vp, vp, vp, vp, vp]
    L.pt_mlp_nparam.restype = i32
    L.pt_mlp_create.argtypes = [vp, vp, C.c_float, C.POINTER(vp)]
    L.pt_mlp_destroy.argtypes = [vp]
    L.pt_mlp_infer.argtypes = [vp, vp, i64, vp, vp]
    L.pt_mlp_loss_grad.argtypes = [vp, vp, vp, i64, vp, vp, vp]
    L.pt_mlp_adam.argtypes = [vp, vp, vp, vp, i64, C.c_float, C.c_float, C.c_float, C.c_float, vp]
    _lib = L
    return L


def check(rc: int, where: str) -> int:
    if rc != PT_OK:
        msg = load().pt_last_error().decode(errors="replace")
        raise PtError(rc, where, msg)
    return rc


def last_error() -> str:
    return load().pt_last_error().decode(errors="replace")
