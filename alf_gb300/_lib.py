"""ctypes binding of the C ABI declared in ``include/alfgpu.h``.

The library is the only compute path: if ``libalfgpu.so`` is missing or a
call fails, an exception is raised (there is no CPU fallback).
"""
from __future__ import annotations

import ctypes as C
import os
import re

from . import build as _build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "alfgpu.h")


class Dims(C.Structure):
    _fields_ = [("ndim", C.c_int32), ("n_fl", C.c_int32), ("n_sun", C.c_int32), ("n_op", C.c_int32),
                ("ltrot", C.c_int32), ("nwrap", C.c_int32), ("n_chains", C.c_int32), ("precision", C.c_int32),
                ("delay_k", C.c_int32), ("ltau", C.c_int32), ("device", C.c_int32), ("reserved", C.c_int32 * 5)]


class Vertices(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("op_n", "op_nz", "op_diag", "op_type", "op_P", "op_g", "op_alpha",
                                           "op_E", "op_U", "op_Eexp", "op_Mexp")]


class Stats(C.Structure):
    _fields_ = [("n_prop", C.c_int64), ("n_acc", C.c_int64), ("n_prop_eff", C.c_int64), ("n_acc_eff", C.c_int64),
                ("ncg", C.c_int64), ("xmeanG_sum", C.c_double), ("xmaxG", C.c_double), ("xmaxP", C.c_double),
                ("ncg_tau", C.c_int64), ("xmean_tau_sum", C.c_double), ("xmax_tau", C.c_double),
                ("sweeps", C.c_int64)]


PROF_PHASES = ["hop", "update", "flush", "propagate", "qr", "orgqr", "solve"]

OBS_CB = C.CFUNCTYPE(None, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_double),
                     C.POINTER(C.c_double))

ERRORS = {0: "ERROR_NONE", 1: "ERROR_GENERIC", 3: "ERROR_UNSTABLE_MATRIX", 5: "ERROR_FIELDS",
          6: "ERROR_HAMILTONIAN", 100: "ERROR_CUDA", 101: "ERROR_ARGUMENT", 102: "ERROR_UNSUPPORTED",
          103: "ERROR_NAN", 104: "ERROR_TIMEOUT", 105: "ERROR_SIZE"}


class AlfGpuError(RuntimeError):
    def __init__(self, code: int, where: str):
        super().__init__(f"{where} failed: {ERRORS.get(code, code)} ({code})")
        self.code = code


def header_functions() -> list:
    """Names of every function declared in include/alfgpu.h."""
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(alfgpu_[a-z0-9_]+)\s*\(", txt)))


_lib = None


def lib(build_if_missing: bool = True):
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"CUDA library {path} is not built")
        _build.build()
    L = C.CDLL(path)
    vp = C.c_void_p
    sig = {
        "alfgpu_create": ([C.POINTER(vp), C.POINTER(Dims)], C.c_int),
        "alfgpu_destroy": ([vp], None),
        "alfgpu_error_string": ([C.c_int], C.c_char_p),
        "alfgpu_upload_hopping": ([vp, vp, vp], C.c_int),
        "alfgpu_upload_vertices": ([vp, C.c_int32, C.POINTER(Vertices)], C.c_int),
        "alfgpu_upload_checkerboard": ([vp, C.c_int32, C.c_int32, vp, vp, vp, vp], C.c_int),
        "alfgpu_set_fields": ([vp, C.c_int32, vp], C.c_int),
        "alfgpu_set_fields_c128": ([vp, C.c_int32, vp], C.c_int),
        "alfgpu_get_fields": ([vp, C.c_int32, vp], C.c_int),
        "alfgpu_set_rng": ([vp, C.c_int32, C.c_uint64, C.c_uint64], C.c_int),
        "alfgpu_init_state": ([vp, vp], C.c_int),
        "alfgpu_sweep": ([vp, vp, OBS_CB, vp], C.c_int),
        "alfgpu_sweep_many": ([vp, C.c_int32, vp, vp], C.c_int),
        "alfgpu_set_delay": ([vp, C.c_int32], C.c_int),
        "alfgpu_get_delay": ([vp, C.POINTER(C.c_int32)], C.c_int),
        "alfgpu_tune_delay": ([vp, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
        "alfgpu_get_green": ([vp, C.c_int32, vp], C.c_int),
        "alfgpu_get_phase": ([vp, vp], C.c_int),
        "alfgpu_get_stats": ([vp, C.c_int32, C.POINTER(Stats)], C.c_int),
        "alfgpu_reset_stats": ([vp], C.c_int),
        "alfgpu_set_recording": ([vp, C.c_int32], C.c_int),
        "alfgpu_get_record": ([vp, C.c_int32, vp, vp, vp, vp, vp], C.c_int),
        "alfgpu_stream": ([vp], vp),
        "alfgpu_set_profiling": ([vp, C.c_int32], C.c_int),
        "alfgpu_get_profile": ([vp, vp, vp], C.c_int),
        "alfgpu_launch_count": ([vp], C.c_int64),
        "alfgpu_cgr": ([C.c_int32, C.c_int32, vp, vp, vp, vp, vp, vp, vp, vp], C.c_int),
        "alfgpu_decompose": ([C.c_int32, C.c_char, vp, vp, vp], C.c_int),
        "alfgpu_decompose_noalloc": ([C.c_int32, C.c_char, vp, vp, vp, vp, vp], C.c_int),
        "alfgpu_last_error": ([vp], C.c_char_p),
        "alfgpu_set_nwrap": ([vp, C.c_int32], C.c_int),
        "alfgpu_set_scalar_obs": ([vp, vp, vp], C.c_int),
        "alfgpu_get_scalar_obs": ([vp, C.c_int32, vp], C.c_int),
        "alfgpu_reset_scalar_obs": ([vp], C.c_int),
        "alfgpu_get_rng_state": ([vp, C.c_int32, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)], C.c_int),
        "alfgpu_set_rng_state": ([vp, C.c_int32, C.c_uint64, C.c_uint64], C.c_int),
        "alfgpu_get_nwrap": ([vp, C.POINTER(C.c_int32)], C.c_int),
        "alfgpu_oz_dgemm": ([C.c_int32, C.c_int32, C.c_int32, vp, C.c_int32, vp, C.c_int32, vp, C.c_int32,
                             C.c_int32], C.c_int),
        "alfgpu_set_lattice_obs": ([vp, C.c_int32, C.c_int32, vp, vp], C.c_int),
        "alfgpu_get_lattice_obs": ([vp, C.c_int32, C.c_int32, vp, vp, vp], C.c_int),
        "alfgpu_reset_lattice_obs": ([vp], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def check(code: int, where: str):
    if code != 0:
        raise AlfGpuError(code, where)
