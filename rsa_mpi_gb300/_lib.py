"""ctypes binding of the sampler's C ABI (include/rsagpu.h).

This is the binding a user of the reference's Python module gets instead of the
pybind11 extension (Interface_python/Interface.cxx): the library is loaded from
the package's _build/ folder and every call goes to the GPU.  There is no CPU
fallback: if the library is missing or has no GPU to run on, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "librsagpu.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "rsagpu.h")

_d = C.POINTER(C.c_double)
_u64 = C.POINTER(C.c_uint64)
_i64 = C.POINTER(C.c_int64)
_i32 = C.POINTER(C.c_int)
_u8 = C.POINTER(C.c_uint8)
_u16 = C.POINTER(C.c_uint16)
_f32 = C.POINTER(C.c_float)
_vp = C.c_void_p

RSAGPU_FORM_FP64 = 0
RSAGPU_FORM_FP32_GUARD = 1
RSAGPU_SCHEDULE_HEURISTIC = 0
RSAGPU_SCHEDULE_LEARNED = 1
RSAGPU_SCHEDULE_REFERENCE = 2
RSAGPU_CAP_REFERENCE = 0
RSAGPU_CAP_EXACT = 1
RSAGPU_ERR_ARG = -1
RSAGPU_ERR_CAPACITY = -7
MAX_DIM = 7


class RsaGpuError(RuntimeError):
    """Raised for a negative status of the C ABI (the reference raises std::runtime_error)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[rsagpu {code}] {msg}")
        self.code = code


class Stats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("rounds", "refinements", "darts", "accepted", "settle_iterations",
                                           "retests", "peak_voxels", "bytes_darts", "bytes_probe", "bytes_settle",
                                           "bytes_commit", "bytes_refine")] + \
              [(n, C.c_double) for n in ("ms_darts", "ms_probe", "ms_settle", "ms_commit", "ms_refine", "ms_total")] + \
              [("final_level", C.c_int32), ("maximal", C.c_int32)] + \
              [(n, C.c_uint64) for n in ("cap_passes", "cap_steps")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class InstanceDesc(C.Structure):
    _fields_ = [("dim", C.c_int), ("sup", C.c_double * MAX_DIM), ("radius", C.c_double), ("seed", C.c_uint64)]


class BatchStats(C.Structure):
    _fields_ = [("seconds", C.c_double)] + [(n, C.c_uint64) for n in (
        "waves", "rounds", "darts", "retests", "peak_voxels", "launches", "budget_bytes")] + \
        [("block", (C.c_int32 * 4) * (MAX_DIM + 1))]


_lib = None

_SIGS = {
    "rsagpu_last_error": (C.c_char_p, []),
    "rsagpu_version": (C.c_char_p, []),
    "rsagpu_kernel_launches": (C.c_uint64, []),
    "rsagpu_domain_create": (C.c_int, [C.c_int, _d, _d, C.c_double, C.POINTER(_vp)]),
    "rsagpu_domain_destroy": (C.c_int, [_vp]),
    "rsagpu_domain_total_volume": (C.c_int, [_vp, _d]),
    "rsagpu_domain_spheres_volume": (C.c_int, [_vp, _d]),
    "rsagpu_domain_count": (C.c_int, [_vp, _u64]),
    "rsagpu_domain_extract": (C.c_int, [_vp, _d, _d, _i32, C.c_uint64, _u64]),
    "rsagpu_domain_check": (C.c_int, [_vp, _u64, _u64]),
    "rsagpu_radgen_create_counts": (C.c_int, [C.c_int, _d, _u64, _i32, C.c_int, C.c_double, C.POINTER(_vp)]),
    "rsagpu_radgen_create_uniform": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_uint64, C.c_int, C.POINTER(_vp)]),
    "rsagpu_radgen_create_table": (C.c_int, [C.c_int, _d, C.c_int, C.c_uint64, C.c_int, C.POINTER(_vp)]),
    "rsagpu_radgen_create_fractions": (C.c_int, [C.c_int, _d, _d, _i32, C.c_int, C.c_double, C.c_double,
                                                 C.POINTER(_vp)]),
    "rsagpu_radgen_destroy": (C.c_int, [_vp]),
    "rsagpu_radgen_max_radius": (C.c_int, [_vp, _d]),
    "rsagpu_radgen_min_radius": (C.c_int, [_vp, _d]),
    "rsagpu_algo_create": (C.c_int, [_vp, _vp, C.c_int, C.POINTER(_vp)]),
    "rsagpu_algo_destroy": (C.c_int, [_vp]),
    "rsagpu_algo_set_form": (C.c_int, [_vp, C.c_int, C.c_int]),
    "rsagpu_algo_set_inherit": (C.c_int, [_vp, C.c_int]),
    "rsagpu_algo_set_cap_rule": (C.c_int, [_vp, C.c_int]),
    "rsagpu_algo_set_schedule_params": (C.c_int, [_vp, C.c_double, C.c_uint64, C.c_uint64, C.c_double]),
    "rsagpu_algo_set_mlp": (C.c_int, [_vp, _u16, C.c_uint64]),
    "rsagpu_algo_proceed": (C.c_int, [_vp, C.c_uint64]),
    "rsagpu_algo_reset_radgen": (C.c_int, [_vp, _vp]),
    "rsagpu_algo_trace": (C.c_int, [_vp, _u64, _u64, _u64, _u8, C.POINTER(C.c_int32), C.c_uint64, _u64]),
    "rsagpu_algo_stats": (C.c_int, [_vp, C.POINTER(Stats)]),
    "rsagpu_algo_set_timing": (C.c_int, [_vp, C.c_int]),
    "rsagpu_algo_kernel_profile": (C.c_int, [_vp, _d, _d, _d, C.c_uint64, _u64]),
    "rsagpu_algo_set_exploration": (C.c_int, [_vp, C.c_double, C.c_uint64]),
    "rsagpu_algo_trace_features": (C.c_int, [_vp, _f32, _u8, _d, _d, C.c_uint64, _u64]),
    "rsagpu_algo_begin": (C.c_int, [_vp]),
    "rsagpu_algo_replay_round": (C.c_int, [_vp, C.c_uint64, _d, _u64, _d, _i32, C.c_uint64, C.c_int, _u8, _u64]),
    "rsagpu_algo_end_round": (C.c_int, [_vp, C.c_uint64, C.c_uint64, _i32, _i32]),
    "rsagpu_algo_refine": (C.c_int, [_vp]),
    "rsagpu_algo_voxels": (C.c_int, [_vp, _i64, C.c_uint64, _u64, C.POINTER(C.c_int32), _d]),
    "rsagpu_algo_draw_darts": (C.c_int, [_vp, C.c_uint64, C.c_uint64, C.c_uint64, _d, _u64, _u64]),
    "rsagpu_batch_run": (C.c_int, [C.POINTER(InstanceDesc), C.c_int, C.c_int, C.c_uint64, C.c_int, _u64, _u64, _d,
                                   C.POINTER(BatchStats)]),
    "rsagpu_mlp_forward": (C.c_int, [_u16, _f32, C.c_uint64, _f32]),
    "rsagpu_resolve_batch_noalloc": (C.c_int, [C.c_int, _d, _d, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.c_uint64, C.c_void_p, C.c_void_p]),
    "rsagpu_mlp_train_step": (C.c_int, [_f32, _u16, _f32, _f32, C.c_uint64, C.c_float, _f32, _f32]),
}


def header_symbols() -> list[str]:
    """Every function declared by include/rsagpu.h."""
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(rsagpu_\w+)\s*\(", txt, flags=re.M)))


def lib():
    """Loads the library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RsaGpuError(-2, f"{LIB_PATH} is missing: run __graft_entry__.build() (nvcc, sm_103a)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(code: int) -> None:
    if code != 0:
        raise RsaGpuError(code, lib().rsagpu_last_error().decode(errors="replace"))


def ptr(a, t):
    return a.ctypes.data_as(t)
