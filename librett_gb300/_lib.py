"""ctypes binding of librett.so's C-ABI (include/librett_c.h).

The library is built in-tree by ``python -m librett_gb300.build`` (or
``__graft_entry__.build()``).  Loading fails loudly when it is missing: there
is no fallback implementation.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "librett.so"

MAXR = 16


class PlanInfo(ctypes.Structure):
    """Mirror of ``librett_plan_info`` in include/librett_c.h."""

    _fields_ = [
        ("method", ctypes.c_int),
        ("element_bytes", ctypes.c_int),
        ("fused_rank", ctypes.c_int),
        ("fused_perm", ctypes.c_int * MAXR),
        ("fused_dim", ctypes.c_longlong * MAXR),
        ("tile_extent", ctypes.c_longlong * MAXR),
        ("volume", ctypes.c_longlong),
        ("num_tiles", ctypes.c_longlong),
        ("threads", ctypes.c_int),
        ("slots", ctypes.c_int),
        ("smem_bytes", ctypes.c_int),
        ("pad_shift", ctypes.c_int),
        ("pipeline", ctypes.c_int),
        ("unit_in_bytes", ctypes.c_int),
        ("unit_out_bytes", ctypes.c_int),
        ("run_in_bytes", ctypes.c_int),
        ("run_out_bytes", ctypes.c_int),
        ("grid", ctypes.c_int),
        ("candidate", ctypes.c_int),
        ("num_candidates", ctypes.c_int),
        ("model_cost", ctypes.c_double),
        ("selected_by", ctypes.c_int),
        ("table_bytes", ctypes.c_int),
    ]

    def as_dict(self) -> dict:
        r = self.fused_rank
        return {
            "method": self.method,
            "element_bytes": self.element_bytes,
            "fused_rank": r,
            "fused_dim": list(self.fused_dim[:r]),
            "fused_perm": list(self.fused_perm[:r]),
            "tile_extent": list(self.tile_extent[:r]),
            "volume": self.volume,
            "num_tiles": self.num_tiles,
            "threads": self.threads,
            "slots": self.slots,
            "smem_bytes": self.smem_bytes,
            "pad_shift": self.pad_shift,
            "pipeline": self.pipeline,
            "unit_in_bytes": self.unit_in_bytes,
            "unit_out_bytes": self.unit_out_bytes,
            "run_in_bytes": self.run_in_bytes,
            "run_out_bytes": self.run_out_bytes,
            "grid": self.grid,
            "candidate": self.candidate,
            "num_candidates": self.num_candidates,
            "model_cost": self.model_cost,
            "selected_by": self.selected_by,
            "table_bytes": self.table_bytes,
        }


# (name, restype, argtypes) of every extern "C" symbol in include/librett_c.h.
_H = ctypes.c_uint
_P = ctypes.c_void_p
_IP = ctypes.POINTER(ctypes.c_int)
C_FUNCTIONS = [
    ("librett_c_initialize", None, []),
    ("librett_c_finalize", None, []),
    ("librett_c_plan", ctypes.c_int,
     [ctypes.POINTER(_H), ctypes.c_int, _IP, _IP, ctypes.c_size_t, _P]),
    ("librett_c_plan_measure", ctypes.c_int,
     [ctypes.POINTER(_H), ctypes.c_int, _IP, _IP, ctypes.c_size_t, _P, _P, _P]),
    ("librett_c_execute", ctypes.c_int, [_H, _P, _P]),
    ("librett_c_destroy", ctypes.c_int, [_H]),
    ("librett_c_plan_info", ctypes.c_int, [_H, ctypes.POINTER(PlanInfo)]),
    ("librett_c_describe", ctypes.c_int,
     [ctypes.c_int, _IP, _IP, ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
      ctypes.POINTER(PlanInfo)]),
    ("librett_c_plan_candidate", ctypes.c_int,
     [ctypes.POINTER(_H), ctypes.c_int, _IP, _IP, ctypes.c_size_t, _P, ctypes.c_int]),
    ("librett_c_transpose_noalloc", ctypes.c_int,
     [ctypes.c_int, _IP, _IP, ctypes.c_size_t, _P, _P, _P]),
    ("librett_c_candidate_features", ctypes.c_int,
     [ctypes.c_int, _IP, _IP, ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
      ctypes.POINTER(ctypes.c_float), ctypes.c_int]),
    ("librett_c_set_candidate_set", ctypes.c_int, [ctypes.c_int]),
    ("librett_c_set_plan_selector", ctypes.c_int, [ctypes.c_int]),
    ("librett_c_set_plan_cache", ctypes.c_int, [ctypes.c_int]),
    ("librett_c_plan_cache_stats", ctypes.c_int,
     [ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong),
      ctypes.POINTER(ctypes.c_int)]),
    ("librett_c_load_plan_model", ctypes.c_int, [ctypes.c_char_p]),
    ("librett_c_mlp_param_count", ctypes.c_int, []),
    ("librett_c_mlp_feature_count", ctypes.c_int, []),
    ("librett_c_mlp_workspace_floats", ctypes.c_int, [ctypes.c_int]),
    ("librett_c_mlp_forward", ctypes.c_int, [_P, _P, ctypes.c_int, _P, _P, _P]),
    ("librett_c_mlp_backward", ctypes.c_int, [_P, _P, ctypes.c_int, _P, _P, _P, _P]),
    ("librett_c_mlp_mse_grad", ctypes.c_int, [_P, _P, ctypes.c_int, _P, _P, _P]),
    ("librett_c_mlp_adam", ctypes.c_int,
     [_P, _P, _P, _P, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float,
      ctypes.c_float, ctypes.c_int, _P]),
    ("librett_c_mlp_predict_host", ctypes.c_int,
     [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float), ctypes.c_int,
      ctypes.POINTER(ctypes.c_float)]),
    ("librett_c_group_create", ctypes.c_int,
     [ctypes.POINTER(_H), ctypes.c_int, ctypes.POINTER(_H), ctypes.POINTER(_P),
      ctypes.POINTER(_P), _P]),
    ("librett_c_group_create_policy", ctypes.c_int,
     [ctypes.POINTER(_H), ctypes.c_int, ctypes.POINTER(_H), ctypes.POINTER(_P),
      ctypes.POINTER(_P), _P, ctypes.POINTER(ctypes.c_int)]),
    ("librett_c_group_tune", ctypes.c_int, [_H]),
    ("librett_c_group_bucket", ctypes.c_int,
     [_H, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
      ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]),
    ("librett_c_group_policy", ctypes.c_int,
     [_H, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    ("librett_c_group_execute", ctypes.c_int, [_H]),
    ("librett_c_group_destroy", ctypes.c_int, [_H]),
    ("librett_c_execute_grouped", ctypes.c_int,
     [ctypes.c_int, ctypes.POINTER(_H), ctypes.POINTER(_P), ctypes.POINTER(_P)]),
    ("librett_c_verify", ctypes.c_int,
     [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), ctypes.c_size_t,
      _P, _P, _P, ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_longlong)]),
    ("librett_c_group_run_check", ctypes.c_int,
     [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), ctypes.c_size_t,
      ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    ("librett_c_bulk_check", ctypes.c_int,
     [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), ctypes.c_size_t,
      ctypes.c_int, ctypes.c_int]),
    ("librett_c_plan_batch", ctypes.c_int,
     [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
      ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_size_t), _P, ctypes.c_int,
      ctypes.POINTER(_H), ctypes.POINTER(ctypes.c_double)]),
    ("librett_c_execute_batch", ctypes.c_int,
     [ctypes.c_int, ctypes.POINTER(_H), ctypes.POINTER(_P), ctypes.POINTER(_P)]),
    ("librett_c_group_info", ctypes.c_int,
     [_H, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
      ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_longlong),
      ctypes.POINTER(ctypes.c_longlong)]),
    ("librett_c_launch_count", ctypes.c_ulonglong, []),
    ("librett_c_table_arena_stats", ctypes.c_int,
     [ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong),
      ctypes.POINTER(ctypes.c_longlong)]),
    ("librett_c_inject_fault", ctypes.c_int, [ctypes.c_int, ctypes.c_longlong]),
    ("librett_c_plan_status", ctypes.c_int, [_H, ctypes.POINTER(ctypes.c_uint)]),
    ("librett_c_bulk_wait_test", ctypes.c_int,
     [_H, _P, _P, ctypes.c_uint, ctypes.POINTER(ctypes.c_uint)]),
    ("librett_c_result_string", ctypes.c_char_p, [ctypes.c_int]),
]

# The C++ (LibreTT-compatible) symbols, by their mangled names.
CXX_SYMBOLS = [
    "_Z17librettInitializev",
    "_Z15librettFinalizev",
    "_Z11librettPlanPjiPiS0_mRP11CUstream_st",
    "_Z18librettPlanMeasurePjiPiS0_mRP11CUstream_stPvS4_",
    "_Z14librettDestroyj",
    "_Z14librettExecutejPvS_",
]

# C++ entry points with no LibreTT counterpart (grouped execution).
CXX_GROUP_SYMBOLS = ["librettGroupCreate", "librettGroupTune", "librettGroupExecute",
                     "librettGroupDestroy", "librettExecuteGrouped"]

_lib = None


def load() -> ctypes.CDLL:
    """Load librett.so (once) and declare the C-ABI signatures."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m librett_gb300.build`; "
                "the transpose engine has no non-CUDA fallback")
        lib = ctypes.CDLL(str(LIB_PATH))
        for name, res, args in C_FUNCTIONS:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def int_array(seq) -> ctypes.Array:
    return (ctypes.c_int * len(seq))(*[int(x) for x in seq])
