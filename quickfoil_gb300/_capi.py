"""ctypes binding of libqfgpu.so (the C ABI declared in include/qfgpu.h).

There is no fallback: if the library is missing or a call fails, an
exception is raised.  ``build()`` in ``quickfoil_gb300._build`` produces the
library in-tree.
"""
from __future__ import annotations

import ctypes
import os

from . import _build

MAX_ARITY = 8
MAX_RADIX_BITS = 15

QFG_OK = 0
QFG_ERR_INVALID = 1
QFG_ERR_OOM = 2
QFG_ERR_BUDGET = 3
QFG_ERR_CUDA = 4
QFG_ERR_TIMEOUT = 5
QFG_ERR_NOT_FOUND = 6
QFG_ERR_MISMATCH = 7

QFG_HOST = 0
QFG_DEVICE_COPY = 1
QFG_DEVICE_BORROW = 2

QFG_COUNTS_HOST = 0
QFG_COUNTS_DEVICE = 1

QFG_OPT_NUM_RADIX_BITS = 1
QFG_OPT_EVAL_BITS = 2
QFG_OPT_WAIT_LIMIT = 3
QFG_OPT_USE_GRAPHS = 4
QFG_OPT_STAGE_TIMING = 5
QFG_OPT_SHARD_INDEX = 6
QFG_OPT_SHARD_COUNT = 7
QFG_OPT_AUTOTUNE = 8
QFG_OPT_PASS1_BITS = 9
QFG_OPT_SERVER_DEPTH = 10
QFG_OPT_TEST_WITHHOLD_COPIES = 11
QFG_OPT_COVERAGE_COMPAT = 12
QFG_OPT_EVAL_MODE = 13

STAGES = ("key_tables", "bind_partition", "evaluate", "per_literal", "unit_plan",
          "coverage_scan", "coverage_examples")


class QfgLiteral(ctypes.Structure):
    _fields_ = [("relation_id", ctypes.c_int32),
                ("num_args", ctypes.c_int32),
                ("join_pos", ctypes.c_int32),
                ("vars", ctypes.c_int32 * MAX_ARITY)]


class QfgError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


c_i32p = ctypes.POINTER(ctypes.c_int32)
c_i64p = ctypes.POINTER(ctypes.c_int64)
c_u32p = ctypes.POINTER(ctypes.c_uint32)
c_u64p = ctypes.POINTER(ctypes.c_uint64)
c_vp = ctypes.c_void_p

# (name, restype, argtypes) for every exported entry point.
SIGNATURES = [
    ("qfg_version", ctypes.c_int, []),
    ("qfg_status_string", ctypes.c_char_p, [ctypes.c_int]),
    ("qfg_ctx_create", ctypes.c_int, [ctypes.c_int, ctypes.c_int64, ctypes.POINTER(c_vp)]),
    ("qfg_ctx_destroy", ctypes.c_int, [c_vp]),
    ("qfg_ctx_last_error", ctypes.c_char_p, [c_vp]),
    ("qfg_ctx_set_stream", ctypes.c_int, [c_vp, c_vp]),
    ("qfg_ctx_synchronize", ctypes.c_int, [c_vp]),
    ("qfg_ctx_set_option", ctypes.c_int, [c_vp, ctypes.c_int, ctypes.c_int64]),
    ("qfg_ctx_memory", ctypes.c_int, [c_vp, c_i64p, c_i64p]),
    ("qfg_ctx_kernel_launches", ctypes.c_int, [c_vp, c_i64p]),
    ("qfg_ctx_stage_times", ctypes.c_int,
     [c_vp, ctypes.POINTER(ctypes.c_double), c_i64p, ctypes.c_int]),
    ("qfg_relation_register", ctypes.c_int,
     [c_vp, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(c_vp), ctypes.c_int64, ctypes.c_int]),
    ("qfg_relation_release", ctypes.c_int, [c_vp, ctypes.c_int32]),
    ("qfg_bindings_create", ctypes.c_int,
     [c_vp, ctypes.c_int32, ctypes.POINTER(c_vp), ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
      ctypes.POINTER(c_vp)]),
    ("qfg_bindings_create_split", ctypes.c_int,
     [c_vp, ctypes.c_int32, ctypes.POINTER(c_vp), ctypes.c_int64, ctypes.POINTER(c_vp),
      ctypes.c_int64, ctypes.c_int, ctypes.POINTER(c_vp)]),
    ("qfg_bindings_destroy", ctypes.c_int, [c_vp, c_vp]),
    ("qfg_bindings_info", ctypes.c_int, [c_vp, c_i32p, c_i64p, c_i64p]),
    ("qfg_bindings_column", ctypes.c_int, [c_vp, ctypes.c_int32, ctypes.POINTER(c_vp)]),
    ("qfg_bindings_download", ctypes.c_int, [c_vp, c_vp, ctypes.POINTER(c_vp)]),
    ("qfg_evaluate_group", ctypes.c_int,
     [c_vp, c_vp, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(QfgLiteral), c_i64p, ctypes.c_int]),
    ("qfg_evaluate_step", ctypes.c_int,
     [c_vp, c_vp, ctypes.c_int32, ctypes.POINTER(QfgLiteral), c_i64p, ctypes.c_int]),
    ("qfg_evaluate_per_literal", ctypes.c_int,
     [c_vp, c_vp, ctypes.c_int32, ctypes.POINTER(QfgLiteral), c_i64p, ctypes.c_int]),
    ("qfg_step_traffic", ctypes.c_int,
     [c_vp, c_vp, ctypes.c_int32, ctypes.POINTER(QfgLiteral), c_i64p]),
    ("qfg_autotune_step", ctypes.c_int,
     [c_vp, c_vp, ctypes.c_int32, ctypes.POINTER(QfgLiteral), c_i32p, c_i32p,
      ctypes.POINTER(ctypes.c_double)]),
    ("qfg_autotune_choice", ctypes.c_int,
     [c_vp, ctypes.c_int64, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
      ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]),
    ("qfg_step_scratch_bytes", ctypes.c_int,
     [c_vp, c_vp, ctypes.c_int32, ctypes.POINTER(QfgLiteral), c_i64p]),
    ("qfg_step_graph_create", ctypes.c_int,
     [c_vp, c_vp, ctypes.c_int32, ctypes.POINTER(QfgLiteral), c_vp, ctypes.POINTER(c_vp)]),
    ("qfg_step_graph_launch", ctypes.c_int, [c_vp, c_vp]),
    ("qfg_step_graph_destroy", ctypes.c_int, [c_vp, c_vp]),
    ("qfg_server_create", ctypes.c_int, [c_vp, ctypes.c_int32, ctypes.c_int64, ctypes.POINTER(c_vp)]),
    ("qfg_server_submit", ctypes.c_int,
     [c_vp, c_vp, ctypes.c_int32, ctypes.POINTER(QfgLiteral), c_i64p, c_i64p]),
    ("qfg_server_poll", ctypes.c_int, [c_vp, c_i64p, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]),
    ("qfg_server_wait", ctypes.c_int, [c_vp, ctypes.c_int64]),
    ("qfg_server_drain", ctypes.c_int, [c_vp]),
    ("qfg_server_stats", ctypes.c_int,
     [c_vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), c_i64p, c_i64p]),
    ("qfg_server_reset_stats", ctypes.c_int, [c_vp]),
    ("qfg_server_destroy", ctypes.c_int, [c_vp]),
    ("qfg_radix_partition", ctypes.c_int,
     [c_vp, c_vp, ctypes.c_int64, ctypes.c_int, c_vp, c_vp]),
    ("qfg_radix_partition_static", ctypes.c_int,
     [c_vp, c_vp, ctypes.c_int64, ctypes.c_int, c_vp, c_vp, ctypes.c_char_p, ctypes.c_int]),
    ("qfg_build_hash_table_on_partitions", ctypes.c_int,
     [c_vp, c_vp, c_vp, ctypes.c_int64, ctypes.c_int, c_vp, c_vp, c_vp, c_vp]),
    ("qfg_build_hash_table_on_table", ctypes.c_int,
     [c_vp, ctypes.POINTER(c_vp), ctypes.c_int32, ctypes.c_int64, c_vp, c_vp, c_u32p]),
    ("qfg_build_hash_table_after_semijoin", ctypes.c_int,
     [c_vp, ctypes.POINTER(c_vp), ctypes.c_int32, ctypes.c_int64, c_vp, ctypes.c_int64,
      ctypes.c_int32, c_vp, c_vp, c_u32p]),
    ("qfg_left_semijoin", ctypes.c_int,
     [c_vp, ctypes.POINTER(c_vp), ctypes.c_int64, ctypes.POINTER(c_vp), ctypes.c_int64,
      ctypes.c_int32, c_vp, c_i64p]),
    ("qfg_right_semijoin", ctypes.c_int,
     [c_vp, ctypes.POINTER(c_vp), ctypes.c_int64, ctypes.POINTER(c_vp), ctypes.c_int64,
      ctypes.c_int32, c_vp, c_i64p]),
    ("qfg_extend_bindings", ctypes.c_int,
     [c_vp, c_vp, ctypes.POINTER(QfgLiteral), ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(c_vp)]),
    ("qfg_coverage", ctypes.c_int,
     [c_vp, c_vp, ctypes.POINTER(QfgLiteral), ctypes.c_int32, ctypes.POINTER(c_vp), ctypes.c_int64,
      ctypes.POINTER(c_vp), ctypes.c_int64, c_vp, c_i64p]),
    ("qfg_examples_create", ctypes.c_int,
     [c_vp, ctypes.c_int32, ctypes.POINTER(c_vp), ctypes.c_int64, ctypes.POINTER(c_vp)]),
    ("qfg_examples_destroy", ctypes.c_int, [c_vp, c_vp]),
    ("qfg_coverage_examples", ctypes.c_int,
     [c_vp, c_vp, ctypes.POINTER(QfgLiteral), c_vp, c_vp, c_vp, c_i64p]),
    ("qfg_run_test", ctypes.c_int,
     [c_vp, ctypes.c_int32, c_i32p, ctypes.POINTER(QfgLiteral), ctypes.c_int32,
      ctypes.POINTER(c_vp), ctypes.c_int64, c_i64p, ctypes.POINTER(c_vp)]),
    ("qfg_parse_text", ctypes.c_int,
     [c_vp, ctypes.c_char_p, ctypes.c_int64, ctypes.c_int, ctypes.c_int32, c_i32p,
      ctypes.POINTER(c_vp), ctypes.c_int64, c_i64p, c_i64p]),
    ("qfg_relation_register_text", ctypes.c_int,
     [c_vp, ctypes.c_int32, ctypes.c_char_p, ctypes.c_int64, ctypes.c_int, ctypes.c_int32, c_i32p,
      c_i64p, c_i64p]),
    ("qfg_compact_rows", ctypes.c_int,
     [c_vp, ctypes.c_int32, ctypes.POINTER(c_vp), ctypes.c_int64, c_vp, ctypes.c_int32,
      ctypes.POINTER(c_vp), ctypes.c_int64, c_i64p]),
]

_lib = None


def library_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Loads libqfgpu.so (building it first when it is absent or stale and a
    CUDA toolkit is present).  Raises if it cannot be loaded."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"libqfgpu.so is missing at {path}; run quickfoil_gb300._build.build()")
    lib = ctypes.CDLL(path)
    for name, restype, argtypes in SIGNATURES:
        f = getattr(lib, name)
        f.restype = restype
        f.argtypes = argtypes
    _lib = lib
    return lib


def check(status: int, ctx=None, what: str = "") -> None:
    if status == QFG_OK:
        return
    lib = load()
    msg = lib.qfg_status_string(status).decode()
    detail = lib.qfg_ctx_last_error(ctx).decode() if ctx else ""
    raise QfgError(status, f"{what}: {msg}" + (f" ({detail})" if detail else ""))


def ptr_array(ptrs):
    arr = (c_vp * max(1, len(ptrs)))()
    for i, p in enumerate(ptrs):
        arr[i] = p
    return arr
