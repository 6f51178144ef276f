"""ctypes access to oracle/_ref/libqfref.so: the reference's own evaluator and
learner compiled from its sources (see oracle/build_ref.sh).

TEST INFRASTRUCTURE ONLY: used to produce and check golden fixtures in this
checkout; the library does not exist where the reference sources are absent,
and the GPU tests read the committed fixtures instead.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import List, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libqfref.so")
_lib = None


def reference_dir():
    """The reference checkout oracle/build_ref.sh reads (QF_REFERENCE or the
    script's default), or None when its sources are absent."""
    res = subprocess.run(["bash", os.path.join(_HERE, "build_ref.sh"), "--where"],
                         capture_output=True, text=True)
    return res.stdout.strip() if res.returncode == 0 else None


def available() -> bool:
    return os.path.exists(LIB_PATH) or reference_dir() is not None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            subprocess.check_call(["bash", os.path.join(_HERE, "build_ref.sh")])
        L = ctypes.CDLL(LIB_PATH)
        i32p = ctypes.POINTER(ctypes.c_int32)
        i64p = ctypes.POINTER(ctypes.c_int64)
        L.qfref_evaluate.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), i64p,
                                     ctypes.POINTER(i32p), ctypes.c_int, ctypes.POINTER(i32p),
                                     ctypes.c_int64, ctypes.c_int64, ctypes.c_int, i32p,
                                     ctypes.c_int, i64p]
        L.qfref_evaluate.restype = ctypes.c_int
        L.qfref_learn.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), i64p,
                                  ctypes.POINTER(i32p), ctypes.c_int, ctypes.c_int64,
                                  ctypes.c_int64, ctypes.POINTER(i32p), ctypes.c_int,
                                  ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]
        L.qfref_learn.restype = ctypes.c_int
        L.qfref_coverage.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), i64p,
                                     ctypes.POINTER(i32p), ctypes.c_int, ctypes.c_int64,
                                     ctypes.c_int64, ctypes.POINTER(i32p), ctypes.c_int,
                                     ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(i32p), i32p,
                                     ctypes.c_int64, ctypes.POINTER(i32p), i64p,
                                     ctypes.POINTER(ctypes.c_uint8)]
        L.qfref_coverage.restype = ctypes.c_int
        L.qfref_learn_test.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), i64p,
                                       ctypes.POINTER(i32p), ctypes.c_int, ctypes.c_int64,
                                       ctypes.c_int64, ctypes.POINTER(i32p), ctypes.c_int,
                                       ctypes.c_int64, ctypes.POINTER(i32p), ctypes.c_int64,
                                       ctypes.POINTER(i32p), ctypes.c_char_p, ctypes.c_int, i64p]
        L.qfref_learn_test.restype = ctypes.c_int
        L.qfref_load_text.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(i32p), ctypes.c_int64, i64p]
        L.qfref_load_text.restype = ctypes.c_int
        L.qfref_learn_compact.argtypes = L.qfref_learn.argtypes + [ctypes.POINTER(ctypes.c_double)]
        L.qfref_learn_compact.restype = ctypes.c_int
        L.qfref_build_after_semijoin.argtypes = [ctypes.c_int, ctypes.POINTER(i32p), ctypes.c_int64,
                                                 ctypes.POINTER(ctypes.c_uint64), ctypes.c_int64,
                                                 ctypes.c_int32, i32p, i32p,
                                                 ctypes.POINTER(ctypes.c_uint32)]
        L.qfref_build_after_semijoin.restype = ctypes.c_int
        _lib = L
    return _lib


def _cols(arrays):
    arrs = [np.ascontiguousarray(a, dtype=np.int32) for a in arrays]
    ptrs = (ctypes.POINTER(ctypes.c_int32) * max(1, len(arrs)))(
        *[a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)) for a in arrs])
    return arrs, ptrs


def _relations(relations):
    flat = [c for r in relations for c in r]
    keep, ptrs = _cols(flat)
    ncols = (ctypes.c_int * max(1, len(relations)))(*[len(r) for r in relations])
    ntup = (ctypes.c_int64 * max(1, len(relations)))(*[len(r[0]) for r in relations])
    return keep, ptrs, ncols, ntup


def evaluate(relations, binding_columns, num_positive: int, literals, radix_bits: int = 5):
    """The reference's CandidateLiteralEvaluator on one binding set, one
    Evaluate call per clause join variable; counts [n, 4] in the order of
    `literals` ((relation, vars, join_pos) or Literal)."""
    keep_r, rptr, rnc, rnt = _relations(relations)
    keep_b, bptr = _cols(binding_columns)
    n = len(keep_b[0]) if keep_b else 0
    desc = np.full((max(1, len(literals)), 10), -1, dtype=np.int32)
    for k, lit in enumerate(literals):
        rel, vars_, _ = lit.as_tuple() if hasattr(lit, "as_tuple") else lit
        desc[k, 0] = rel
        desc[k, 1] = len(vars_)
        desc[k, 2:2 + len(vars_)] = vars_
    counts = np.zeros((max(1, len(literals)), 4), dtype=np.int64)
    rc = lib().qfref_evaluate(len(relations), rnc, rnt, rptr, len(keep_b), bptr, num_positive,
                              n - num_positive, len(literals),
                              desc.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), radix_bits,
                              counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    if rc != 0:
        raise ValueError(f"reference driver rejected the input ({rc})")
    return counts[:len(literals)]


def learn(relations, target_columns, num_positive: int, max_clause_length: int,
          trace_path: str = None) -> List[str]:
    """Runs the reference learner; returns its learnt clauses (ToString)."""
    keep_r, rptr, rnc, rnt = _relations(relations)
    keep_t, tptr = _cols(target_columns)
    out = ctypes.create_string_buffer(1 << 16)
    rc = lib().qfref_learn(len(relations), rnc, rnt, rptr, len(keep_t), len(keep_t[0]),
                           num_positive, tptr, max_clause_length,
                           trace_path.encode() if trace_path else None, out, len(out))
    if rc != 0:
        raise RuntimeError(f"reference learner failed ({rc})")
    return [l for l in out.value.decode().splitlines() if l]


def learn_compact(relations, target_columns, num_positive: int, max_clause_length: int,
                  trace_path: str):
    """Runs the reference learner with the compact trace (column checksums,
    coverage steps; see oracle/ref_driver.cpp); returns (learnt clauses,
    seconds in Learn, inside Evaluate, inside extensions, inside coverage)."""
    keep_r, rptr, rnc, rnt = _relations(relations)
    keep_t, tptr = _cols(target_columns)
    out = ctypes.create_string_buffer(1 << 16)
    secs = (ctypes.c_double * 4)()
    rc = lib().qfref_learn_compact(len(relations), rnc, rnt, rptr, len(keep_t), len(keep_t[0]),
                                   num_positive, tptr, max_clause_length, trace_path.encode(), out,
                                   len(out), secs)
    if rc != 0:
        raise RuntimeError(f"reference learner failed ({rc})")
    return [l for l in out.value.decode().splitlines() if l], tuple(secs)


def coverage(relations, target_columns, target_num_positive: int, binding_columns,
             bind_num_positive: int, literal, uncovered_columns):
    """QuickFoil::ComputeCoverageOnUncoveredData (learner/QuickFoil.cpp:471-573)
    for `literal` appended to a building clause whose binding set is
    `binding_columns` (first bind_num_positive rows positive, the first
    len(target_columns) columns the target's variables).  The target's
    negatives (rows from target_num_positive on) are the original negative
    data.  Returns ((covered positives, covered negatives), uint8 flag per
    uncovered positive row)."""
    keep_r, rptr, rnc, rnt = _relations(relations)
    keep_t, tptr = _cols(target_columns)
    keep_b, bptr = _cols(binding_columns)
    keep_u, uptr = _cols(uncovered_columns)
    rel, vars_, _ = literal.as_tuple() if hasattr(literal, "as_tuple") else literal
    desc = np.full(10, -1, dtype=np.int32)
    desc[0] = rel
    desc[1] = len(vars_)
    desc[2:2 + len(vars_)] = vars_
    nb = len(keep_b[0])
    nu = len(keep_u[0])
    counts = np.zeros(2, dtype=np.int64)
    covered = np.zeros(max(1, nu), dtype=np.uint8)
    rc = lib().qfref_coverage(len(relations), rnc, rnt, rptr, len(keep_t), len(keep_t[0]),
                              target_num_positive, tptr, len(keep_b), bind_num_positive,
                              nb - bind_num_positive, bptr,
                              desc.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), nu, uptr,
                              counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                              covered.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    if rc != 0:
        raise ValueError(f"reference driver rejected the input ({rc})")
    return (int(counts[0]), int(counts[1])), covered[:nu].astype(bool)


def learn_test(relations, target_columns, num_positive: int, max_clause_length: int,
               test_positive, test_negative):
    """Runs the reference learner, then its test runner on the two test
    tables; returns (learnt clauses, (uncovered test positives, uncovered
    test negatives))."""
    keep_r, rptr, rnc, rnt = _relations(relations)
    keep_t, tptr = _cols(target_columns)
    keep_p, pptr = _cols(test_positive)
    keep_n, nptr = _cols(test_negative)
    out = ctypes.create_string_buffer(1 << 16)
    unc = np.zeros(2, dtype=np.int64)
    rc = lib().qfref_learn_test(len(relations), rnc, rnt, rptr, len(keep_t), len(keep_t[0]),
                                num_positive, tptr, max_clause_length, len(keep_p[0]), pptr,
                                len(keep_n[0]), nptr, out, len(out),
                                unc.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    if rc != 0:
        raise RuntimeError(f"reference learner failed ({rc})")
    return [l for l in out.value.decode().splitlines() if l], (int(unc[0]), int(unc[1]))


def load_text(path: str, num_args: int, skipped=None):
    """The reference's LoadData (main/main.cpp:49-109) on a file: the kept
    argument columns.  A line the reference rejects aborts the process, so
    only valid files are given to it."""
    with open(path, "rb") as f:
        cap = f.read().count(b"\n") + 1
    skip = (ctypes.c_int * num_args)(*[int(bool(x)) for x in (skipped or [0] * num_args)])
    kept = num_args - sum(1 for x in (skipped or []) if x)
    outs = [np.zeros(cap, dtype=np.int32) for _ in range(max(kept, 1))]
    keep, ptrs = _cols(outs)
    rows = ctypes.c_int64()
    rc = lib().qfref_load_text(path.encode(), num_args, skip, ptrs, cap, ctypes.byref(rows))
    if rc != 0:
        raise RuntimeError(f"reference loader: {rc}")
    return [o[:rows.value] for o in keep[:kept]]


def build_after_semijoin(keys, bits, chunk_rows: int, num_build_tuples: int, num_rows=None):
    """The reference's BuildHashTableAfterSemiJoin (operations/BuildHashTable.
    cpp:212-236) over the first num_rows rows (default: all) of `keys`
    (projected columns, which may run longer) cut into chunk_rows-row chunks
    with their semi-join bits (uint64 blocks); returns (buckets, next, mask)
    with next[] zero at positions no chain reaches."""
    keep, ptrs = _cols(keys)
    n = len(keep[0]) if num_rows is None else num_rows
    bits = np.ascontiguousarray(bits, dtype=np.uint64)
    nb = 1
    while nb < num_build_tuples:
        nb <<= 1
    buckets = np.zeros(nb, dtype=np.int32)
    nxt = np.zeros(num_build_tuples, dtype=np.int32)
    mask = ctypes.c_uint32()
    rc = lib().qfref_build_after_semijoin(
        len(keep), ptrs, n, bits.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), chunk_rows,
        num_build_tuples, buckets.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
        nxt.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), ctypes.byref(mask))
    if rc != 0:
        raise ValueError(f"reference driver rejected the input ({rc})")
    return buckets, nxt, int(mask.value)
