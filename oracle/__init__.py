"""CPU oracle for the QuickFOIL candidate-literal hot path.

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, by ``__graft_entry__.smoke``
and by the CPU-baseline leg of ``bench.py`` as the checker.  The product
package (``quickfoil_gb300``) never imports this module.

``qf_oracle.c`` restates the reference operator chain in plain C; this module
compiles it with gcc (``build()``) and exposes it through ctypes.  The
restatement is pinned against the reference's own RadixPartition test cases
and against count fixtures produced by the reference's own sources
(``tests/golden``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_DIR = os.path.join(_HERE, "_lib")
_LIB_PATH = os.path.join(_LIB_DIR, "libqforacle.so")
MAX_ARITY = 8

_lib = None


def build(force: bool = False) -> str:
    """Compile ``qf_oracle.c`` into ``oracle/_lib/libqforacle.so``."""
    src = os.path.join(_HERE, "qf_oracle.c")
    hdr = os.path.join(_HERE, "qf_oracle.h")
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return _LIB_PATH
    os.makedirs(_LIB_DIR, exist_ok=True)
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-pthread",
                           "-Wall", "-o", tmp, src])
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


class _Table(ctypes.Structure):
    _fields_ = [("num_columns", ctypes.c_int32),
                ("num_tuples", ctypes.c_int64),
                ("columns", ctypes.POINTER(ctypes.POINTER(ctypes.c_int32)))]


class _Literal(ctypes.Structure):
    _fields_ = [("relation", ctypes.c_int32),
                ("num_args", ctypes.c_int32),
                ("join_pos", ctypes.c_int32),
                ("vars", ctypes.c_int32 * MAX_ARITY)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        i64p = ctypes.POINTER(ctypes.c_int64)
        i32p = ctypes.POINTER(ctypes.c_int32)
        L.qfo_radix_partition.argtypes = [i32p, ctypes.c_int64, ctypes.c_int, i32p, i64p]
        L.qfo_radix_partition.restype = None
        L.qfo_num_buckets.argtypes = [ctypes.c_int32]
        L.qfo_num_buckets.restype = ctypes.c_int32
        L.qfo_build_partition_hash_table.argtypes = [i32p, ctypes.c_int32, ctypes.c_int, i32p, i32p]
        L.qfo_build_partition_hash_table.restype = ctypes.c_uint32
        L.qfo_build_table_hash_table.argtypes = [ctypes.POINTER(i32p), ctypes.c_int, ctypes.c_int64,
                                                 i32p, i32p]
        L.qfo_build_table_hash_table.restype = ctypes.c_uint32
        L.qfo_build_hash_table_after_semijoin.argtypes = [
            ctypes.POINTER(i32p), ctypes.c_int, ctypes.c_int64, ctypes.POINTER(ctypes.c_uint64),
            ctypes.c_int64, ctypes.c_int32, i32p, i32p]
        L.qfo_build_hash_table_after_semijoin.restype = ctypes.c_uint32
        L.qfo_relcache_create.argtypes = []
        L.qfo_relcache_create.restype = ctypes.c_void_p
        L.qfo_relcache_destroy.argtypes = [ctypes.c_void_p]
        L.qfo_relcache_destroy.restype = None
        L.qfo_evaluate.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Table), ctypes.c_int,
                                   ctypes.POINTER(_Table), ctypes.c_int64,
                                   ctypes.POINTER(_Literal), ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, i64p]
        L.qfo_evaluate.restype = ctypes.c_int
        u64p = ctypes.POINTER(ctypes.c_uint64)
        for name in ("qfo_left_semijoin", "qfo_right_semijoin"):
            f = getattr(L, name)
            f.argtypes = [ctypes.POINTER(i32p), ctypes.c_int64, ctypes.POINTER(i32p),
                          ctypes.c_int64, ctypes.c_int, u64p]
            f.restype = ctypes.c_int64
        L.qfo_extend_bindings.argtypes = [ctypes.POINTER(_Table), ctypes.c_int64,
                                          ctypes.POINTER(_Table), ctypes.POINTER(_Literal),
                                          ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(i32p)]
        L.qfo_extend_bindings.restype = ctypes.c_int
        L.qfo_coverage.argtypes = [ctypes.POINTER(_Table), ctypes.c_int64, ctypes.POINTER(_Table),
                                   ctypes.POINTER(_Literal), ctypes.c_int, ctypes.POINTER(_Table),
                                   ctypes.POINTER(_Table), u64p, i64p]
        L.qfo_coverage.restype = ctypes.c_int
        L.qfo_coverage_compat.argtypes = L.qfo_coverage.argtypes
        L.qfo_coverage_compat.restype = L.qfo_coverage.restype
        L.qfo_compact_rows.argtypes = [ctypes.c_int, ctypes.POINTER(i32p), ctypes.c_int64, u64p,
                                       ctypes.c_int, ctypes.POINTER(i32p)]
        L.qfo_compact_rows.restype = ctypes.c_int64
        L.qfo_parse_text.argtypes = [ctypes.c_char_p, ctypes.c_int64, ctypes.c_int, i32p,
                                     ctypes.POINTER(i32p), ctypes.c_int64, i64p, i64p]
        L.qfo_parse_text.restype = ctypes.c_int
        _lib = L
    return _lib


def _i32ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def _colptrs(cols: Sequence[np.ndarray]):
    arr = (ctypes.POINTER(ctypes.c_int32) * max(1, len(cols)))()
    for i, c in enumerate(cols):
        arr[i] = _i32ptr(c)
    return arr


def _as_cols(cols) -> list:
    return [np.ascontiguousarray(c, dtype=np.int32) for c in cols]


class _TableHandle:
    """Keeps the numpy columns alive while C holds pointers into them."""

    def __init__(self, cols):
        self.cols = _as_cols(cols)
        self.ptrs = _colptrs(self.cols)
        n = len(self.cols[0]) if self.cols else 0
        self.struct = _Table(len(self.cols), n, self.ptrs)


def _literal_struct(lit) -> _Literal:
    relation, vars_, join_pos = lit
    s = _Literal()
    s.relation = relation
    s.num_args = len(vars_)
    s.join_pos = join_pos
    for i in range(MAX_ARITY):
        s.vars[i] = vars_[i] if i < len(vars_) else -1
    return s


def radix_partition(values: np.ndarray, bits: int):
    """Returns (tuples[n,2] int32 (value, tuple_id), offsets[2^bits+1] int64)."""
    values = np.ascontiguousarray(values, dtype=np.int32)
    n = len(values)
    out = np.empty((max(n, 1), 2), dtype=np.int32)
    offsets = np.empty((1 << bits) + 1, dtype=np.int64)
    lib().qfo_radix_partition(_i32ptr(values), n, bits, _i32ptr(out),
                              offsets.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    return out[:n], offsets


def build_partition_hash_table(part_tuples: np.ndarray, bits: int):
    """FoilHashTable over one partition: (buckets, next, mask)."""
    part_tuples = np.ascontiguousarray(part_tuples, dtype=np.int32)
    n = len(part_tuples)
    nb = lib().qfo_num_buckets(n)
    buckets = np.empty(nb, dtype=np.int32)
    nxt = np.empty(n, dtype=np.int32)
    mask = lib().qfo_build_partition_hash_table(_i32ptr(part_tuples), n, bits,
                                                _i32ptr(buckets), _i32ptr(nxt))
    return buckets, nxt, mask


def build_table_hash_table(keys):
    keys = _as_cols(keys)
    n = len(keys[0])
    nb = lib().qfo_num_buckets(n)
    buckets = np.empty(nb, dtype=np.int32)
    nxt = np.empty(max(n, 1), dtype=np.int32)
    mask = lib().qfo_build_table_hash_table(_colptrs(keys), len(keys), n,
                                            _i32ptr(buckets), _i32ptr(nxt))
    return buckets, nxt[:n], mask


class Oracle:
    """Holds a relation-partition cache across evaluations, like the
    reference's per-predicate TableView (partitions persist for the run)."""

    def __init__(self, relations):
        self._rels = [_TableHandle(r) for r in relations]
        self._rel_structs = (_Table * max(1, len(self._rels)))(*[h.struct for h in self._rels])
        self._cache = lib().qfo_relcache_create()

    def close(self):
        if self._cache:
            lib().qfo_relcache_destroy(self._cache)
            self._cache = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def evaluate(self, binding_columns, num_positive: int, literals, bits: int = 5,
                 nthreads: int = 1) -> np.ndarray:
        """Counts [n_literals, 4] int64: covered_pos, covered_neg, binding_pos,
        binding_neg.  ``literals`` is a list of (relation, vars, join_pos)."""
        b = _TableHandle(binding_columns)
        lits = (_Literal * max(1, len(literals)))(*[_literal_struct(l) for l in literals])
        counts = np.zeros((max(1, len(literals)), 4), dtype=np.int64)
        rc = lib().qfo_evaluate(self._cache, self._rel_structs, len(self._rels),
                                ctypes.byref(b.struct), num_positive, lits, len(literals),
                                bits, nthreads,
                                counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
        if rc != 0:
            raise ValueError(f"oracle rejected the literal list (status {rc})")
        return counts[:len(literals)]


def evaluate(relations, binding_columns, num_positive, literals, bits=5, nthreads=1):
    o = Oracle(relations)
    try:
        return o.evaluate(binding_columns, num_positive, literals, bits, nthreads)
    finally:
        o.close()


def _semijoin(name, probe_keys, build_keys, nbits_rows):
    probe_keys = _as_cols(probe_keys)
    build_keys = _as_cols(build_keys)
    out = np.zeros(max(1, (nbits_rows + 63) // 64), dtype=np.uint64)
    ones = getattr(lib(), name)(_colptrs(probe_keys), len(probe_keys[0]), _colptrs(build_keys),
                                len(build_keys[0]), len(probe_keys),
                                out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
    return out[:(nbits_rows + 63) // 64], int(ones)


def left_semijoin(probe_keys, build_keys):
    """Bit per probe row (uint64 blocks), number of set bits."""
    return _semijoin("qfo_left_semijoin", probe_keys, build_keys, len(probe_keys[0]))


def right_semijoin(probe_keys, build_keys):
    """Bit per build row (uint64 blocks), number of set bits."""
    return _semijoin("qfo_right_semijoin", probe_keys, build_keys, len(build_keys[0]))


def extend_bindings(binding_columns, num_positive, relation_columns, literal,
                    num_out_positive, num_out_negative):
    """Label-aware binding-set extension; returns the list of new columns."""
    b = _TableHandle(binding_columns)
    r = _TableHandle(relation_columns)
    _, vars_, _ = literal
    n_unbound = sum(1 for v in vars_ if v < 0)
    total = num_out_positive + num_out_negative
    outs = [np.zeros(max(total, 1), dtype=np.int32) for _ in range(len(b.cols) + n_unbound)]
    lit = _literal_struct(literal)
    rc = lib().qfo_extend_bindings(ctypes.byref(b.struct), num_positive, ctypes.byref(r.struct),
                                   ctypes.byref(lit), num_out_positive, num_out_negative,
                                   _colptrs(outs))
    if rc != 0:
        raise ValueError(f"extension produced row counts different from the given ones ({rc})")
    return [o[:total] for o in outs]


def coverage(binding_columns, num_positive, relation_columns, literal, num_target_columns,
             uncovered_positive, negative=None, compat=False):
    """Covered counts of a literal appended to the building clause and the
    uncovered positives' bits; returns ((covered positives, covered
    negatives), uint64 bit blocks).  compat: the reference's own procedure
    with its chunk-relative projection tables (qfo_coverage_compat) instead
    of set membership."""
    b = _TableHandle(binding_columns)
    r = _TableHandle(relation_columns)
    u = _TableHandle(uncovered_positive)
    ng = _TableHandle(negative) if negative is not None else None
    nu = len(u.cols[0]) if u.cols else 0
    bits = np.zeros(max(1, (nu + 63) // 64), dtype=np.uint64)
    counts = np.zeros(2, dtype=np.int64)
    lit = _literal_struct(literal)
    fn = lib().qfo_coverage_compat if compat else lib().qfo_coverage
    rc = fn(ctypes.byref(b.struct), num_positive, ctypes.byref(r.struct),
                            ctypes.byref(lit), num_target_columns, ctypes.byref(u.struct),
                            ctypes.byref(ng.struct) if ng is not None else None,
                            bits.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                            counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    if rc != 0:
        raise ValueError(f"invalid literal for a coverage ({rc})")
    return (int(counts[0]), int(counts[1])), bits[:(nu + 63) // 64]


def compact_rows(columns, bits, keep_set=False):
    """Rows whose bit is clear (set with keep_set), in order."""
    cols = _as_cols(columns)
    n = len(cols[0]) if cols else 0
    outs = [np.zeros(max(1, n), dtype=np.int32) for _ in cols]
    bits = np.ascontiguousarray(bits, dtype=np.uint64)
    if len(bits) < (n + 63) // 64:
        raise ValueError("fewer bit blocks than rows")
    if len(bits) == 0:
        bits = np.zeros(1, dtype=np.uint64)
    m = lib().qfo_compact_rows(len(cols), _colptrs(cols), n,
                               bits.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                               1 if keep_set else 0, _colptrs(outs))
    return [o[:m] for o in outs]


def run_test(relations, clauses, test_columns):
    """QuickFoilTestRunner::RunTest (learner/QuickFoilTestRunner.cpp:128-161)
    composed from the restatements above: per clause the full test table is
    extended by every body literal but the last (CreateBindingTable as the
    positive side of the label-aware extension, sized by the evaluation's
    binding count), then the last literal's coverage removes the test rows it
    covers from those still uncovered.  clauses: lists of (relation, vars)
    with vars naming binding columns (-1 new).  Returns the uncovered rows."""
    test = _as_cols(test_columns)
    k = len(test)
    left = [c.copy() for c in test]
    for body in clauses:
        if len(left[0]) == 0:
            break
        B, empty = [c for c in test], len(test[0]) == 0
        for rel, vars_ in body[:-1]:
            lit = (rel, tuple(vars_), next(i for i, v in enumerate(vars_) if v >= 0))
            npos = int(evaluate(relations, B, len(B[0]), [lit])[0][2])
            if npos == 0:
                empty = True
                break
            B = extend_bindings(B, len(B[0]), relations[rel], lit, npos, 0)
        if empty:
            continue
        rel, vars_ = body[-1]
        lit = (rel, tuple(vars_), next(i for i, v in enumerate(vars_) if v >= 0))
        (cp, _), bits = coverage(B, len(B[0]), relations[rel], lit, k, left)
        if cp:
            left = compact_rows(left, bits)
    return left


class TextError(ValueError):
    """A line the loader rejects: .line (1-based) and .code (2 field count,
    3 no digits, 4 out of range)."""

    def __init__(self, code, line):
        super().__init__(f"line {line}: error {code}")
        self.code, self.line = code, line


def parse_text(text: bytes, num_args: int, skipped=None):
    """LoadData restated: the kept argument columns (int32) of the text."""
    cap = text.count(b"\n") + 1
    skip = np.array([int(bool(x)) for x in (skipped or [0] * num_args)], dtype=np.int32)
    kept = int(num_args - skip.sum())
    outs = [np.zeros(cap, dtype=np.int32) for _ in range(max(kept, 1))]
    rows, err = ctypes.c_int64(), ctypes.c_int64()
    rc = lib().qfo_parse_text(text, len(text), num_args, _i32ptr(skip), _colptrs(outs), cap,
                              ctypes.byref(rows), ctypes.byref(err))
    if rc != 0:
        raise TextError(rc, err.value)
    return [o[:rows.value] for o in outs[:kept]]


def build_hash_table_after_semijoin(keys, bits, chunk_rows: int, num_build_tuples: int):
    """BuildHashTableAfterSemiJoin restated (qf_oracle.c): (buckets, next,
    mask) for `keys` cut into chunk_rows-row chunks (<= 0: one chunk) with
    semi-join bits (uint64 blocks); next is 0 at positions never inserted."""
    keys = _as_cols(keys)
    n = len(keys[0])
    bits = np.ascontiguousarray(bits, dtype=np.uint64)
    nb = int(lib().qfo_num_buckets(num_build_tuples))
    buckets = np.zeros(nb, dtype=np.int32)
    nxt = np.zeros(num_build_tuples, dtype=np.int32)
    mask = lib().qfo_build_hash_table_after_semijoin(
        _colptrs(keys), len(keys), n, bits.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
        chunk_rows, num_build_tuples, buckets.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
        nxt.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    return buckets, nxt, int(mask)


def reachable_next(buckets, nxt):
    """next[] with the entries of positions that no chain reaches set to 0:
    the part of a chained table a probe can observe (the reference leaves
    next[] of never-inserted positions uninitialised)."""
    out = np.zeros_like(nxt)
    seen = np.zeros(len(nxt), dtype=bool)
    for h in buckets:
        pos = int(h) - 1
        while pos >= 0 and not seen[pos]:
            seen[pos] = True
            out[pos] = nxt[pos]
            pos = int(nxt[pos]) - 1
    return out
