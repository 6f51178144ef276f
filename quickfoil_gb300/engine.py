"""Host-side mirror of the reference's operator interface over libqfgpu.

Names follow the reference (jbalint/quickfoil):

* ``Literal``             -- FoilLiteral (schema/FoilLiteral.hpp:21-164)
* ``CandidateLiteralInfo`` -- learner/CandidateLiteralInfo.hpp:15-26
* ``CandidateLiteralEvaluator.Evaluate`` --
  learner/CandidateLiteralEvaluator.hpp:28-31 (same argument meaning, same
  result order: literal groups in iteration order, each group in its order)
* ``Engine.radix_partition`` / ``build_hash_table_on_partitions`` /
  ``build_hash_table_on_table`` / ``left_semijoin`` / ``right_semijoin`` /
  ``extend_bindings`` -- operations/RadixPartition, BuildHashTable,
  LeftSemiJoin, RightSemiJoin, MultiColumnHashJoin.

Every call goes to the CUDA library; errors raise ``QfgError`` (the reference
aborts through CHECK instead).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Dict, Iterable, List, Optional, Sequence, Tuple

import numpy as np

from . import _capi as C


@dataclass(frozen=True)
class Literal:
    """A candidate literal: ``vars[i] >= 0`` binds argument i to clause
    variable ``vars[i]``; -1 is a new (unbound) variable."""
    relation: int
    vars: Tuple[int, ...]
    join_pos: int = -1

    def __post_init__(self):
        if self.join_pos < 0:
            object.__setattr__(self, "join_pos", join_key(self.vars))

    def to_c(self) -> C.QfgLiteral:
        s = C.QfgLiteral()
        s.relation_id = self.relation
        s.num_args = len(self.vars)
        s.join_pos = self.join_pos
        for i in range(C.MAX_ARITY):
            s.vars[i] = self.vars[i] if i < len(self.vars) else -1
        return s

    def as_tuple(self):
        return (self.relation, list(self.vars), self.join_pos)


def join_key(vars_: Sequence[int], var_types: Optional[Sequence[int]] = None) -> int:
    """FoilLiteral::UpdateJoinKey (schema/FoilLiteral.hpp:133-140): the bound
    argument with the largest variable type id, the first one on ties."""
    best = -1
    for pos, v in enumerate(vars_):
        if v < 0:
            continue
        t = var_types[pos] if var_types is not None else 0
        if best == -1 or (var_types is not None and var_types[best] < t):
            best = pos
    if best < 0:
        raise ValueError("a candidate literal needs at least one bound argument")
    return best


def parse_clause(text: str):
    """A learnt clause as the reference prints it (FoilClause::ToString,
    e.g. ``target(0, 1) :-  r1(0), r3(2, 0), r0(2, 1)``, relation ids after
    the ``r``): (head arity, body literals) with each literal's vars naming
    binding columns the way the binding tables grow -- a variable id below
    the column count so far is bound (operations/MultiColumnHashJoin.cpp:
    37-44), any other argument is new (-1) and appends a column."""
    import re
    head, _, body = text.partition(":-")
    arity = len(re.findall(r"-?\d+", head.split("(", 1)[1]))
    lits = []
    ncols = arity
    for name, args in re.findall(r"r(\d+)\(([^)]*)\)", body):
        ids = [int(a) for a in args.split(",")]
        vars_ = tuple(v if v < ncols else -1 for v in ids)
        ncols += sum(1 for v in vars_ if v < 0)
        lits.append(Literal(int(name), vars_))
    return arity, lits


@dataclass
class CandidateLiteralInfo:
    literal: Literal
    num_covered_positive: int = 0
    num_covered_negative: int = 0
    num_binding_positive: int = 0
    num_binding_negative: int = 0

    def counts(self):
        return (self.num_covered_positive, self.num_covered_negative,
                self.num_binding_positive, self.num_binding_negative)


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _column_ptrs(columns):
    """Returns (pointer list, flag, keepalive) for numpy (host) or torch
    (device if CUDA, host otherwise) int32 columns."""
    keep = []
    ptrs = []
    flag = C.QFG_HOST
    for col in columns:
        if _is_torch(col):
            import torch
            if col.dtype != torch.int32:
                raise TypeError("columns must be int32")
            col = col.contiguous()
            if col.is_cuda:
                flag = C.QFG_DEVICE_BORROW
            keep.append(col)
            ptrs.append(col.data_ptr())
        else:
            a = np.ascontiguousarray(col, dtype=np.int32)
            keep.append(a)
            ptrs.append(a.ctypes.data)
    kinds = {(_is_torch(c) and c.is_cuda) for c in keep}
    if len(kinds) > 1:
        raise ValueError("columns must all be on the host or all on the device")
    return ptrs, flag, keep


class BindingSet:
    """A device-resident binding set (positives first)."""

    def __init__(self, engine: "Engine", handle, num_columns, num_positive, num_negative, keep=None):
        self.engine = engine
        self.handle = handle
        self.num_columns = num_columns
        self.num_positive = num_positive
        self.num_negative = num_negative
        self._keep = keep

    @property
    def num_tuples(self):
        return self.num_positive + self.num_negative

    def download(self) -> List[np.ndarray]:
        n = self.num_tuples
        outs = [np.empty(max(n, 1), dtype=np.int32) for _ in range(self.num_columns)]
        C.check(self.engine.lib.qfg_bindings_download(
            self.engine.ctx, self.handle, C.ptr_array([o.ctypes.data for o in outs])),
            self.engine.ctx, "qfg_bindings_download")
        return [o[:n] for o in outs]

    def column_ptr(self, c: int) -> int:
        p = ctypes.c_void_p()
        C.check(self.engine.lib.qfg_bindings_column(self.handle, c, ctypes.byref(p)),
                None, "qfg_bindings_column")
        return p.value or 0

    def close(self):
        if self.handle:
            self.engine.lib.qfg_bindings_destroy(self.engine.ctx, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Engine:
    """One GPU context (qfg_ctx): relations, binding sets, evaluation."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self.lib = C.load()
        ctx = ctypes.c_void_p()
        C.check(self.lib.qfg_ctx_create(device, hbm_budget, ctypes.byref(ctx)), None,
                "qfg_ctx_create")
        self.ctx = ctx
        self.device = device
        self._relations = {}

    def close(self):
        if self.ctx:
            self.lib.qfg_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- configuration ------------------------------------------------------
    def set_option(self, option: int, value: int):
        C.check(self.lib.qfg_ctx_set_option(self.ctx, option, value), self.ctx, "set_option")

    def set_stream(self, stream_ptr: int):
        C.check(self.lib.qfg_ctx_set_stream(self.ctx, stream_ptr), self.ctx, "set_stream")

    def synchronize(self):
        C.check(self.lib.qfg_ctx_synchronize(self.ctx), self.ctx, "synchronize")

    def memory(self):
        used, budget = ctypes.c_int64(), ctypes.c_int64()
        C.check(self.lib.qfg_ctx_memory(self.ctx, ctypes.byref(used), ctypes.byref(budget)),
                self.ctx, "memory")
        return used.value, budget.value

    def stage_times(self, reset: bool = True):
        """{stage: (milliseconds, calls)} accumulated under QFG_OPT_STAGE_TIMING."""
        ms = (ctypes.c_double * len(C.STAGES))()
        calls = (ctypes.c_int64 * len(C.STAGES))()
        C.check(self.lib.qfg_ctx_stage_times(self.ctx, ms, calls, int(reset)), self.ctx,
                "stage_times")
        return {name: (ms[i], calls[i]) for i, name in enumerate(C.STAGES)}

    def kernel_launches(self) -> int:
        n = ctypes.c_int64()
        C.check(self.lib.qfg_ctx_kernel_launches(self.ctx, ctypes.byref(n)), self.ctx, "launches")
        return n.value

    # -- data ----------------------------------------------------------------
    def register_relation(self, relation_id: int, columns) -> None:
        ptrs, flag, keep = _column_ptrs(columns)
        n = len(keep[0]) if keep else 0
        C.check(self.lib.qfg_relation_register(self.ctx, relation_id, len(ptrs),
                                                C.ptr_array(ptrs), n, flag),
                self.ctx, "qfg_relation_register")
        self._relations[relation_id] = keep if flag == C.QFG_DEVICE_BORROW else None

    def release_relation(self, relation_id: int) -> None:
        C.check(self.lib.qfg_relation_release(self.ctx, relation_id), self.ctx,
                "qfg_relation_release")
        self._relations.pop(relation_id, None)

    def bindings(self, columns, num_positive: int, num_negative: Optional[int] = None) -> BindingSet:
        ptrs, flag, keep = _column_ptrs(columns)
        n = len(keep[0]) if keep else 0
        if num_negative is None:
            num_negative = n - num_positive
        h = ctypes.c_void_p()
        C.check(self.lib.qfg_bindings_create(self.ctx, len(ptrs), C.ptr_array(ptrs), num_positive,
                                              num_negative, flag, ctypes.byref(h)),
                self.ctx, "qfg_bindings_create")
        return BindingSet(self, h, len(ptrs), num_positive, num_negative,
                          keep if flag == C.QFG_DEVICE_BORROW else None)

    def bindings_split(self, positive_columns, negative_columns) -> BindingSet:
        pp, f1, k1 = _column_ptrs(positive_columns)
        nn, f2, k2 = _column_ptrs(negative_columns)
        if f1 != f2:
            raise ValueError("positive and negative blocks must live in the same memory")
        flag = C.QFG_DEVICE_COPY if f1 == C.QFG_DEVICE_BORROW else C.QFG_HOST
        h = ctypes.c_void_p()
        npos, nneg = len(k1[0]), len(k2[0])
        C.check(self.lib.qfg_bindings_create_split(self.ctx, len(pp), C.ptr_array(pp), npos,
                                                    C.ptr_array(nn), nneg, flag, ctypes.byref(h)),
                self.ctx, "qfg_bindings_create_split")
        return BindingSet(self, h, len(pp), npos, nneg)

    # -- evaluation ----------------------------------------------------------
    def _evaluate(self, fn, bindings: BindingSet, literals: Sequence[Literal], *extra) -> np.ndarray:
        lits = (C.QfgLiteral * max(1, len(literals)))(*[l.to_c() for l in literals])
        counts = np.zeros((max(1, len(literals)), 4), dtype=np.int64)
        args = [self.ctx, bindings.handle, *extra, len(literals), lits,
                counts.ctypes.data_as(C.c_i64p), C.QFG_COUNTS_HOST]
        C.check(fn(*args), self.ctx, fn.__name__)
        return counts[:len(literals)]

    def evaluate_step(self, bindings: BindingSet, literals: Sequence[Literal]) -> np.ndarray:
        """All literals of a refinement step, batched: counts [n, 4] int64
        (covered_pos, covered_neg, binding_pos, binding_neg)."""
        return self._evaluate(self.lib.qfg_evaluate_step, bindings, literals)

    def evaluate_per_literal(self, bindings: BindingSet, literals: Sequence[Literal]) -> np.ndarray:
        """The plain per-literal GPU path, same counts."""
        return self._evaluate(self.lib.qfg_evaluate_per_literal, bindings, literals)

    def evaluate_group(self, bindings: BindingSet, clause_join_key_id: int,
                       literals: Sequence[Literal]) -> np.ndarray:
        return self._evaluate(self.lib.qfg_evaluate_group, bindings, literals, clause_join_key_id)

    def step_traffic(self, bindings: BindingSet, literals: Sequence[Literal]):
        """{stage: algorithmic bytes} of a batched step over ``literals``."""
        lits = (C.QfgLiteral * max(1, len(literals)))(*[l.to_c() for l in literals])
        out = (ctypes.c_int64 * len(C.STAGES))()
        C.check(self.lib.qfg_step_traffic(self.ctx, bindings.handle, len(literals), lits, out),
                self.ctx, "qfg_step_traffic")
        return {name: out[i] for i, name in enumerate(C.STAGES)}

    def evaluate_step_device(self, bindings: BindingSet, literals_c, n: int, counts_dev_ptr: int):
        """Asynchronous batched evaluation into device memory (``literals_c``
        is a ctypes QfgLiteral array, ``counts_dev_ptr`` a device pointer to
        4*n int64)."""
        C.check(self.lib.qfg_evaluate_step(self.ctx, bindings.handle, n, literals_c,
                                           ctypes.cast(counts_dev_ptr, C.c_i64p),
                                           C.QFG_COUNTS_DEVICE),
                self.ctx, "qfg_evaluate_step")

    def autotune_step(self, bindings: BindingSet, literals: Sequence[Literal]):
        """Times the batched step at a few partition settings and records the
        fastest for the binding set's size class; returns (partition bits,
        pass-1 bits (0 = one pass), ms).  Used by later steps under
        QFG_OPT_AUTOTUNE = 1."""
        lits = (C.QfgLiteral * max(1, len(literals)))(*[l.to_c() for l in literals])
        bits, cbits, ms = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_double()
        C.check(self.lib.qfg_autotune_step(self.ctx, bindings.handle, len(literals), lits,
                                           ctypes.byref(bits), ctypes.byref(cbits), ctypes.byref(ms)),
                self.ctx, "qfg_autotune_step")
        return bits.value, cbits.value, ms.value

    def autotune_choice(self, num_rows: int):
        """The autotuner's setting for binding sets of num_rows rows:
        {"mode": "tiled" | "streamed" | None, "bits", "pass1_bits", "bias"}."""
        v = [ctypes.c_int32() for _ in range(4)]
        C.check(self.lib.qfg_autotune_choice(self.ctx, num_rows, *[ctypes.byref(x) for x in v]),
                self.ctx, "qfg_autotune_choice")
        mode = {1: "tiled", 2: "streamed"}.get(v[0].value)
        return {"mode": mode, "bits": v[1].value, "pass1_bits": v[2].value, "bias": v[3].value}

    def step_scratch_bytes(self, bindings: BindingSet, literals: Sequence[Literal]) -> int:
        """Device scratch a batched step of these literals needs."""
        lits = (C.QfgLiteral * max(1, len(literals)))(*[l.to_c() for l in literals])
        out = ctypes.c_int64()
        C.check(self.lib.qfg_step_scratch_bytes(self.ctx, bindings.handle, len(literals), lits,
                                                ctypes.byref(out)),
                self.ctx, "qfg_step_scratch_bytes")
        return out.value

    def step_graph(self, bindings: BindingSet, literals: Sequence[Literal],
                   counts_dev_ptr: int) -> "StepGraph":
        """A batched step captured into a CUDA graph; each ``launch()`` writes
        the counts of the binding set's current contents to ``counts_dev_ptr``
        (device, 4*n int64)."""
        return StepGraph(self, bindings, literals, counts_dev_ptr)

    def server(self, slots: int = 4, hbm_budget: int = 0, depth: int = 1) -> "StepServer":
        """A serving loop over concurrent requests of many rule searches;
        ``depth`` requests a slot holds at once (queued on its stream)."""
        self.set_option(C.QFG_OPT_SERVER_DEPTH, depth)
        return StepServer(self, slots, hbm_budget)

    # -- API-kept operators (torch CUDA tensors) ------------------------------
    def radix_partition(self, values, bits: int):
        """RadixPartition: returns (tuples [n, 2] int32, offsets [2^bits+1] int64)."""
        import torch
        n = values.numel()
        tuples = torch.empty((max(n, 1), 2), dtype=torch.int32, device=values.device)
        offsets = torch.empty((1 << bits) + 1, dtype=torch.int64, device=values.device)
        C.check(self.lib.qfg_radix_partition(self.ctx, values.data_ptr() if n else None, n, bits,
                                             tuples.data_ptr(), offsets.data_ptr()),
                self.ctx, "qfg_radix_partition")
        return tuples[:n], offsets

    def build_hash_table_on_partitions(self, tuples, offsets, bits: int):
        """BuildHashTableOnPartitions: (buckets, bucket_offsets, masks (uint32
        bit patterns in an int32 tensor), next)."""
        import torch
        n = tuples.shape[0]
        dev = tuples.device
        buckets = torch.empty(max(1, 2 * n + (1 << bits)), dtype=torch.int32, device=dev)
        bucket_offsets = torch.empty((1 << bits) + 1, dtype=torch.int64, device=dev)
        masks = torch.empty(1 << bits, dtype=torch.int32, device=dev)
        nxt = torch.empty(max(1, n), dtype=torch.int32, device=dev)
        C.check(self.lib.qfg_build_hash_table_on_partitions(
            self.ctx, tuples.data_ptr(), offsets.data_ptr(), n, bits, buckets.data_ptr(),
            bucket_offsets.data_ptr(), masks.data_ptr(), nxt.data_ptr()),
            self.ctx, "qfg_build_hash_table_on_partitions")
        return buckets, bucket_offsets, masks, nxt[:n]

    def build_hash_table_on_table(self, keys):
        """BuildHashTableOnTable: (buckets, next, mask)."""
        import torch
        n = keys[0].numel()
        nb = 1
        while nb < n:
            nb <<= 1
        buckets = torch.empty(nb, dtype=torch.int32, device=keys[0].device)
        nxt = torch.empty(n, dtype=torch.int32, device=keys[0].device)
        mask = ctypes.c_uint32()
        C.check(self.lib.qfg_build_hash_table_on_table(
            self.ctx, C.ptr_array([k.data_ptr() for k in keys]), len(keys), n, buckets.data_ptr(),
            nxt.data_ptr(), ctypes.byref(mask)), self.ctx, "qfg_build_hash_table_on_table")
        return buckets, nxt, mask.value

    def build_hash_table_after_semijoin(self, keys, bits, chunk_rows: int, num_build_tuples: int):
        """BuildHashTableAfterSemiJoin over the semi-join's projected device
        columns `keys` and its bit blocks `bits` (int64/uint64 device
        tensor), cut into chunk_rows-row chunks (<= 0: one chunk): (buckets,
        next, mask)."""
        import torch
        n = keys[0].numel()
        nb = 1
        while nb < num_build_tuples:
            nb <<= 1
        buckets = torch.empty(nb, dtype=torch.int32, device=keys[0].device)
        nxt = torch.empty(num_build_tuples, dtype=torch.int32, device=keys[0].device)
        mask = ctypes.c_uint32()
        C.check(self.lib.qfg_build_hash_table_after_semijoin(
            self.ctx, C.ptr_array([k.data_ptr() for k in keys]), len(keys), n, bits.data_ptr(),
            chunk_rows, num_build_tuples, buckets.data_ptr(), nxt.data_ptr(), ctypes.byref(mask)),
            self.ctx, "qfg_build_hash_table_after_semijoin")
        return buckets, nxt, mask.value

    def _semijoin(self, fn, probe_keys, build_keys, nrows):
        import torch
        bits = torch.empty(max(1, (nrows + 63) // 64), dtype=torch.int64, device=probe_keys[0].device)
        ones = ctypes.c_int64()
        C.check(fn(self.ctx, C.ptr_array([k.data_ptr() for k in probe_keys]), probe_keys[0].numel(),
                   C.ptr_array([k.data_ptr() for k in build_keys]), build_keys[0].numel(),
                   len(probe_keys), bits.data_ptr(), ctypes.byref(ones)), self.ctx, fn.__name__)
        return bits[:(nrows + 63) // 64], ones.value

    def left_semijoin(self, probe_keys, build_keys):
        """LeftSemiJoin: (bit blocks over probe rows, number of ones)."""
        return self._semijoin(self.lib.qfg_left_semijoin, probe_keys, build_keys,
                              probe_keys[0].numel())

    def right_semijoin(self, probe_keys, build_keys):
        """RightSemiJoin: (bit blocks over build rows, number of ones)."""
        return self._semijoin(self.lib.qfg_right_semijoin, probe_keys, build_keys,
                              build_keys[0].numel())

    def extend_bindings(self, bindings: BindingSet, literal: Literal, num_out_positive: int,
                        num_out_negative: int) -> BindingSet:
        """CreateLabelAwareBindingTables: the binding set extended by
        ``literal`` (device-resident)."""
        h = ctypes.c_void_p()
        lit = literal.to_c()
        C.check(self.lib.qfg_extend_bindings(self.ctx, bindings.handle, ctypes.byref(lit),
                                             num_out_positive, num_out_negative, ctypes.byref(h)),
                self.ctx, "qfg_extend_bindings")
        ncols = bindings.num_columns + sum(1 for v in literal.vars if v < 0)
        return BindingSet(self, h, ncols, num_out_positive, num_out_negative)


    def coverage(self, bindings: BindingSet, literal: Literal, num_target_columns: int,
                 uncovered_positive, negative=None, positive_bits: bool = True):
        """ComputeCoverageOnUncoveredData / ComputeCoveredPositives of
        ``literal`` appended to the clause whose binding set is ``bindings``.
        ``uncovered_positive`` and ``negative`` are lists of CUDA int32
        tensors (``negative`` None: positives only).  Returns ((covered
        positives, covered negatives), bit blocks over the uncovered positives
        as an int64 CUDA tensor, or None)."""
        import torch
        nu = uncovered_positive[0].numel() if uncovered_positive else 0
        nn = negative[0].numel() if negative else 0
        bits = None
        if positive_bits:
            bits = torch.empty(max(1, (nu + 63) // 64), dtype=torch.int64, device="cuda")
        counts = (ctypes.c_int64 * 2)()
        lit = literal.to_c()
        up = C.ptr_array([t.data_ptr() for t in uncovered_positive]) if nu else None
        npt = C.ptr_array([t.data_ptr() for t in negative]) if nn else None
        C.check(self.lib.qfg_coverage(self.ctx, bindings.handle, ctypes.byref(lit),
                                      num_target_columns, up, nu, npt, nn,
                                      bits.data_ptr() if bits is not None else None, counts),
                self.ctx, "qfg_coverage")
        if bits is not None:
            bits = bits[:(nu + 63) // 64]
        return (counts[0], counts[1]), bits

    def parse_text(self, text, num_arguments: int, skipped: Optional[Sequence[bool]] = None):
        """qfg_parse_text (LoadData): '|'-delimited facts -> CUDA int32
        columns of the kept arguments.  ``text`` is bytes (host) or a CUDA
        uint8 tensor.  A bad line raises QfgError naming it."""
        import torch
        on_dev = _is_torch(text)
        n = text.numel() if on_dev else len(text)
        cap = (int((text == 10).sum().item()) if on_dev else text.count(b"\n")) + 1
        skip = (ctypes.c_int32 * num_arguments)(*[int(bool(x)) for x in (skipped or [0] * num_arguments)])
        kept = num_arguments - sum(1 for x in (skipped or []) if x)
        outs = [torch.empty(max(1, cap), dtype=torch.int32, device="cuda") for _ in range(kept)]
        rows, err = ctypes.c_int64(), ctypes.c_int64()
        ptr = ctypes.cast(ctypes.c_void_p(text.data_ptr()), ctypes.c_char_p) if on_dev else text
        C.check(self.lib.qfg_parse_text(self.ctx, ptr, n, C.QFG_DEVICE_BORROW if on_dev else C.QFG_HOST,
                                        num_arguments, skip,
                                        C.ptr_array([o.data_ptr() for o in outs]), cap,
                                        ctypes.byref(rows), ctypes.byref(err)),
                self.ctx, "qfg_parse_text")
        return [o[:rows.value] for o in outs]

    def register_relation_text(self, relation_id: int, text: bytes, num_arguments: int,
                               skipped: Optional[Sequence[bool]] = None) -> int:
        """qfg_relation_register_text: a relation straight from its text;
        returns the fact count."""
        skip = (ctypes.c_int32 * num_arguments)(*[int(bool(x)) for x in (skipped or [0] * num_arguments)])
        rows, err = ctypes.c_int64(), ctypes.c_int64()
        C.check(self.lib.qfg_relation_register_text(self.ctx, relation_id, text, len(text), C.QFG_HOST,
                                                    num_arguments, skip, ctypes.byref(rows),
                                                    ctypes.byref(err)),
                self.ctx, "qfg_relation_register_text")
        return rows.value

    def examples(self, columns) -> "ExampleTable":
        """qfg_examples_create: an example table (CUDA int32 columns, kept
        unchanged while the handle lives) prepared for many coverage calls."""
        return ExampleTable(self, columns)

    def coverage_examples(self, bindings: BindingSet, literal: Literal,
                          uncovered_positive: "ExampleTable",
                          negative: Optional["ExampleTable"] = None, positive_bits: bool = True):
        """qfg_coverage_examples: coverage() on prepared example tables."""
        import torch
        nu = uncovered_positive.num_rows
        bits = None
        if positive_bits:
            bits = torch.empty(max(1, (nu + 63) // 64), dtype=torch.int64, device="cuda")
        counts = (ctypes.c_int64 * 2)()
        lit = literal.to_c()
        C.check(self.lib.qfg_coverage_examples(
            self.ctx, bindings.handle, ctypes.byref(lit), uncovered_positive.handle,
            negative.handle if negative is not None else None,
            bits.data_ptr() if bits is not None else None, counts),
            self.ctx, "qfg_coverage_examples")
        if bits is not None:
            bits = bits[:(nu + 63) // 64]
        return (counts[0], counts[1]), bits

    def run_test(self, clauses: Sequence[Sequence[Literal]], test_columns, rows: bool = False):
        """qfg_run_test (QuickFoilTestRunner::RunTest): the test rows (CUDA
        int32 target columns) no clause covers.  Returns the count, or with
        ``rows`` (count, the rows as CUDA columns)."""
        import torch
        n = test_columns[0].numel() if test_columns else 0
        lens = (ctypes.c_int32 * max(1, len(clauses)))(*[len(c) for c in clauses])
        flat = [l.to_c() for c in clauses for l in c]
        lits = (C.QfgLiteral * max(1, len(flat)))(*flat)
        outs = [torch.empty(max(1, n), dtype=torch.int32, device="cuda") for _ in test_columns] \
            if rows else None
        left = ctypes.c_int64()
        C.check(self.lib.qfg_run_test(
            self.ctx, len(clauses), lens, lits, len(test_columns),
            C.ptr_array([t.data_ptr() for t in test_columns]), n, ctypes.byref(left),
            C.ptr_array([t.data_ptr() for t in outs]) if outs is not None else None),
            self.ctx, "qfg_run_test")
        if not rows:
            return left.value
        return left.value, [o[:left.value] for o in outs]

    def compact_rows(self, columns, bits, keep_set: bool = False, capacity: Optional[int] = None):
        """The uncovered-example compaction: rows of the CUDA int32 ``columns``
        whose bit in ``bits`` is clear (set with ``keep_set``), in order."""
        import torch
        n = columns[0].numel() if columns else 0
        cap = n if capacity is None else capacity
        outs = [torch.empty(max(1, cap), dtype=torch.int32, device="cuda") for _ in columns]
        kept = ctypes.c_int64()
        C.check(self.lib.qfg_compact_rows(
            self.ctx, len(columns), C.ptr_array([t.data_ptr() for t in columns]), n,
            bits.data_ptr() if bits is not None else None, 1 if keep_set else 0,
            C.ptr_array([t.data_ptr() for t in outs]), cap, ctypes.byref(kept)),
            self.ctx, "qfg_compact_rows")
        return [o[:kept.value] for o in outs]


class ExampleTable:
    """qfg_examples_*: example columns with their key set, kept for many
    coverage calls."""

    def __init__(self, engine: Engine, columns):
        self.engine = engine
        self._keep = list(columns)
        self.num_columns = len(self._keep)
        self.num_rows = self._keep[0].numel() if self._keep else 0
        h = C.c_vp()
        C.check(engine.lib.qfg_examples_create(
            engine.ctx, self.num_columns, C.ptr_array([t.data_ptr() for t in self._keep]),
            self.num_rows, ctypes.byref(h)), engine.ctx, "qfg_examples_create")
        self.handle = h

    def close(self):
        if self.handle is not None:
            self.engine.lib.qfg_examples_destroy(self.engine.ctx, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class StepGraph:
    """qfg_step_graph_*: one refinement step replayed with a single launch."""

    def __init__(self, engine: Engine, bindings: BindingSet, literals: Sequence[Literal],
                 counts_dev_ptr: int):
        self.engine = engine
        self._keep = bindings
        self.num_literals = len(literals)
        self._lits = (C.QfgLiteral * max(1, len(literals)))(*[l.to_c() for l in literals])
        h = C.c_vp()
        C.check(engine.lib.qfg_step_graph_create(engine.ctx, bindings.handle, len(literals),
                                                 self._lits, counts_dev_ptr, ctypes.byref(h)),
                engine.ctx, "qfg_step_graph_create")
        self.handle = h

    def launch(self):
        C.check(self.engine.lib.qfg_step_graph_launch(self.engine.ctx, self.handle),
                self.engine.ctx, "qfg_step_graph_launch")

    def close(self):
        if self.handle:
            self.engine.lib.qfg_step_graph_destroy(self.engine.ctx, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class StepServer:
    """qfg_server_*: requests (binding set + candidate literals) of many
    concurrent rule searches, admitted under an HBM budget and run on
    separate streams; counts land in host arrays."""

    def __init__(self, engine: Engine, slots: int, hbm_budget: int):
        self.engine = engine
        h = C.c_vp()
        C.check(engine.lib.qfg_server_create(engine.ctx, slots, hbm_budget, ctypes.byref(h)),
                engine.ctx, "qfg_server_create")
        self.handle = h
        self._pending: Dict[int, Tuple[BindingSet, object, np.ndarray]] = {}

    def submit(self, bindings: BindingSet, literals: Sequence[Literal]) -> int:
        lits = (C.QfgLiteral * max(1, len(literals)))(*[l.to_c() for l in literals])
        counts = np.zeros((max(1, len(literals)), 4), dtype=np.int64)
        rid = ctypes.c_int64()
        C.check(self.engine.lib.qfg_server_submit(self.handle, bindings.handle, len(literals), lits,
                                                  counts.ctypes.data_as(C.c_i64p),
                                                  ctypes.byref(rid)),
                self.engine.ctx, "qfg_server_submit")
        self._pending[rid.value] = (bindings, lits, counts[:len(literals)])
        return rid.value

    def poll(self) -> List[int]:
        ids = (ctypes.c_int64 * 256)()
        n = ctypes.c_int32()
        out: List[int] = []
        while True:
            C.check(self.engine.lib.qfg_server_poll(self.handle, ids, 256, ctypes.byref(n)),
                    self.engine.ctx, "qfg_server_poll")
            out.extend(ids[i] for i in range(n.value))
            if n.value < 256:
                return out

    def result(self, request_id: int) -> np.ndarray:
        """Waits for the request; its counts [n, 4]."""
        C.check(self.engine.lib.qfg_server_wait(self.handle, request_id), self.engine.ctx,
                "qfg_server_wait")
        return self._pending[request_id][2]

    def drain(self):
        C.check(self.engine.lib.qfg_server_drain(self.handle), self.engine.ctx, "qfg_server_drain")

    def stats(self):
        p50, p99 = ctypes.c_double(), ctypes.c_double()
        done, peak = ctypes.c_int64(), ctypes.c_int64()
        C.check(self.engine.lib.qfg_server_stats(self.handle, ctypes.byref(p50), ctypes.byref(p99),
                                                 ctypes.byref(done), ctypes.byref(peak)),
                self.engine.ctx, "qfg_server_stats")
        return {"p50_ms": p50.value, "p99_ms": p99.value, "completed": done.value,
                "peak_in_flight": peak.value}

    def reset_stats(self):
        C.check(self.engine.lib.qfg_server_reset_stats(self.handle), self.engine.ctx,
                "qfg_server_reset_stats")

    def close(self):
        if self.handle:
            self.engine.lib.qfg_server_destroy(self.handle)
            self.handle = None
            self._pending.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CandidateLiteralEvaluator:
    """learner/CandidateLiteralEvaluator.hpp:23-45 over a device binding set."""

    def __init__(self, engine: Engine, building_bindings: BindingSet):
        self.engine = engine
        self.bindings = building_bindings

    def Evaluate(self, clause_join_key_id: int,
                 literal_groups: Dict[int, Sequence[Literal]]) -> List[CandidateLiteralInfo]:
        """Same result order as the reference (learner/CandidateLiteralEvaluator.cpp:
        281-289): groups in iteration order, literals in group order."""
        ordered: List[Literal] = []
        for _pred, lits in literal_groups.items():
            ordered.extend(lits)
        if not ordered:
            return []
        counts = self.engine.evaluate_group(self.bindings, clause_join_key_id, ordered)
        return [CandidateLiteralInfo(l, *map(int, c)) for l, c in zip(ordered, counts)]
