"""Device-resident replay of the reference learner's compact trace (BASELINE
config 4 at full scale, tests/golden/bongard_kb_trace.npz) through the C ABI.

TEST INFRASTRUCTURE: used by tests/test_gpu_learn_scale.py and by the
learn-loop leg of bench.py as the checker of the GPU learn loop.

The knowledge base is regenerated from its seed (workloads.bongard_kb) and
checked against the fixture's column checksums.  The replay starts from the
target table as the first building clause's binding set and keeps every
binding set on the device:

* EVALUATE: the call's binding set (found by its column checksums) and its
  literals through qfg_evaluate_group (the drop-in for
  CandidateLiteralEvaluator::Evaluate); the counts must equal the
  reference's.
* EXTEND: qfg_extend_bindings on the device-resident input; the output's
  column checksums, computed on the device, must equal the reference's.  The
  output becomes the binding set of later calls; nothing is uploaded from the
  reference.
* SELJ / EXAMPLES / PROBE: one label side of a coverage (QuickFoil::
  ComputeCoverageOnUncoveredData, LiteralSelector::ComputeCoveredPositives):
  the side is found among the device binding sets by its checksums, the
  examples among the device example tables (the target's positives and
  negatives, and every compaction of an earlier probe's examples by its
  coverage bits, qfg_compact_rows, as the learner compacts uncovered
  positives); qfg_coverage gives the covered count and bits, which must equal
  the reference's (count and two sums over the covered positions).

Checksum of a column: sum over rows r of ((uint32)v + 0x9e3779b9) * (2r+1)
modulo 2^64, as oracle/ref_driver.cpp writes it.
"""
from __future__ import annotations

import os
import time

import numpy as np

from quickfoil_gb300 import workloads
from quickfoil_gb300 import _capi as C
from quickfoil_gb300.engine import Literal

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "bongard_kb_trace.npz")
_U64 = 1 << 64


def host_checksum(v) -> int:
    v = np.asarray(v, dtype=np.int32).view(np.uint32).astype(np.uint64) + np.uint64(0x9E3779B9)
    r = np.arange(len(v), dtype=np.uint64) * np.uint64(2) + np.uint64(1)
    return int(np.sum(v * r, dtype=np.uint64))


def device_checksum(torch, col) -> int:
    """The checksum of an int32 device column, computed on the device
    (int64 arithmetic wraps modulo 2^64)."""
    v = (col.to(torch.int64) & 0xFFFFFFFF) + 0x9E3779B9
    r = torch.arange(col.numel(), device=col.device, dtype=torch.int64) * 2 + 1
    return int(torch.sum(v * r).item()) % _U64


def bit_sums(torch, bits, n: int):
    """(set count, sum of e + 1, sum of (e + 1)^2 mod 2^64) over the set
    positions e of n bits in int64 blocks (device)."""
    words = bits.view(torch.int64)
    shifts = torch.arange(64, device=bits.device, dtype=torch.int64)
    flags = ((words.unsqueeze(1) >> shifts) & 1).reshape(-1)[:n].bool()
    e = torch.nonzero(flags).reshape(-1).to(torch.int64) + 1
    s1 = int(torch.sum(e).item()) % _U64 if e.numel() else 0
    s2 = int(torch.sum(e * e).item()) % _U64 if e.numel() else 0
    return int(e.numel()), s1, s2


def load_trace():
    z = np.load(FIXTURE)
    text = bytes(z["trace"]).decode()
    return z, [l.split() for l in text.splitlines() if l]


def _literal(tok):
    rel, nargs, join = int(tok[1]), int(tok[2]), int(tok[3])
    return Literal(rel, tuple(int(v) for v in tok[4:4 + nargs]), join)


def replay(engine, torch, compat: bool = False, log=None):
    """Replays the whole trace; returns a summary (calls of each kind, GPU
    seconds of the calls, the reference's seconds, clauses).  Raises
    AssertionError on the first result that differs from the reference's."""
    z, lines = load_trace()
    seed, pictures, max_positive, max_len = (int(x) for x in z["params"])
    kb = workloads.bongard_kb(seed=seed, pictures=pictures, max_positive=max_positive,
                              max_clause_length=max_len)
    want_rel = [int(x) for x in z["relation_checksums"]]
    got_rel = [host_checksum(c) for r in kb.relations for c in r]
    assert got_rel == want_rel, "the knowledge base does not regenerate"
    assert host_checksum(kb.target_columns[0]) == int(z["target_checksum"][0])
    dev = torch.device("cuda")
    for rid, cols in enumerate(kb.relations):
        engine.register_relation(rid, cols)
    engine.set_option(C.QFG_OPT_COVERAGE_COMPAT, 1 if compat else 0)
    P = kb.num_positive
    target = torch.from_numpy(kb.target_columns[0]).to(dev)
    k = len(kb.target_columns)
    sets = {}      # (P, N, column checksums) -> BindingSet
    examples = {}  # (rows, column checksums) -> [device columns]

    def set_key(b, cols):
        return (b.num_positive, b.num_negative, tuple(device_checksum(torch, c) for c in cols))

    def add_set(b):
        cols = [_column(b, c) for c in range(b.num_columns)]
        sets[set_key(b, cols)] = b

    def _column(b, c):
        n = b.num_positive + b.num_negative
        return torch.as_tensor(np.empty(0), device=dev) if n == 0 else _wrap(b.column_ptr(c), n)

    def _wrap(ptr, n):
        # a view of a device column the engine owns (no copy)
        return torch.as_tensor(_DeviceColumn(ptr, n), device=dev)

    def add_examples(cols):
        n = int(cols[0].numel())
        examples[(n, tuple(device_checksum(torch, c) for c in cols))] = cols

    first = engine.bindings([target], P)
    add_set(first)
    add_examples([target[:P].contiguous()])
    add_examples([target[P:].contiguous()])
    gpu_s = {"evaluate": 0.0, "extend": 0.0, "coverage": 0.0, "compaction": 0.0}
    calls = {"evaluate": 0, "extend": 0, "coverage": 0}
    i = 0
    side = None
    clauses = []

    def timed(kind, fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        gpu_s[kind] += time.perf_counter() - t0
        return out

    def find_set(ncols, p, n, cs):
        key = (p, n, tuple(cs))
        assert key in sets, f"binding set not produced on the device (line {i})"
        return sets[key]

    while i < len(lines):
        tok = lines[i]
        if tok[0] == "EVALUATE":
            j, m = int(tok[1]), int(tok[2])
            _, ncols, p, n = lines[i + 1]
            cs = [int(lines[i + 2 + q][1]) for q in range(int(ncols))]
            b = find_set(int(ncols), int(p), int(n), cs)
            i += 2 + int(ncols)
            lits, want = [], []
            for _ in range(m):
                lits.append(_literal(lines[i]))
                want.append([int(x) for x in lines[i + 1][1:5]])
                i += 2
            got = timed("evaluate", lambda: engine.evaluate_group(b, j, lits))
            assert np.array_equal(got, np.array(want, dtype=np.int64)), f"Evaluate counts (line {i})"
            calls["evaluate"] += 1
        elif tok[0] == "EXTEND":
            npos, nneg = int(tok[1]), int(tok[2])
            _, ncols, p, n = lines[i + 1]
            cs = [int(lines[i + 2 + q][1]) for q in range(int(ncols))]
            b = find_set(int(ncols), int(p), int(n), cs)
            i += 2 + int(ncols)
            lit = _literal(lines[i])
            i += 1
            want_cs = []
            while i < len(lines) and lines[i][0] == "OUTCS":
                want_cs.append(int(lines[i][1]))
                i += 1
            out = timed("extend", lambda: engine.extend_bindings(b, lit, npos, nneg))
            cols = [_column(out, c) for c in range(out.num_columns)]
            got_cs = [device_checksum(torch, c) for c in cols]
            assert got_cs == want_cs, f"extension output differs (line {i})"
            sets[(npos, nneg, tuple(got_cs))] = out
            calls["extend"] += 1
        elif tok[0] == "SELJ":
            rel, nk = int(tok[1]), int(tok[2])
            pairs = [(int(tok[3 + 2 * q]), int(tok[4 + 2 * q])) for q in range(nk)]
            srow = lines[i + 1]
            rows, scs = int(srow[1]), [int(x) for x in srow[2:]]
            side = None
            for (p, n, cs), b in sets.items():
                for s, cnt in ((0, p), (1, n)):
                    if cnt != rows or len(cs) != len(scs) or side is not None:
                        continue
                    off = 0 if s == 0 else p
                    sc = [device_checksum(torch, _column(b, c)[off:off + rows])
                          for c in range(len(cs))]
                    if sc == scs:
                        side = (b, s)
            assert side is not None, f"label side not found on the device (line {i})"
            arity = len(kb.relations[rel])
            vars_ = [-1] * arity
            for bc, arg in pairs:
                vars_[arg] = bc
            lit = Literal(rel, tuple(vars_), pairs[0][1])
            side = side + (lit,)
            i += 2
        elif tok[0] == "EXAMPLES":
            rows, ecs = int(tok[1]), tuple(int(x) for x in tok[2:])
            assert (rows, ecs) in examples, f"example table not produced on the device (line {i})"
            ex = examples[(rows, ecs)]
            probe = lines[i + 1]
            assert probe[0] == "PROBE"
            want = (int(probe[3]), int(probe[4]), int(probe[5]))
            b, s, lit = side
            if s == 0:
                (cp, _), bits = timed("coverage", lambda: engine.coverage(b, lit, k, ex, None))
                got = bit_sums(torch, bits, rows)
                assert got[0] == cp and got == want, f"coverage differs (line {i})"
                # the learner's compaction of these examples by the probe's bits
                left = timed("compaction", lambda: engine.compact_rows(ex, bits))
                add_examples([c.contiguous() for c in left])
            else:
                empty = [torch.empty(0, dtype=torch.int32, device=dev) for _ in range(k)]
                (_, cn), _ = timed("coverage", lambda: engine.coverage(b, lit, k, empty, ex,
                                                                       positive_bits=False))
                assert cn == want[0], f"negative coverage differs (line {i})"
            calls["coverage"] += 1
            i += 2
        elif tok[0] == "CLAUSES":
            i += 1
            while lines[i][0] != "END":
                clauses.append(" ".join(lines[i]))
                i += 1
            i += 1
        else:
            raise AssertionError(f"unexpected trace line {' '.join(tok)[:40]}")
    engine.set_option(C.QFG_OPT_COVERAGE_COMPAT, 0)
    for b in list(sets.values()):
        b.close()
    ref_s = [float(x) for x in z["reference_seconds"]]
    return {"calls": calls, "gpu_seconds": gpu_s, "gpu_seconds_total": sum(gpu_s.values()),
            "reference_seconds": {"learn": ref_s[0], "evaluate": ref_s[1], "extend": ref_s[2],
                                  "coverage": ref_s[3]},
            "reference_clauses": [str(c) for c in z["clauses"]],
            "knowledge_base": {"pictures": pictures, "element": len(kb.relations[0][0]),
                               "inside": len(kb.relations[4][0]), "positives": P,
                               "negatives": len(kb.target_columns[0]) - P}}


class _DeviceColumn:
    """Exposes an engine-owned int32 device column through
    __cuda_array_interface__, so torch can wrap it without a copy."""

    def __init__(self, ptr: int, n: int):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<i4", "data": (ptr, False),
                                         "version": 3, "strides": None}
