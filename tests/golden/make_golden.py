"""Generates the golden fixtures in this directory from the reference's own
code (oracle/_ref, built from the reference sources by oracle/build_ref.sh).

    python tests/golden/make_golden.py [--coverage | --text]
        (--coverage: coverage_cases.npz and test_runs.npz only;
         --text: text_cases.npz only)

* eval_cases.npz   -- seeded evaluation cases (uniform and Zipf relations,
                      atoms, repeated variables, P = 0 / P = n, no join
                      result) with the counts the reference's
                      CandidateLiteralEvaluator produced.
* batched_step_reference.npz (--batched-step, about 6 minutes) -- the
                      reference's counts for every distinct literal of the
                      full-size batched step with checksums of its inputs.
* kinship.npz      -- the kinship knowledge base (relations, target) and the
                      reference learner's trace: every Evaluate call
                      (binding set, literals in result order, counts) and
                      every CreateLabelAwareBindingTables call (binding set,
                      literal, announced counts, output columns), plus the
                      learnt clauses.
* bongard.npz      -- the same for a Bongard-like knowledge base (2000
                      pictures, planted rule "a circle inside a triangle",
                      clauses up to 4 literals).
* test_runs.npz    -- the reference learner's clauses and its test runner's
                      uncovered counts (QuickFoilTestRunner::RunTest) on
                      held-out test tables of the kinship and Bongard
                      knowledge bases (every rule-true example as a test
                      positive, fresh negatives).
* text_cases.npz   -- '|'-delimited texts (comments, empty lines, white
                      space, signs, trailing characters, CR LF endings,
                      int32 limits, skipped arguments, no final newline, a
                      200K-line random file) and the columns the reference's
                      own LoadData (main/main.cpp:49-109) read from them.
* coverage_cases.npz -- the reference's ComputeCoverageOnUncoveredData
                      (covered counts, covered flag per uncovered positive)
                      on seeded synthetic cases (repeated and unbound
                      arguments, 1-3 target columns, no uncovered positive,
                      label sides above 32768 rows smaller than the
                      relation) and on every Evaluate call of the kinship
                      and Bongard traces, each literal appended to that
                      call's binding set.  One case marked divergent has a
                      label side of more than 32768 rows that is not smaller
                      than the relation, where the reference's chunk-relative
                      row ids make its counts differ from set membership.

* bongard_kb_trace.npz (--bongard-kb, about a minute) -- BASELINE config 4
                      at full scale (1M pictures): the reference learner's
                      compact trace (checksums in place of binding sets,
                      coverage steps included), its clauses and its times.
* after_semijoin_cases.npz (--after-semijoin) -- the reference's
                      BuildHashTableAfterSemiJoin tables (buckets, the
                      next links chains reach, mask) for seeded projected
                      columns and semi-join bits in one or many chunks.

Only this script reads the reference; the tests read the fixtures, so they
also run where the reference sources are absent.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle.ref as ref  # noqa: E402
from quickfoil_gb300 import workloads  # noqa: E402
from quickfoil_gb300.engine import Literal  # noqa: E402
from tests.golden import (column_checksums, coverage_case_checksum, coverage_synthetic,  # noqa: E402
                          input_checksum, text_rejects, text_texts)


def pack_relations(relations, prefix, out):
    out[f"{prefix}num"] = np.array([len(relations)])
    for i, r in enumerate(relations):
        for k, c in enumerate(r):
            out[f"{prefix}{i}_{k}"] = np.asarray(c, dtype=np.int32)


def pack_literals(lits):
    a = np.full((len(lits), 10), -1, dtype=np.int32)
    for i, l in enumerate(lits):
        rel, vars_, jp = l.as_tuple()
        a[i, 0], a[i, 1] = rel, jp
        a[i, 2:2 + len(vars_)] = vars_
        a[i, 2 + len(vars_):] = -2  # arity terminator
    return a


def eval_cases():
    out = {}
    cases = []
    for seed in range(8):
        w = workloads.small_random(seed, n_bindings=2000, max_tuples=1500, num_literals=30,
                                   zipf=seed % 2 == 0)
        P = w.num_positive
        if seed == 6:
            P = 0
        if seed == 7:
            P = w.num_bindings
        cases.append((w.relations, w.binding_columns, P, list(dict.fromkeys(w.literals))))
    # a call with no join result at all: the reference would crash, the
    # driver answers zeros (operations/CountAggregator.cpp:112-116)
    rng = np.random.default_rng(99)
    B = [rng.integers(0, 10, 200).astype(np.int32) for _ in range(2)]
    R = [[np.arange(100, 120, dtype=np.int32), np.arange(20, dtype=np.int32)]]
    cases.append((R, B, 50, [Literal(0, (0, -1)), Literal(0, (1, 0))]))
    for i, (rels, B, P, lits) in enumerate(cases):
        counts = ref.evaluate(rels, B, P, lits, radix_bits=5)
        pack_relations(rels, f"c{i}_r", out)
        for k, c in enumerate(B):
            out[f"c{i}_b{k}"] = np.asarray(c, dtype=np.int32)
        out[f"c{i}_meta"] = np.array([len(B), P])
        out[f"c{i}_lits"] = pack_literals(lits)
        out[f"c{i}_counts"] = counts
    out["num_cases"] = np.array([len(cases)])
    np.savez_compressed(os.path.join(HERE, "eval_cases.npz"), **out)
    print("eval_cases.npz:", len(cases), "cases")


def parse_trace(path):
    """Trace lines written by oracle/ref_driver.cpp."""
    lines = open(path).read().splitlines()
    i = 0
    calls = []

    def read_bindings():
        nonlocal i
        _, ncols, P, N = lines[i].split()
        i += 1
        cols = []
        for _ in range(int(ncols)):
            vals = lines[i].split()[1:]
            cols.append(np.array([int(v) for v in vals], dtype=np.int32))
            i += 1
        return cols, int(P), int(N)

    def read_literal():
        nonlocal i
        parts = [int(v) for v in lines[i].split()[1:]]
        i += 1
        pred, nvars, jk = parts[:3]
        return Literal(pred, tuple(parts[3:3 + nvars]), jk)

    clauses = []
    while i < len(lines):
        head = lines[i].split()
        if head[0] == "EVALUATE":
            key, n = int(head[1]), int(head[2])
            i += 1
            cols, P, N = read_bindings()
            lits, counts = [], []
            for _ in range(n):
                lits.append(read_literal())
                counts.append([int(v) for v in lines[i].split()[1:]])
                i += 1
            calls.append(("evaluate", key, cols, P, lits, np.array(counts, dtype=np.int64)))
        elif head[0] == "EXTEND":
            npos, nneg = int(head[1]), int(head[2])
            i += 1
            cols, P, N = read_bindings()
            lit = read_literal()
            outs = []
            while i < len(lines) and lines[i].startswith("OUT"):
                vals = lines[i].split()[1:]
                outs.append(np.array([int(v) for v in vals], dtype=np.int32))
                i += 1
            calls.append(("extend", (npos, nneg), cols, P, [lit], outs))
        elif head[0] == "CLAUSES":
            i += 1
            while lines[i] != "END":
                clauses.append(lines[i])
                i += 1
            i += 1
        else:
            raise ValueError(f"unexpected trace line {lines[i][:40]}")
    return calls, clauses


def learn_fixture(task, name):
    trace = os.path.join(HERE, f"_{name}_trace.txt")
    clauses = ref.learn(task.relations, task.target_columns, task.num_positive,
                        task.max_clause_length, trace)
    calls, traced_clauses = parse_trace(trace)
    os.remove(trace)
    assert traced_clauses == clauses
    out = {}
    pack_relations(task.relations, "r", out)
    for k, c in enumerate(task.target_columns):
        out[f"target{k}"] = c
    out["meta"] = np.array([len(task.target_columns), task.num_positive, task.max_clause_length])
    out["num_calls"] = np.array([len(calls)])
    for j, (kind, key, cols, P, lits, result) in enumerate(calls):
        out[f"k{j}_kind"] = np.array([0 if kind == "evaluate" else 1])
        out[f"k{j}_key"] = np.array(key if kind == "extend" else [key, 0])
        out[f"k{j}_meta"] = np.array([len(cols), P])
        for k, c in enumerate(cols):
            out[f"k{j}_b{k}"] = c
        out[f"k{j}_lits"] = pack_literals(lits)
        if kind == "evaluate":
            out[f"k{j}_counts"] = result
        else:
            out[f"k{j}_nout"] = np.array([len(result)])
            for k, c in enumerate(result):
                out[f"k{j}_out{k}"] = c
    out["clauses"] = np.array(clauses)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}.npz:", len(calls), "calls;", clauses)


def kinship():
    learn_fixture(workloads.kinship(seed=1), "kinship")


def bongard():
    learn_fixture(workloads.bongard(seed=1, pictures=2000, max_positive=300), "bongard")


def _coverage_from_traces():
    """(trace name, call index, literal index, uncovered rows) of every
    literal of every Evaluate call of the kinship and Bongard traces."""
    from tests.golden import learn_trace
    out = []
    for name in ("kinship", "bongard"):
        rels, calls, _ = learn_trace(name)
        target = next(c for c in calls if c[0] == "evaluate")
        P = target[3]
        rng = np.random.default_rng(len(name))
        for j, call in enumerate(calls):
            if call[0] != "evaluate":
                continue
            for i in range(len(call[4])):
                rows = np.arange(P, dtype=np.int32)
                if (i + j) % 2:
                    rows = np.flatnonzero(rng.random(P) < 0.5).astype(np.int32)
                out.append((name, j, i, rows))
    return out


def coverage_cases():
    from tests.golden import learn_trace
    out = {}
    syn = coverage_synthetic()
    for i, (rels, T, tP, B, bP, lit, rows, divergent) in enumerate(syn):
        U = [t[rows] for t in T]
        counts, flags = ref.coverage(rels, T, tP, B, bP, lit, U)
        out[f"s{i}_checksum"] = np.array(coverage_case_checksum(syn[i]), dtype=np.uint64)
        out[f"s{i}_counts"] = np.array(counts, dtype=np.int64)
        out[f"s{i}_flags"] = np.packbits(flags, bitorder="little")
    out["num_synthetic"] = np.array([len(syn)])
    traced = _coverage_from_traces()
    cache = {}
    for i, (name, j, li, rows) in enumerate(traced):
        if name not in cache:
            cache[name] = learn_trace(name)
        rels, calls, _ = cache[name]
        target = next(c for c in calls if c[0] == "evaluate")
        T, tP = target[2], target[3]
        _, _, B, bP, lits, _ = calls[j]
        U = [t[rows] for t in T]
        counts, flags = ref.coverage(rels, T, tP, B, bP, lits[li], U)
        out[f"t{i}_key"] = np.array([0 if name == "kinship" else 1, j, li])
        out[f"t{i}_rows"] = rows
        out[f"t{i}_counts"] = np.array(counts, dtype=np.int64)
        out[f"t{i}_flags"] = np.packbits(flags, bitorder="little")
    out["num_traced"] = np.array([len(traced)])
    np.savez_compressed(os.path.join(HERE, "coverage_cases.npz"), **out)
    print("coverage_cases.npz:", len(syn), "synthetic,", len(traced), "traced cases")


def test_runs():
    out = {}
    tasks = [("kinship", workloads.kinship(seed=1),
              workloads.kinship(seed=1, max_positive=10 ** 6, num_negative=2000)),
             ("bongard", workloads.bongard(seed=1, pictures=2000, max_positive=300),
              workloads.bongard(seed=1, pictures=2000, max_positive=10 ** 6))]
    for i, (name, train, test) in enumerate(tasks):
        assert all(np.array_equal(a, b) for ra, rb in zip(train.relations, test.relations)
                   for a, b in zip(ra, rb))
        P = test.num_positive
        # Mixed test tables: a quarter of each side's rows come from the
        # other side, so a test table is neither all covered nor all not.
        rng = np.random.default_rng(7 + i)
        n = len(test.target_columns[0])
        pos_rows = np.concatenate([np.arange(P), rng.choice(np.arange(P, n), (n - P) // 4)])
        neg_rows = np.concatenate([np.arange(P, n), rng.choice(np.arange(P), P // 4)])
        pos_rows, neg_rows = rng.permutation(pos_rows), rng.permutation(neg_rows)
        tpos = [c[pos_rows] for c in test.target_columns]
        tneg = [c[neg_rows] for c in test.target_columns]
        clauses, unc = ref.learn_test(train.relations, train.target_columns, train.num_positive,
                                      train.max_clause_length, tpos, tneg)
        out[f"t{i}_name"] = np.array([name])
        out[f"t{i}_clauses"] = np.array(clauses)
        for q, c in enumerate(tpos):
            out[f"t{i}_pos{q}"] = c
        for q, c in enumerate(tneg):
            out[f"t{i}_neg{q}"] = c
        out[f"t{i}_uncovered"] = np.array(unc, dtype=np.int64)
        print(name, clauses, "uncovered test rows", unc, "of", len(tpos[0]), len(tneg[0]))
    out["num_runs"] = np.array([len(tasks)])
    np.savez_compressed(os.path.join(HERE, "test_runs.npz"), **out)


def text_cases():
    import tempfile
    out = {}
    cases = text_texts()
    for i, (name, text, nargs, skipped) in enumerate(cases):
        with tempfile.NamedTemporaryFile(suffix=".txt", delete=False) as f:
            f.write(text)
            path = f.name
        try:
            cols = ref.load_text(path, nargs, skipped)
        finally:
            os.unlink(path)
        out[f"x{i}_name"] = np.array([name])
        out[f"x{i}_rows"] = np.array([len(cols[0]) if cols else 0])
        out[f"x{i}_checksum"] = np.array(column_checksums(cols), dtype=np.uint64)
        if len(text) < 100_000:  # small texts keep the reference's columns too
            for q, c in enumerate(cols):
                out[f"x{i}_c{q}"] = c
        out[f"x{i}_ncols"] = np.array([len(cols)])
        print(name, [len(c) for c in cols], [c[:4].tolist() for c in cols])
    out["num_texts"] = np.array([len(cases)])
    # Texts the reference rejects: its LoadData aborts the process (CHECK or
    # LOG(FATAL)), so each runs in a child process; the fixture records
    # whether the reference accepted it.
    import subprocess
    bad = text_rejects()
    accepted = []
    for j, (text, nargs) in enumerate(bad):
        with tempfile.NamedTemporaryFile(suffix=".txt", delete=False) as f:
            f.write(text)
            path = f.name
        try:
            rc = subprocess.run([sys.executable, "-c",
                                 "import sys; sys.path.insert(0, %r); import oracle.ref as r; "
                                 "r.load_text(%r, %d)" % (ROOT, path, nargs)],
                                capture_output=True).returncode
        finally:
            os.unlink(path)
        accepted.append(rc == 0)
    out["rejects_accepted"] = np.array(accepted)
    print("reference accepted", sum(accepted), "of", len(bad), "rejected texts")
    np.savez_compressed(os.path.join(HERE, "text_cases.npz"), **out)


def after_semijoin_cases():
    """The reference's BuildHashTableAfterSemiJoin on seeded projected columns
    and semi-join bits: one chunk (a right semi-join's output) and several
    32768-row chunks (a left semi-join's), where positions are chunk-relative
    (operations/LeftSemiJoin.hpp:55-83), plus short chunks, no or all bits
    set and more than six keys (Hash<k> over every key, utility/Hash.hpp:
    47-55).  num_build_tuples is the projected side's row count, as the
    learner passes it (learner/QuickFoil.cpp:515-517)."""
    rng = np.random.default_rng(77)
    specs = [  # rows, keys, key domain, chunk rows, density of set bits
        (1000, 1, 300, 0, 0.5), (5000, 2, 40, 0, 0.7), (3000, 3, 8, 0, 0.9),
        (100_000, 1, 5000, 32768, 0.6), (100_000, 2, 60, 32768, 0.5), (70_000, 3, 12, 32768, 0.8),
        (20_000, 2, 30, 1000, 0.5), (4000, 2, 50, 0, 0.0), (4000, 2, 50, 0, 1.0),
        (2000, 7, 3, 0, 0.6), (33_000, 1, 100_000, 32768, 0.9)]
    out = {"num_cases": np.array([len(specs)])}
    for j, (n, k, dom, chunk, dens) in enumerate(specs):
        keys = [rng.integers(0, dom, n).astype(np.int32) for _ in range(k)]
        flags = rng.random(n) < dens
        bits = np.packbits(np.concatenate([flags, np.zeros((-n) % 64, bool)]).reshape(-1, 64)[:, ::-1],
                           axis=1).view(">u8").astype(np.uint64).ravel()
        # In a short last chunk the reference compares against chain positions
        # past the chunk's end, reading past the end of its columns.  The
        # columns handed to it are padded with -1 (outside every key domain
        # here), so those reads compare unequal, as the engine defines them.
        padded = [np.concatenate([c, np.full(max(chunk, 1), -1, np.int32)]) for c in keys]
        buckets, nxt, mask = ref.build_after_semijoin(padded, bits, chunk, n, num_rows=n)
        out[f"c{j}_meta"] = np.array([n, k, chunk, n, mask], dtype=np.int64)
        for q, c in enumerate(keys):
            out[f"c{j}_k{q}"] = c
        out[f"c{j}_bits"] = bits
        out[f"c{j}_buckets"] = buckets
        out[f"c{j}_next"] = nxt
    np.savez_compressed(os.path.join(HERE, "after_semijoin_cases.npz"), **out)
    print("after_semijoin_cases.npz:", len(specs), "cases")


def column_checksum(v):
    """The trace's column checksum (oracle/ref_driver.cpp ColumnChecksum)."""
    v = (np.asarray(v, dtype=np.int32).view(np.uint32).astype(np.uint64) + np.uint64(0x9E3779B9))
    r = np.arange(len(v), dtype=np.uint64) * np.uint64(2) + np.uint64(1)
    return int(np.sum(v * r, dtype=np.uint64))


def bongard_kb_trace():
    """BASELINE config 4 at full scale: the Bongard-like knowledge base of
    workloads.bongard_kb() (1M pictures, element 10M, inside about 16M,
    100K positives) and the reference learner's compact trace on it --
    every Evaluate call (binding-set checksums, literals, counts), every
    binding-set extension (input and output checksums), every coverage step
    (relation and bound arguments, label-side checksums, examples' checksum,
    covered count and bit sums) -- with its learnt clauses and its times."""
    k = workloads.bongard_kb()
    path = os.path.join(HERE, "_bongard_kb_trace.txt")
    clauses, secs = ref.learn_compact(k.relations, k.target_columns, k.num_positive,
                                      k.max_clause_length, path)
    with open(path, "rb") as f:
        text = f.read()
    os.remove(path)
    out = {"trace": np.frombuffer(text, dtype=np.uint8),
           "params": np.array([4, 1_000_000, 100_000, k.max_clause_length]),
           "relation_checksums": np.array([column_checksum(c) for r in k.relations for c in r],
                                          dtype=np.uint64),
           "target_checksum": np.array([column_checksum(k.target_columns[0]), k.num_positive],
                                       dtype=np.uint64),
           "clauses": np.array(clauses),
           "reference_seconds": np.array(secs),
           "reference_host": np.array(["x86_64 build container, 1 thread, -O3"])}
    np.savez_compressed(os.path.join(HERE, "bongard_kb_trace.npz"), **out)
    print("bongard_kb_trace.npz:", text.count(b"\n"), "lines;", clauses, secs)


if __name__ == "__main__" and "--bongard-kb" in sys.argv:
    bongard_kb_trace()
    sys.exit(0)


if __name__ == "__main__" and "--after-semijoin" in sys.argv:
    after_semijoin_cases()
    sys.exit(0)


if __name__ == "__main__" and "--batched-step" not in sys.argv:
    if "--text" in sys.argv:
        text_cases()
        sys.exit(0)
    if "--coverage" not in sys.argv:
        text_cases()
        eval_cases()
        kinship()
        bongard()
    coverage_cases()
    test_runs()


def batched_step_reference():
    """Reference counts for every distinct literal of the full-size batched
    step (32M x 6 bindings, 32 relations, 256 literals) plus checksums of the
    generated inputs, so a test can regenerate the step and compare the GPU
    engine with the reference's own counts at full size."""
    w = workloads.batched_step()
    lits = list(dict.fromkeys(w.literals))
    counts = ref.evaluate(w.relations, w.binding_columns, w.num_positive, lits, radix_bits=5)
    out = {"lits": pack_literals(lits), "counts": counts,
           "checksum": np.array(input_checksum(w), dtype=np.uint64)}
    np.savez_compressed(os.path.join(HERE, "batched_step_reference.npz"), **out)
    print("batched_step_reference.npz:", len(lits), "literals")


if __name__ == "__main__" and "--batched-step" in sys.argv:
    batched_step_reference()
