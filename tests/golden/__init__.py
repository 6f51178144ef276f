"""Readers of the golden fixtures (produced by make_golden.py from the
reference's own code)."""
from __future__ import annotations

import os

import numpy as np

from quickfoil_gb300.engine import Literal

HERE = os.path.dirname(os.path.abspath(__file__))


def unpack_relations(z, prefix):
    rels = []
    for i in range(int(z[f"{prefix}num"][0])):
        cols = []
        k = 0
        while f"{prefix}{i}_{k}" in z:
            cols.append(z[f"{prefix}{i}_{k}"])
            k += 1
        rels.append(cols)
    return rels


def unpack_literals(a):
    lits = []
    for row in a:
        vars_ = []
        for v in row[2:]:
            if v == -2:
                break
            vars_.append(int(v))
        lits.append(Literal(int(row[0]), tuple(vars_), int(row[1])))
    return lits


def eval_cases():
    """[(relations, binding_columns, num_positive, literals, reference counts)]"""
    z = np.load(os.path.join(HERE, "eval_cases.npz"))
    out = []
    for i in range(int(z["num_cases"][0])):
        nb, P = (int(v) for v in z[f"c{i}_meta"])
        out.append((unpack_relations(z, f"c{i}_r"), [z[f"c{i}_b{k}"] for k in range(nb)], P,
                    unpack_literals(z[f"c{i}_lits"]), z[f"c{i}_counts"]))
    return out


def kinship():
    return learn_trace("kinship")


def bongard():
    return learn_trace("bongard")


def learn_trace(name):
    """(relations, calls, clauses) of a learn-loop fixture; calls are
    ("evaluate", join_var, binding_columns, P, literals, counts) and
    ("extend", (npos, nneg), binding_columns, P, [literal], output_columns)."""
    z = np.load(os.path.join(HERE, f"{name}.npz"))
    rels = unpack_relations(z, "r")
    calls = []
    for j in range(int(z["num_calls"][0])):
        ncols, P = (int(v) for v in z[f"k{j}_meta"])
        cols = [z[f"k{j}_b{k}"] for k in range(ncols)]
        lits = unpack_literals(z[f"k{j}_lits"])
        if int(z[f"k{j}_kind"][0]) == 0:
            calls.append(("evaluate", int(z[f"k{j}_key"][0]), cols, P, lits, z[f"k{j}_counts"]))
        else:
            nout = int(z[f"k{j}_nout"][0])
            calls.append(("extend", tuple(int(v) for v in z[f"k{j}_key"]), cols, P, lits,
                          [z[f"k{j}_out{k}"] for k in range(nout)]))
    return rels, calls, [str(c) for c in z["clauses"]]


def input_checksum(w):
    """Order-sensitive checksums of a workload's binding columns and relations
    (one per column, below 2^61)."""
    def col_sum(c):
        c = np.asarray(c, dtype=np.int64)
        return int((c * (np.arange(len(c), dtype=np.int64) % 1000003 + 1)).sum() % (1 << 61))
    return [col_sum(c) for c in w.binding_columns] + [col_sum(c) for r in w.relations for c in r]


def batched_step_reference():
    """(distinct literals, reference counts, input checksums) of the full-size
    batched step (32M x 6 bindings, 32 relations, 256 literals)."""
    z = np.load(os.path.join(HERE, "batched_step_reference.npz"))
    return unpack_literals(z["lits"]), z["counts"], [int(v) for v in z["checksum"]]


def coverage_synthetic():
    """Seeded coverage cases: (relations, target columns, target positives,
    binding columns, binding positives, literal, uncovered rows of the
    target, divergent).  Regenerated here rather than stored; the fixture
    keeps a checksum of each case so a changed generator is caught."""
    rng = np.random.default_rng(2024)
    cases = []
    shapes = [  # (binding rows, relation tuples, domain, target columns, binding columns, arity)
        (500, 2000, 60, 2, 3, 2), (3000, 800, 80, 1, 3, 3), (4000, 300, 150, 3, 4, 2),
        (20000, 5000, 300, 2, 3, 2), (900, 900, 20, 2, 5, 3), (60, 40, 10, 1, 2, 1),
        (70000, 100000, 300, 2, 3, 2),  # sides above 32768 rows, both smaller than the relation
        (2500, 1500, 100, 3, 3, 3)]
    for i, (nb, nrel, dom, k, nc, ar) in enumerate(shapes):
        T = [rng.integers(0, dom, 3000).astype(np.int32) for _ in range(k)]
        tP = 1400
        rel = [rng.integers(0, dom, nrel).astype(np.int32) for _ in range(ar)]
        B = [rng.integers(0, dom, nb).astype(np.int32) for _ in range(nc)]
        bP = int(rng.integers(1, nb))
        if i == 6:
            bP = nb // 2
        vars_ = [int(rng.integers(-1, nc)) for _ in range(ar)]
        if i == 4:
            vars_ = [1, 1, -1]  # repeated variable
        if i == 7:
            vars_ = [0, 2, 0]
        if all(v < 0 for v in vars_):
            vars_[0] = 0
        rows = np.flatnonzero(rng.random(tP) < 0.7).astype(np.int32)
        if i == 5:
            rows = rows[:0]  # no uncovered positive left
        cases.append(([rel], T, tP, B, bP, Literal(0, tuple(vars_)), rows, False))
    # the divergent case: 35000 positive binding rows against 1000 tuples
    T = [rng.integers(0, 300, 3000).astype(np.int32) for _ in range(2)]
    rel = [rng.integers(0, 300, 1000).astype(np.int32) for _ in range(2)]
    B = [rng.integers(0, 300, 70000).astype(np.int32) for _ in range(3)]
    cases.append(([rel], T, 1500, B, 35000, Literal(0, (1, -1)),
                  np.arange(0, 1500, 2, dtype=np.int32), True))
    return cases


def coverage_case_checksum(case):
    rels, T, tP, B, bP, lit, rows, _ = case
    return input_checksum(_Cols(list(B) + list(T) + [rows], rels)) + [tP, bP]


class _Cols:
    def __init__(self, binding_columns, relations):
        self.binding_columns = binding_columns
        self.relations = relations


def coverage_cases():
    """(synthetic, traced): synthetic = [(case, counts, flags, checksum)],
    traced = [(trace name, call index, literal index, uncovered rows,
    counts, flags)]; flags are bool per uncovered positive."""
    z = np.load(os.path.join(HERE, "coverage_cases.npz"))
    syn = []
    gen = coverage_synthetic()
    for i in range(int(z["num_synthetic"][0])):
        case = gen[i]
        n = len(case[6])
        syn.append((case, tuple(int(v) for v in z[f"s{i}_counts"]),
                    np.unpackbits(z[f"s{i}_flags"], bitorder="little")[:n].astype(bool),
                    [int(v) for v in z[f"s{i}_checksum"]]))
    traced = []
    for i in range(int(z["num_traced"][0])):
        kb, j, li = (int(v) for v in z[f"t{i}_key"])
        rows = z[f"t{i}_rows"]
        traced.append((("kinship", "bongard")[kb], j, li, rows,
                       tuple(int(v) for v in z[f"t{i}_counts"]),
                       np.unpackbits(z[f"t{i}_flags"], bitorder="little")[:len(rows)].astype(bool)))
    return syn, traced


def test_runs():
    """[(name, learnt clauses, test positive columns, test negative columns,
    (reference uncovered positives, uncovered negatives))]"""
    z = np.load(os.path.join(HERE, "test_runs.npz"))
    out = []
    for i in range(int(z["num_runs"][0])):
        k = 0
        while f"t{i}_pos{k}" in z:
            k += 1
        out.append((str(z[f"t{i}_name"][0]), [str(c) for c in z[f"t{i}_clauses"]],
                    [z[f"t{i}_pos{q}"] for q in range(k)], [z[f"t{i}_neg{q}"] for q in range(k)],
                    tuple(int(v) for v in z[f"t{i}_uncovered"])))
    return out


def text_texts():
    """Texts for the loader: (name, text bytes, argument count, skipped
    flags).  Regenerated here rather than stored; the fixture keeps the
    reference's columns (small texts) or their checksums."""
    rng = np.random.default_rng(31)
    cases = []
    lines = []
    for i in range(1000):
        if i % 97 == 0:
            lines.append(b"# comment " + str(i).encode())
        elif i % 89 == 0:
            lines.append(b"")
        lines.append(b"%d|%d" % (rng.integers(-10 ** 6, 10 ** 6), rng.integers(0, 10 ** 9)))
    cases.append(("plain", b"\n".join(lines) + b"\n", 2, None))
    tricky = [b"  12|\t-7", b"+5|0007", b"12abc|3 4", b"-0|+0", b"2147483647|-2147483648",
              b"\t \v42|\f9x", b"#|not|a|row", b"8|9\r", b"", b"  -13  |  +21  "]
    cases.append(("tricky", b"\n".join(tricky) + b"\n", 2, None))
    cases.append(("crlf", b"1|2\r\n3|4\r\n#c\r\n5|6\r\n", 2, None))
    cases.append(("skipped", b"1|xyz|3|4\n5||7|8\n9|  |11|12\n", 4, [0, 1, 0, 0]))
    cases.append(("no_final_newline", b"10|20\n30|40", 2, None))
    cases.append(("only_comments", b"# a\n#b\n\n", 1, None))
    cases.append(("one_line", b"-99", 1, None))
    big = rng.integers(-2 ** 31, 2 ** 31, (200_000, 3))
    rows = [b"|".join(b"%d" % v for v in r) for r in big]
    for i in range(0, len(rows), 1000):
        rows[i] = b"#" + rows[i]
    cases.append(("random_200k", b"\n".join(rows) + b"\n", 3, None))
    return cases


def text_rejects():
    """(text, argument count) pairs the loader rejects, with the oracle's
    error code and first bad line in test_textload.py."""
    return [(b"1|2\n3\n", 2), (b"1|2|3\n", 2), (b"1|2\n|5\n", 2), (b"1|x\n", 2),
            (b"+-1|2\n", 2), (b"- 1|2\n", 2), (b"   \n", 1), (b"1\n\r\n", 1),
            (b"2147483648\n", 1), (b"#x\n-2147483649\n", 1),
            (b"99999999999999999999999\n", 1), (b"1|2\n3|4|5\n6|x\n", 2)]


def column_checksums(cols):
    """Order-sensitive checksum per column (below 2^61)."""
    return [input_checksum(_Cols([np.asarray(c)], []))[0] for c in cols]


def text_rejects_accepted():
    """Per text_rejects() entry: whether the reference's LoadData accepted
    it (it aborts on a rejected text)."""
    z = np.load(os.path.join(HERE, "text_cases.npz"))
    return [bool(v) for v in z["rejects_accepted"]]


def text_cases():
    """[(name, text, argument count, skipped flags, reference columns or
    None, row count, column checksums)]"""
    z = np.load(os.path.join(HERE, "text_cases.npz"))
    out = []
    for i, (name, text, nargs, skipped) in enumerate(text_texts()):
        assert str(z[f"x{i}_name"][0]) == name
        ncols = int(z[f"x{i}_ncols"][0])
        cols = [z[f"x{i}_c{q}"] for q in range(ncols)] if f"x{i}_c0" in z else None
        out.append((name, text, nargs, skipped, cols, int(z[f"x{i}_rows"][0]),
                    [int(v) for v in z[f"x{i}_checksum"]]))
    return out


def after_semijoin_cases():
    """[(keys, bits (uint64 blocks), chunk_rows, num_build_tuples, reference
    buckets, reference next (0 where no chain reaches), reference mask)] of
    BuildHashTableAfterSemiJoin (after_semijoin_cases.npz)."""
    z = np.load(os.path.join(HERE, "after_semijoin_cases.npz"))
    out = []
    for j in range(int(z["num_cases"][0])):
        n, k, chunk, nbt, mask = (int(v) for v in z[f"c{j}_meta"])
        out.append(([z[f"c{j}_k{q}"] for q in range(k)], z[f"c{j}_bits"], chunk, nbt,
                    z[f"c{j}_buckets"], z[f"c{j}_next"], mask))
    return out
