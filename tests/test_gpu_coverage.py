"""GPU coverage (qfg_coverage, the drop-in for ComputeCoverageOnUncoveredData
and ComputeCoveredPositives) and the uncovered-example compaction
(qfg_compact_rows), bit-exact: against the reference's own results (golden
fixture: synthetic cases and every Evaluate call of the kinship and Bongard
learn traces), against the oracle on seeded cases up to 8M binding rows, and
through the learner's own invariant -- after compaction nothing left is
covered by the same literal."""
import numpy as np
import pytest

import oracle
from quickfoil_gb300 import QfgError
from quickfoil_gb300.engine import Literal
from tests import golden
from tests.test_coverage import bits_to_flags

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

_ids = [900_000]


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).cuda()


def _register(engine, rels):
    base = _ids[0]
    _ids[0] += len(rels) + 10
    for i, r in enumerate(rels):
        engine.register_relation(base + i, r)
    return base


def _gpu_coverage(engine, rels, B, bP, lit, k, U, negatives, bits=True, prepared=False,
                  compat=False):
    """Through qfg_coverage, or (prepared) through qfg_coverage_examples;
    compat: under QFG_OPT_COVERAGE_COMPAT."""
    from quickfoil_gb300 import _capi as C
    engine.set_option(C.QFG_OPT_COVERAGE_COMPAT, 1 if compat else 0)
    try:
        return _gpu_coverage_run(engine, rels, B, bP, lit, k, U, negatives, bits, prepared)
    finally:
        engine.set_option(C.QFG_OPT_COVERAGE_COMPAT, 0)


def _gpu_coverage_run(engine, rels, B, bP, lit, k, U, negatives, bits, prepared):
    base = _register(engine, rels)
    b = engine.bindings([dev(c) for c in B], bP)
    dU = [dev(c) for c in U]
    dN = None if negatives is None else [dev(c) for c in negatives]
    try:
        glit = Literal(base + lit.relation, lit.vars, lit.join_pos)
        if prepared:
            eu = engine.examples(dU)
            en = engine.examples(dN) if dN is not None else None
            counts, dbits = engine.coverage_examples(b, glit, eu, en, positive_bits=bits)
            eu.close()
            if en is not None:
                en.close()
        else:
            counts, dbits = engine.coverage(b, glit, k, dU, dN, positive_bits=bits)
    finally:
        b.close()
    flags = None if dbits is None else bits_to_flags(dbits.cpu().numpy().view(np.uint64), len(U[0]))
    return counts, flags


def test_coverage_matches_reference_on_synthetic_cases(engine):
    for case, want_counts, want_flags, _ in golden.coverage_cases()[0]:
        rels, T, tP, B, bP, lit, rows, divergent = case
        U = [t[rows] for t in T]
        counts, flags = _gpu_coverage(engine, rels, B, bP, lit, len(T), U, [t[tP:] for t in T])
        if divergent:  # set membership: the oracle's answer
            want_counts, wbits = oracle.coverage(B, bP, rels[0], lit.as_tuple(), len(T), U,
                                                 [t[tP:] for t in T])
            want_flags = bits_to_flags(wbits, len(rows))
        assert counts == want_counts
        np.testing.assert_array_equal(flags, want_flags)


@pytest.mark.parametrize("prepared", [False, True])
def test_compat_coverage_matches_reference_everywhere(engine, prepared):
    """QFG_OPT_COVERAGE_COMPAT: the reference's own procedure, chunk-relative
    projection tables included -- equal to the reference on every synthetic
    case, the divergent one (a label side of more than 32768 rows, not
    smaller than the relation) included."""
    seen_divergent = False
    for case, want_counts, want_flags, _ in golden.coverage_cases()[0]:
        rels, T, tP, B, bP, lit, rows, divergent = case
        U = [t[rows] for t in T]
        counts, flags = _gpu_coverage(engine, rels, B, bP, lit, len(T), U, [t[tP:] for t in T],
                                      prepared=prepared, compat=True)
        assert counts == want_counts, divergent
        np.testing.assert_array_equal(flags, want_flags)
        seen_divergent |= bool(divergent)
    assert seen_divergent


@pytest.mark.parametrize("seed,nb,nrel,dom,k", [(0, 100_000, 5000, 300, 2), (1, 200_000, 900, 40, 1),
                                                (2, 80_000, 80_001, 50, 2), (3, 150_000, 20_000, 9, 3)])
def test_compat_coverage_matches_compat_oracle(engine, seed, nb, nrel, dom, k):
    rng = np.random.default_rng(seed)
    B = [rng.integers(0, dom, nb).astype(np.int32) for _ in range(4)]
    bP = nb // 3
    rel = [rng.integers(0, dom, nrel).astype(np.int32) for _ in range(2)]
    lit = Literal(0, (k - 1 if k > 1 else 0, 3), 0)
    U = [rng.integers(0, dom, 40_000).astype(np.int32) for _ in range(k)]
    Ng = [rng.integers(0, dom, 60_000).astype(np.int32) for _ in range(k)]
    counts, flags = _gpu_coverage(engine, [rel], B, bP, lit, k, U, Ng, compat=True)
    want, wbits = oracle.coverage(B, bP, rel, lit.as_tuple(), k, U, Ng, compat=True)
    assert counts == want
    np.testing.assert_array_equal(flags, bits_to_flags(wbits, len(U[0])))


@pytest.mark.parametrize("name", ["kinship", "bongard"])
def test_coverage_matches_reference_on_learn_traces(engine, name):
    rels, calls, _ = golden.learn_trace(name)
    target = next(c for c in calls if c[0] == "evaluate")
    T, tP = target[2], target[3]
    base = _register(engine, rels)
    negatives = [dev(t[tP:]) for t in T]
    n = 0
    for kb, j, li, rows, want_counts, want_flags in golden.coverage_cases()[1]:
        if kb != name:
            continue
        _, _, B, bP, lits, _ = calls[j]
        lit = lits[li]
        b = engine.bindings([dev(c) for c in B], bP)
        counts, bits = engine.coverage(b, Literal(base + lit.relation, lit.vars, lit.join_pos),
                                       len(T), [dev(t[rows]) for t in T], negatives)
        b.close()
        assert counts == want_counts, (j, li)
        np.testing.assert_array_equal(bits_to_flags(bits.cpu().numpy().view(np.uint64), len(rows)),
                                      want_flags)
        n += 1
    assert n > 10


@pytest.mark.parametrize("seed,nb,nrel,dom,k,nc,ar", [
    (0, 5000, 3000, 50, 2, 3, 2), (1, 20000, 200, 400, 1, 2, 3), (2, 100000, 100000, 2000, 3, 4, 2),
    (3, 777, 5, 3, 2, 5, 3), (4, 1, 1, 1, 1, 1, 1), (5, 300000, 70000, 5000, 2, 3, 2),
    (6, 2, 100, 4, 2, 2, 2), (7, 50000, 20000, 12, 4, 5, 4), (8, 40000, 3000, 6, 5, 6, 5)])
def test_coverage_matches_oracle(engine, seed, nb, nrel, dom, k, nc, ar):
    rng = np.random.default_rng(seed)
    rel = [rng.integers(0, dom, nrel).astype(np.int32) for _ in range(ar)]
    B = [rng.integers(0, dom, nb).astype(np.int32) for _ in range(nc)]
    U = [rng.integers(0, dom, 3000).astype(np.int32) for _ in range(k)]
    neg = [rng.integers(0, dom, 2500).astype(np.int32) for _ in range(k)]
    for bP in sorted({0, nb // 3, nb}):
        vars_ = [int(rng.integers(-1, nc)) for _ in range(ar)]
        if all(v < 0 for v in vars_):
            vars_[0] = int(rng.integers(0, nc))
        lit = Literal(0, tuple(vars_))
        want = oracle.coverage(B, bP, rel, lit.as_tuple(), k, U, neg)
        for prepared in (False, True):
            counts, flags = _gpu_coverage(engine, [rel], B, bP, lit, k, U, neg, prepared=prepared)
            assert counts == want[0]
            np.testing.assert_array_equal(flags, bits_to_flags(want[1], len(U[0])))
        # positives only (ComputeCoveredPositives), no bit vector
        counts, flags = _gpu_coverage(engine, [rel], B, bP, lit, k, U, None, bits=False)
        assert counts == (want[0][0], 0) and flags is None


def test_coverage_of_empty_inputs(engine):
    rel = [np.array([1, 2, 3], dtype=np.int32)]
    B = [np.array([1, 2, 5, 1], dtype=np.int32)]
    U0 = [np.zeros(0, dtype=np.int32)]
    base = _register(engine, [rel])
    b = engine.bindings([dev(c) for c in B], 2)
    lit = Literal(base, (0,))
    assert engine.coverage(b, lit, 1, [dev(c) for c in U0], None)[0] == (0, 0)
    counts, bits = engine.coverage(b, lit, 1, [dev(np.array([1, 2, 5, 3, 1], np.int32))],
                                   [dev(np.array([1, 5, 2], np.int32))])
    assert counts == (3, 1)
    assert bits_to_flags(bits.cpu().numpy().view(np.uint64), 5).tolist() == [True, True, False,
                                                                             False, True]
    with pytest.raises(ValueError):  # the host-side literal already refuses it
        Literal(base, (-1,))
    # the C ABI refuses it too
    from quickfoil_gb300 import _capi as C
    raw = C.QfgLiteral()
    raw.relation_id, raw.num_args, raw.join_pos = base, 1, 0
    raw.vars[0] = -1
    counts = (C.ctypes.c_int64 * 2)()
    assert engine.lib.qfg_coverage(engine.ctx, b.handle, C.ctypes.byref(raw), 1, None, 0, None, 0,
                                   None, counts) == C.QFG_ERR_INVALID
    with pytest.raises(QfgError):
        engine.coverage(b, lit, 2, [dev(c) for c in U0], None)
    b.close()


def _bits_of(flags):
    n = len(flags)
    return torch.from_numpy(np.packbits(np.concatenate([flags, np.zeros((-n) % 64, bool)]),
                                        bitorder="little").view(np.int64).copy()).cuda()


@pytest.mark.parametrize("n", [1, 31, 32, 33, 2047, 2048, 2049, 100_000, 3_000_001])
@pytest.mark.parametrize("keep_set", [False, True])
def test_compaction_keeps_rows_in_order(engine, n, keep_set):
    rng = np.random.default_rng(n)
    ncols = 10 if n == 2049 else 3  # more columns than one launch carries
    cols = [rng.integers(-9, 9, n).astype(np.int32) for _ in range(ncols)]
    flags = rng.random(n) < (0.999 if n == 33 else 0.4)
    got = engine.compact_rows([dev(c) for c in cols], _bits_of(flags), keep_set=keep_set)
    want = oracle.compact_rows(cols, np.packbits(np.concatenate([flags, np.zeros((-n) % 64, bool)]),
                                                 bitorder="little").view(np.uint64), keep_set)
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g.cpu().numpy(), w)


def test_compaction_ignores_bits_past_the_last_row_and_checks_capacity(engine):
    cols = [dev(np.arange(70, dtype=np.int32))]
    bits = torch.tensor([0, -1], dtype=torch.int64, device="cuda")  # rows 64.. set, and bits past 70
    got = engine.compact_rows(cols, bits, keep_set=True)
    assert got[0].cpu().tolist() == list(range(64, 70))
    with pytest.raises(QfgError):
        engine.compact_rows(cols, bits, keep_set=False, capacity=10)


def test_accepting_a_literal_leaves_nothing_it_covers(engine):
    """The learner's step on acceptance at 8M binding rows: coverage bits,
    compaction of the uncovered positives, and coverage of the compacted set,
    which the same literal no longer covers; the counts equal the oracle's."""
    rng = np.random.default_rng(77)
    nb, dom = 8_000_000, 1 << 20
    rel = [rng.integers(0, dom, 2_000_000).astype(np.int32) for _ in range(2)]
    B = [rng.integers(0, dom, nb).astype(np.int32) for _ in range(3)]
    T = [B[0][:1_000_000][::-1].copy(), B[1][:1_000_000][::-1].copy()]  # many examples have bindings
    lit = Literal(0, (2, -1))
    want = oracle.coverage(B, nb // 2, rel, lit.as_tuple(), 2, T, None)
    base = _register(engine, [rel])
    b = engine.bindings([dev(c) for c in B], nb // 2)
    glit = Literal(base, lit.vars)
    U = [dev(t) for t in T]
    counts, bits = engine.coverage(b, glit, 2, U, None)
    assert counts == want[0] and counts[0] > 0
    np.testing.assert_array_equal(bits.cpu().numpy().view(np.uint64), want[1])
    left = engine.compact_rows(U, bits)
    assert left[0].numel() == len(T[0]) - counts[0]
    again, _ = engine.coverage(b, glit, 2, left, None)
    assert again == (0, 0)
    b.close()


def test_coverage_of_all_ones_key_tuples(engine):
    """(-1, -1) bound keys: the one key pair whose inline encoding is the
    empty-slot marker."""
    B = [np.array([-1, -1, 3, -1, 7, -1], np.int32), np.array([-1, 2, 3, -1, -1, -1], np.int32),
         np.array([1, 2, 3, 4, 5, 6], np.int32)]
    U = [np.array([1, 2, 3, 4, 5, 6, 9], np.int32)]
    for rel in ([np.array([-1, 3], np.int32), np.array([-1, 3], np.int32)],
                [np.array([5, 3], np.int32), np.array([-1, 3], np.int32)],
                [np.array([-1], np.int32), np.array([2], np.int32)]):
        for prepared in (False, True):
            got = _gpu_coverage(engine, [rel], [B[2], B[0], B[1]], 3, Literal(0, (1, 2)), 1,
                                [U[0]], [U[0]], prepared=prepared)
            want = oracle.coverage([B[2], B[0], B[1]], 3, rel, (0, (1, 2), 0), 1, [U[0]], [U[0]])
            assert got[0] == want[0]
            np.testing.assert_array_equal(got[1], bits_to_flags(want[1], len(U[0])))


def test_relation_key_sets_follow_relation_changes(engine):
    rng = np.random.default_rng(12)
    B = [rng.integers(0, 50, 20000).astype(np.int32) for _ in range(3)]
    U = [rng.integers(0, 50, 4000).astype(np.int32) for _ in range(2)]
    rid = _ids[0]
    _ids[0] += 10
    b = engine.bindings([dev(c) for c in B], 7000)
    dU = [dev(c) for c in U]
    for version in range(3):
        rel = [rng.integers(0, 50 + 40 * version, 300).astype(np.int32) for _ in range(2)]
        engine.register_relation(rid, rel)
        for vars_ in ((2, -1), (2, 1)):
            got = engine.coverage(b, Literal(rid, vars_), 2, dU, dU)
            want = oracle.coverage(B, 7000, rel, (0, vars_, 0), 2, U, U)
            assert got[0] == want[0]
    b.close()


def test_prepared_examples_serve_many_literals(engine):
    """One prepared negative table and one uncovered-positive table against
    every literal of a step, as the learner checks its best candidates."""
    from quickfoil_gb300 import workloads
    w = workloads.small_random(31, n_bindings=60000, max_tuples=5000, num_literals=40)
    base = _register(engine, w.relations)
    b = engine.bindings([dev(c) for c in w.binding_columns], w.num_positive)
    rng = np.random.default_rng(1)
    U = [rng.integers(0, w.domain, 5000).astype(np.int32) for _ in range(2)]
    N = [rng.integers(0, w.domain, 9000).astype(np.int32) for _ in range(2)]
    eu, en = engine.examples([dev(c) for c in U]), engine.examples([dev(c) for c in N])
    for l in dict.fromkeys(w.literals):
        got = engine.coverage_examples(b, Literal(base + l.relation, l.vars, l.join_pos), eu, en)
        want = oracle.coverage(w.binding_columns, w.num_positive, w.relations[l.relation],
                               l.as_tuple(), 2, U, N)
        assert got[0] == want[0]
        np.testing.assert_array_equal(got[1].cpu().numpy().view(np.uint64), want[1])
    with pytest.raises(QfgError):  # column counts of the two tables differ
        e1 = engine.examples([dev(U[0])])
        engine.coverage_examples(b, Literal(base, (0,) * len(w.relations[0])), e1, en)
    e1.close()
    eu.close()
    en.close()
    b.close()


@pytest.mark.parametrize("arity,distinct", [(1, 150_000), (1, 600_000), (2, 600_000)])
def test_coverage_with_and_without_the_relation_filter(engine, arity, distinct):
    """Relations with up to 2^18 distinct key tuples take the shared-memory
    filter; larger ones probe the key set directly.  Half the binding rows
    carry keys of the relation, the examples are target tuples of binding
    rows (and random ones)."""
    rng = np.random.default_rng(distinct + arity)
    dom = 1 << 24
    rel = [rng.integers(0, dom, distinct).astype(np.int32) for _ in range(arity)]
    n = 1_000_000
    pick = rng.integers(0, distinct, n)
    B = [rng.integers(0, dom, n).astype(np.int32) for _ in range(2)]
    for a in range(arity):
        col = rng.integers(0, dom, n).astype(np.int32)
        half = rng.random(n) < 0.5
        col[half] = rel[a][pick[half]]
        B.append(col)
    bound = tuple(range(2, 2 + arity))
    rows = rng.integers(0, n, 60000)
    U = [np.concatenate([B[0][rows], rng.integers(0, dom, 20000).astype(np.int32)]),
         np.concatenate([B[1][rows], rng.integers(0, dom, 20000).astype(np.int32)])]
    lit = Literal(0, bound)
    want = oracle.coverage(B, n // 3, rel, lit.as_tuple(), 2, U, U)
    assert want[0][0] > 1000
    for prepared in (False, True):
        got = _gpu_coverage(engine, [rel], B, n // 3, lit, 2, U, U, prepared=prepared)
        assert got[0] == want[0]
        np.testing.assert_array_equal(got[1], bits_to_flags(want[1], len(U[0])))


def test_coverage_on_a_split_binding_set(engine):
    """Positives and negatives uploaded from separate arrays
    (qfg_bindings_create_split) give the same coverage as one table."""
    rng = np.random.default_rng(44)
    rel = [rng.integers(0, 80, 3000).astype(np.int32) for _ in range(2)]
    P, N = 7001, 12003
    B = [rng.integers(0, 80, P + N).astype(np.int32) for _ in range(3)]
    U = [rng.integers(0, 80, 2500).astype(np.int32) for _ in range(2)]
    base = _register(engine, [rel])
    lit = Literal(base, (2, -1))
    whole = engine.bindings([dev(c) for c in B], P)
    split = engine.bindings_split([dev(c[:P]) for c in B], [dev(c[P:]) for c in B])
    a = engine.coverage(whole, lit, 2, [dev(c) for c in U], [dev(c) for c in U])
    b = engine.coverage(split, lit, 2, [dev(c) for c in U], [dev(c) for c in U])
    want = oracle.coverage(B, P, rel, lit.as_tuple(), 2, U, U)
    assert a[0] == b[0] == want[0]
    assert torch.equal(a[1], b[1])
    whole.close()
    split.close()
