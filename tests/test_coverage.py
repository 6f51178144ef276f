"""Coverage of a literal appended to the building clause and the
uncovered-example compaction, on the oracle (CPU): against the reference's
own ComputeCoverageOnUncoveredData (golden fixture), against a brute-force
set-membership count, and the compaction against numpy."""
import numpy as np
import pytest

import oracle
from tests import golden


def bits_to_flags(bits, n):
    return np.unpackbits(np.asarray(bits, dtype=np.uint64).view(np.uint8), bitorder="little")[:n].astype(bool)


def brute_coverage(B, bP, rel, lit, k, U, negatives):
    """Set membership, one Python set per label side."""
    _, vars_, _ = lit.as_tuple() if hasattr(lit, "as_tuple") else lit
    bound = [(a, v) for a, v in enumerate(vars_) if v >= 0]
    keys = {tuple(int(rel[a][t]) for a, _ in bound) for t in range(len(rel[0]))}

    def side(lo, hi):
        return {tuple(int(B[q][r]) for q in range(k)) for r in range(lo, hi)
                if tuple(int(B[v][r]) for _, v in bound) in keys}

    n = len(B[0])
    sp, sn = side(0, bP), side(bP, n)
    flags = np.array([tuple(int(U[q][i]) for q in range(k)) in sp for i in range(len(U[0]) if U else 0)],
                     dtype=bool)
    nn = 0 if negatives is None else sum(
        tuple(int(negatives[q][i]) for q in range(k)) in sn for i in range(len(negatives[0])))
    return (int(flags.sum()), nn), flags


def _synthetic():
    return golden.coverage_cases()[0]


def test_synthetic_cases_regenerate():
    for case, _, _, checksum in _synthetic():
        assert golden.coverage_case_checksum(case) == checksum


def test_oracle_matches_reference_coverage_on_synthetic_cases():
    divergent = 0
    for case, want_counts, want_flags, _ in _synthetic():
        rels, T, tP, B, bP, lit, rows, is_divergent = case
        U = [t[rows] for t in T]
        counts, bits = oracle.coverage(B, bP, rels[lit.relation], lit.as_tuple(), len(T), U,
                                       [t[tP:] for t in T])
        flags = bits_to_flags(bits, len(rows))
        if is_divergent:
            # the reference's chunk-relative row ids lose covered examples here
            divergent += 1
            assert counts != want_counts and counts[0] > want_counts[0]
            continue
        assert counts == want_counts
        np.testing.assert_array_equal(flags, want_flags)
    assert divergent == 1


def test_divergent_case_is_set_membership():
    case = [c for c, *_ in _synthetic() if c[7]][0]
    rels, T, tP, B, bP, lit, rows, _ = case
    U = [t[rows] for t in T]
    counts, bits = oracle.coverage(B, bP, rels[0], lit.as_tuple(), len(T), U, [t[tP:] for t in T])
    want_counts, want_flags = brute_coverage(B, bP, rels[0], lit, len(T), U, [t[tP:] for t in T])
    assert counts == want_counts
    np.testing.assert_array_equal(bits_to_flags(bits, len(rows)), want_flags)


def test_fixture_covers_the_edge_cases():
    syn, traced = golden.coverage_cases()
    cases = [c for c, *_ in syn]
    assert any(len(c[6]) == 0 for c in cases)                       # nothing left uncovered
    assert any(len(set(v for v in c[5].vars if v >= 0)) < sum(v >= 0 for v in c[5].vars)
               for c in cases)                                      # repeated variable
    assert any(any(v < 0 for v in c[5].vars) for c in cases)        # unbound argument
    assert {len(c[1]) for c in cases} >= {1, 2, 3}                  # target arities
    assert any(min(c[4], len(c[3][0]) - c[4]) > 32768 and not c[7] for c in cases)
    assert {t[0] for t in traced} == {"kinship", "bongard"}
    assert any(t[4][0] > 0 for t in traced) and any(t[4][0] == 0 for t in traced)


@pytest.mark.parametrize("name", ["kinship", "bongard"])
def test_oracle_matches_reference_coverage_on_learn_traces(name):
    rels, calls, _ = golden.learn_trace(name)
    target = next(c for c in calls if c[0] == "evaluate")
    T, tP = target[2], target[3]
    n = 0
    for kb, j, li, rows, want_counts, want_flags in golden.coverage_cases()[1]:
        if kb != name:
            continue
        _, _, B, bP, lits, _ = calls[j]
        lit = lits[li]
        U = [t[rows] for t in T]
        counts, bits = oracle.coverage(B, bP, rels[lit.relation], lit.as_tuple(), len(T), U,
                                       [t[tP:] for t in T])
        assert counts == want_counts, (j, li)
        np.testing.assert_array_equal(bits_to_flags(bits, len(rows)), want_flags)
        n += 1
    assert n > 10


def test_oracle_coverage_equals_brute_force():
    rng = np.random.default_rng(3)
    for trial in range(25):
        nb = int(rng.integers(2, 3000))
        dom = int(rng.integers(2, 60))
        k = int(rng.integers(1, 4))
        nc = k + int(rng.integers(0, 3))
        ar = int(rng.integers(1, 4))
        nrel = int(rng.integers(1, 2000))
        rel = [rng.integers(0, dom, nrel).astype(np.int32) for _ in range(ar)]
        B = [rng.integers(0, dom, nb).astype(np.int32) for _ in range(nc)]
        bP = int(rng.integers(0, nb + 1))
        vars_ = [int(rng.integers(-1, nc)) for _ in range(ar)]
        if all(v < 0 for v in vars_):
            vars_[0] = int(rng.integers(0, nc))
        U = [rng.integers(0, dom, 400).astype(np.int32) for _ in range(k)]
        neg = [rng.integers(0, dom, 300).astype(np.int32) for _ in range(k)]
        lit = (0, tuple(vars_), 0)
        counts, bits = oracle.coverage(B, bP, rel, lit, k, U, neg)
        want_counts, want_flags = brute_coverage(B, bP, rel, lit, k, U, neg)
        assert counts == want_counts
        np.testing.assert_array_equal(bits_to_flags(bits, 400), want_flags)


def test_oracle_coverage_without_negatives_and_invalid_literals():
    B = [np.arange(10, dtype=np.int32), np.arange(10, dtype=np.int32) % 3]
    rel = [np.array([0, 1, 2], dtype=np.int32)]
    U = [np.arange(12, dtype=np.int32)]
    counts, bits = oracle.coverage(B, 6, rel, (0, (1,), 0), 1, U, None)
    assert counts == (int(((np.arange(12) < 6)).sum()), 0)
    with pytest.raises(ValueError):
        oracle.coverage(B, 6, rel, (0, (-1,), 0), 1, U, None)      # nothing bound
    with pytest.raises(ValueError):
        oracle.coverage(B, 6, rel, (0, (0,), 0), 3, U, None)       # more target columns than bindings


@pytest.mark.parametrize("n", [0, 1, 63, 64, 65, 2047, 2048, 2049, 10000])
@pytest.mark.parametrize("keep_set", [False, True])
def test_oracle_compaction_keeps_rows_in_order(n, keep_set):
    rng = np.random.default_rng(n)
    cols = [rng.integers(-5, 5, n).astype(np.int32) for _ in range(3)]
    flags = rng.random(n) < 0.4
    bits = np.packbits(np.concatenate([flags, np.zeros((-n) % 64, bool)]), bitorder="little").view(np.uint64)
    got = oracle.compact_rows(cols, bits, keep_set=keep_set)
    keep = flags if keep_set else ~flags
    for g, c in zip(got, cols):
        np.testing.assert_array_equal(g, c[keep])


def test_compat_coverage_oracle_equals_the_reference_everywhere():
    """The oracle's restatement of the reference's own coverage procedure
    (chunk-relative projection tables, qfo_coverage_compat) equals the
    reference on every synthetic case, the divergent one included, where
    set membership does not."""
    from tests import golden
    seen_divergent = False
    for case, want_counts, want_flags, _ in golden.coverage_cases()[0]:
        rels, T, tP, B, bP, lit, rows, divergent = case
        U = [t[rows] for t in T]
        got, bits = oracle.coverage(B, bP, rels[0], lit.as_tuple(), len(T), U, [t[tP:] for t in T],
                                    compat=True)
        assert got == want_counts
        np.testing.assert_array_equal(bits_to_flags(bits, len(rows)), want_flags)
        if divergent:
            seen_divergent = True
            member, _ = oracle.coverage(B, bP, rels[0], lit.as_tuple(), len(T), U,
                                        [t[tP:] for t in T])
            assert member != want_counts
    assert seen_divergent
