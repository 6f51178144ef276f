"""CPU tests of the oracle (no GPU).

* the reference's own RadixPartition test cases
  (operations/RadixPartition_test.cpp:106-168) against the C restatement;
* FoilHashTable chain structure (storage/FoilHashTable.cpp,
  operations/BuildHashTable.cpp);
* evaluation counts against a brute-force count from the definitions,
  including the edge cases the reference cannot run (no join result at all);
* semi-joins and the label-aware extension against direct definitions.
"""
import collections

import numpy as np
import pytest

import oracle
from quickfoil_gb300 import workloads
from quickfoil_gb300.engine import Literal
from tests.brute import brute_counts

RADIX_BITS = [1, 3, 7, 12]
SIZES = [10, 20, 40, 100, 1000, 100000]


def _check_partitions(values, bits, expected):
    tuples, offsets = oracle.radix_partition(np.asarray(values, dtype=np.int32), bits)
    assert len(offsets) == (1 << bits) + 1
    for p in range(1 << bits):
        part = tuples[offsets[p]:offsets[p + 1]]
        got = collections.Counter(map(tuple, part.tolist()))
        assert got == collections.Counter(expected.get(p, [])), f"partition {p}"
        # stronger than the reference test: input order kept inside a partition
        assert np.all(np.diff(part[:, 1]) > 0)


@pytest.mark.parametrize("bits", RADIX_BITS)
@pytest.mark.parametrize("size", SIZES)
def test_radix_partition_simple(bits, size):
    # RadixPartitionTest.SimpleTests: value i lands in partition i % 2^bits.
    exp = collections.defaultdict(list)
    for i in range(size):
        exp[i % (1 << bits)].append((i, i))
    _check_partitions(np.arange(size), bits, exp)


@pytest.mark.parametrize("bits", RADIX_BITS)
@pytest.mark.parametrize("size", SIZES)
def test_radix_partition_all_zero(bits, size):
    # RadixPartitionTest.AllZero
    _check_partitions(np.zeros(size), bits, {0: [(0, i) for i in range(size)]})


@pytest.mark.parametrize("bits", RADIX_BITS)
@pytest.mark.parametrize("size", SIZES)
def test_radix_partition_zero_interleave_one(bits, size):
    # RadixPartitionTest.ZeroInterleaveOne
    vals = np.tile([0, 1], size // 2)
    exp = {0: [(0, 2 * i) for i in range(size // 2)], 1: [(1, 2 * i + 1) for i in range(size // 2)]}
    _check_partitions(vals, bits, exp)


def test_radix_partition_negative_values():
    vals = np.array([-1, -2, -3, 5, -2147483648, 2147483647], dtype=np.int32)
    tuples, offsets = oracle.radix_partition(vals, 3)
    for p in range(8):
        for v, _ in tuples[offsets[p]:offsets[p + 1]]:
            assert (np.uint32(np.int32(v).view(np.uint32)) & 7) == p


@pytest.mark.parametrize("n,bits", [(1, 3), (7, 2), (1000, 5), (4097, 4)])
def test_partition_hash_table_chains(n, bits):
    rng = np.random.default_rng(n)
    vals = rng.integers(-50, 50, n).astype(np.int32)
    tuples, offsets = oracle.radix_partition(vals, bits)
    for p in range(1 << bits):
        part = tuples[offsets[p]:offsets[p + 1]]
        if len(part) == 0:
            continue
        buckets, nxt, mask = oracle.build_partition_hash_table(part, bits)
        nb = len(buckets)
        assert nb & (nb - 1) == 0 and nb >= len(part) and nb < 2 * len(part) + 1
        assert mask == ((nb - 1) << bits) & 0xffffffff
        for b in range(nb):
            chain = []
            pos = buckets[b] - 1
            while pos >= 0:
                chain.append(pos)
                pos = nxt[pos] - 1
            want = [i for i in range(len(part))
                    if ((int(np.int32(part[i, 0]).view(np.uint32)) & mask) >> bits) == b]
            assert chain == sorted(want, reverse=True)


@pytest.mark.parametrize("seed", range(6))
def test_evaluate_matches_brute_force(seed):
    w = workloads.small_random(seed, zipf=seed % 2 == 0)
    got = oracle.evaluate(w.relations, w.binding_columns, w.num_positive,
                          [l.as_tuple() for l in w.literals], bits=5)
    want = brute_counts(w.relations, w.binding_columns, w.num_positive, w.literals)
    np.testing.assert_array_equal(got, want)


def test_evaluate_thread_count_and_bits_do_not_change_counts():
    w = workloads.small_random(11)
    lits = [l.as_tuple() for l in w.literals]
    ref = oracle.evaluate(w.relations, w.binding_columns, w.num_positive, lits, bits=1)
    for bits, th in [(5, 1), (5, 4), (9, 3)]:
        got = oracle.evaluate(w.relations, w.binding_columns, w.num_positive, lits, bits=bits,
                              nthreads=th)
        np.testing.assert_array_equal(got, ref)


def test_evaluate_edge_cases():
    rng = np.random.default_rng(0)
    B = [rng.integers(0, 10, 100).astype(np.int32) for _ in range(3)]
    rels = [[np.arange(100, 110, dtype=np.int32)],                       # disjoint: no result
            [np.array([1, 1, 1, 2], dtype=np.int32), np.array([3, 3, 4, 5], dtype=np.int32)]]
    lits = [Literal(0, (0,)), Literal(1, (1, 1)), Literal(1, (2, -1)), Literal(1, (-1, 0))]
    for P in (0, 37, 100):
        got = oracle.evaluate(rels, B, P, [l.as_tuple() for l in lits], bits=3)
        np.testing.assert_array_equal(got, brute_counts(rels, B, P, lits))
    # the reference crashes when a call has no join result at all; the oracle returns zeros
    got = oracle.evaluate(rels, B, 50, [Literal(0, (1,)).as_tuple()], bits=5)
    assert got.tolist() == [[0, 0, 0, 0]]
    # empty binding set
    E = [np.zeros(0, dtype=np.int32) for _ in range(3)]
    got = oracle.evaluate(rels, E, 0, [l.as_tuple() for l in lits], bits=5)
    assert not got.any()


def test_evaluate_rejects_bad_literals():
    B = [np.zeros(4, dtype=np.int32)]
    with pytest.raises(ValueError):
        oracle.evaluate([[np.zeros(3, dtype=np.int32)]], B, 2, [(0, [5], 0)])
    with pytest.raises(ValueError):
        oracle.evaluate([[np.zeros(3, dtype=np.int32)]], B, 2, [(1, [0], 0)])


def _brute_left(probe, build):
    s = set(zip(*[c.tolist() for c in build]))
    return np.array([t in s for t in zip(*[c.tolist() for c in probe])], dtype=bool)


def _bits_to_bool(blocks, n):
    b = np.unpackbits(blocks.view(np.uint8), bitorder="little")[:n]
    return b.astype(bool)


@pytest.mark.parametrize("k", [1, 2, 3, 6])
def test_semijoins(k):
    rng = np.random.default_rng(k)
    probe = [rng.integers(0, 6, 777).astype(np.int32) for _ in range(k)]
    build = [rng.integers(0, 6, 333).astype(np.int32) for _ in range(k)]
    bits, ones = oracle.left_semijoin(probe, build)
    want = _brute_left(probe, build)
    np.testing.assert_array_equal(_bits_to_bool(bits, 777), want)
    assert ones == want.sum()
    bits, ones = oracle.right_semijoin(probe, build)
    want = _brute_left(build, probe)
    np.testing.assert_array_equal(_bits_to_bool(bits, 333), want)
    assert ones == want.sum()


def reference_order_extension(B, P, R, lit):
    """Row order of CreateLabelAwareBindingTables written out directly:
    probe side in row order, matches on the build side in descending row
    order (chains are built by head insertion)."""
    _, vars_, _ = lit.as_tuple()
    bound = [k for k in range(len(vars_)) if vars_[k] >= 0]
    unbound = [k for k in range(len(vars_)) if vars_[k] < 0]
    n = len(B[0])
    nR = len(R[0])
    out = []
    for lo, hi in ((0, P), (P, n)):
        rows = []
        rel_probe = P < nR and (n - P) < nR
        bkey = lambda b: tuple(int(B[vars_[k]][b]) for k in bound)
        rkey = lambda r: tuple(int(R[k][r]) for k in bound)
        if rel_probe:
            for r in range(nR):
                for b in range(hi - 1, lo - 1, -1):
                    if bkey(b) == rkey(r):
                        rows.append([int(c[b]) for c in B] + [int(R[u][r]) for u in unbound])
        else:
            for b in range(lo, hi):
                for r in range(nR - 1, -1, -1):
                    if bkey(b) == rkey(r):
                        rows.append([int(c[b]) for c in B] + [int(R[u][r]) for u in unbound])
        out.append(rows)
    return out


@pytest.mark.parametrize("case", range(4))
def test_extend_bindings_reference_order(case):
    rng = np.random.default_rng(case)
    n, P = 60, 20
    B = [rng.integers(0, 5, n).astype(np.int32) for _ in range(2)]
    nR = [10, 100, 30, 15][case]
    R = [rng.integers(0, 5, nR).astype(np.int32) for _ in range(2)]
    lit = [Literal(0, (0, -1)), Literal(0, (1, 0)), Literal(0, (-1, 1)), Literal(0, (0, 0))][case]
    pos_rows, neg_rows = reference_order_extension(B, P, R, lit)
    cols = oracle.extend_bindings(B, P, R, lit.as_tuple(), len(pos_rows), len(neg_rows))
    got = np.stack(cols, axis=1).tolist() if cols and len(cols[0]) else []
    assert got == pos_rows + neg_rows
    counts = brute_counts([R], B, P, [lit])[0]
    assert (counts[2], counts[3]) == (len(pos_rows), len(neg_rows))
    with pytest.raises(ValueError):
        oracle.extend_bindings(B, P, R, lit.as_tuple(), len(pos_rows) + 1, len(neg_rows))
