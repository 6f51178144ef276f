"""GPU parity: every CUDA path through the C ABI against the oracle, bit-exact.

Integer work throughout, so the tolerance is zero: counts, partition tuples,
offsets and hash-table arrays must be identical to the oracle's.
"""
import numpy as np
import pytest

import oracle
from quickfoil_gb300 import workloads
from quickfoil_gb300.engine import Literal
from tests.brute import brute_counts

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).cuda()


# --- RadixPartition ---------------------------------------------------------

@pytest.mark.parametrize("bits", [1, 3, 5, 7, 12, 15])
@pytest.mark.parametrize("kind", ["identity", "zero", "zero_one", "random"])
@pytest.mark.parametrize("size", [0, 1, 10, 1000, 100000, 1 << 20])
def test_radix_partition_exact(engine, bits, kind, size):
    rng = np.random.default_rng(size + bits)
    vals = {"identity": np.arange(size), "zero": np.zeros(size),
            "zero_one": np.tile([0, 1], size // 2 + 1)[:size],
            "random": rng.integers(-2**31, 2**31, size)}[kind].astype(np.int32)
    tuples, offsets = engine.radix_partition(dev(vals), bits)
    want_t, want_o = oracle.radix_partition(vals, bits)
    np.testing.assert_array_equal(offsets.cpu().numpy(), want_o)
    np.testing.assert_array_equal(tuples.cpu().numpy().reshape(-1, 2), want_t.reshape(-1, 2))


@pytest.mark.parametrize("n,bits", [(1, 1), (5, 3), (1000, 5), (300000, 5), (200000, 12)])
def test_build_hash_table_on_partitions_exact(engine, n, bits):
    rng = np.random.default_rng(n)
    vals = rng.integers(-1000, 1000, n).astype(np.int32)
    tuples, offsets = engine.radix_partition(dev(vals), bits)
    buckets, boff, masks, nxt = engine.build_hash_table_on_partitions(tuples, offsets, bits)
    buckets, boff = buckets.cpu().numpy(), boff.cpu().numpy()
    masks, nxt = masks.cpu().numpy().view(np.uint32), nxt.cpu().numpy()
    want_t, want_o = oracle.radix_partition(vals, bits)
    for p in range(1 << bits):
        part = want_t[want_o[p]:want_o[p + 1]]
        if len(part) == 0:
            assert masks[p] == 0 and boff[p + 1] == boff[p]
            continue
        wb, wn, wm = oracle.build_partition_hash_table(part, bits)
        assert masks[p] == wm
        np.testing.assert_array_equal(buckets[boff[p]:boff[p + 1]], wb)
        np.testing.assert_array_equal(nxt[want_o[p]:want_o[p + 1]], wn)


@pytest.mark.parametrize("k,n", [(1, 1), (1, 5000), (2, 70000), (3, 1000), (6, 2000)])
def test_build_hash_table_on_table_exact(engine, k, n):
    rng = np.random.default_rng(k * n)
    keys = [rng.integers(-20, 20, n).astype(np.int32) for _ in range(k)]
    buckets, nxt, mask = engine.build_hash_table_on_table([dev(c) for c in keys])
    wb, wn, wm = oracle.build_table_hash_table(keys)
    assert mask == wm
    np.testing.assert_array_equal(buckets.cpu().numpy(), wb)
    np.testing.assert_array_equal(nxt.cpu().numpy(), wn)


# --- candidate-literal evaluation ---------------------------------------------

def _register(engine, w, base_id):
    for rid, cols in enumerate(w.relations):
        engine.register_relation(base_id + rid, cols)
    return [Literal(base_id + l.relation, l.vars, l.join_pos) for l in w.literals]


_next_id = [1000]


def fresh_ids(n):
    base = _next_id[0]
    _next_id[0] += n + 10
    return base


@pytest.mark.parametrize("seed", range(8))
def test_evaluate_small_random(engine, seed):
    w = workloads.small_random(seed, zipf=seed % 2 == 0)
    base = fresh_ids(len(w.relations))
    lits = _register(engine, w, base)
    b = engine.bindings(w.binding_columns, w.num_positive)
    want = oracle.evaluate(w.relations, w.binding_columns, w.num_positive,
                           [l.as_tuple() for l in w.literals], bits=5)
    np.testing.assert_array_equal(engine.evaluate_step(b, lits), want)
    np.testing.assert_array_equal(engine.evaluate_per_literal(b, lits), want)
    b.close()


def test_evaluate_edge_cases(engine):
    rng = np.random.default_rng(0)
    B = [rng.integers(0, 10, 100).astype(np.int32) for _ in range(3)]
    rels = [[np.arange(100, 110, dtype=np.int32)],
            [np.array([1, 1, 1, 2], dtype=np.int32), np.array([3, 3, 4, 5], dtype=np.int32)],
            [np.zeros(0, dtype=np.int32), np.zeros(0, dtype=np.int32)]]
    base = fresh_ids(len(rels))
    for i, r in enumerate(rels):
        engine.register_relation(base + i, r)
    lits = [Literal(0, (0,)), Literal(1, (1, 1)), Literal(1, (2, -1)), Literal(1, (-1, 0)),
            Literal(2, (0, 1)), Literal(1, (0, 0))]
    glits = [Literal(base + l.relation, l.vars, l.join_pos) for l in lits]
    for P in (0, 37, 100):
        b = engine.bindings(B, P)
        want = brute_counts(rels, B, P, lits)
        np.testing.assert_array_equal(engine.evaluate_step(b, glits), want)
        np.testing.assert_array_equal(engine.evaluate_per_literal(b, glits), want)
        b.close()
    E = engine.bindings([np.zeros(0, dtype=np.int32)] * 3, 0)
    assert not engine.evaluate_step(E, glits).any()
    assert not engine.evaluate_per_literal(E, glits).any()
    assert engine.evaluate_step(E, []).shape == (0, 4)


def test_evaluate_group_and_evaluator_order(engine):
    from quickfoil_gb300 import CandidateLiteralEvaluator
    w = workloads.small_random(42)
    base = fresh_ids(len(w.relations))
    lits = _register(engine, w, base)
    b = engine.bindings(w.binding_columns, w.num_positive)
    j = lits[0].vars[lits[0].join_pos]
    group = [l for l in lits if l.vars[l.join_pos] == j]
    by_pred = {}
    for l in group:
        by_pred.setdefault(l.relation, []).append(l)
    infos = CandidateLiteralEvaluator(engine, b).Evaluate(j, by_pred)
    ordered = [l for ls in by_pred.values() for l in ls]
    assert [i.literal for i in infos] == ordered
    want = brute_counts([None] * base + w.relations, w.binding_columns, w.num_positive, ordered)
    np.testing.assert_array_equal(np.array([i.counts() for i in infos]), want)
    with pytest.raises(Exception):
        engine.evaluate_group(b, j + 1 if j + 1 < len(w.binding_columns) else j - 1, group)


def test_split_binding_layout(engine):
    w = workloads.small_random(7)
    base = fresh_ids(len(w.relations))
    lits = _register(engine, w, base)
    P = w.num_positive
    b1 = engine.bindings(w.binding_columns, P)
    b2 = engine.bindings_split([c[:P] for c in w.binding_columns], [c[P:] for c in w.binding_columns])
    np.testing.assert_array_equal(engine.evaluate_step(b1, lits), engine.evaluate_step(b2, lits))
    got = b2.download()
    for g, c in zip(got, w.binding_columns):
        np.testing.assert_array_equal(g, c)


def test_invalid_literals_are_rejected(engine):
    from quickfoil_gb300 import QfgError
    base = fresh_ids(1)
    engine.register_relation(base, [np.arange(10, dtype=np.int32)] * 2)
    b = engine.bindings([np.arange(5, dtype=np.int32)], 2)
    for bad in (Literal(base, (0, 3), 0), Literal(base + 5, (0, 0), 0), Literal(base, (0,), 0),
                Literal(base, (-1, 0), 0)):
        with pytest.raises(QfgError):
            engine.evaluate_step(b, [bad])


def test_medium_batched_equals_oracle(engine):
    w = workloads.batched_step(n_bindings=400_000, num_relations=12, min_tuples=100,
                               max_tuples=300_000, num_literals=64, domain=50_000, seed=9)
    base = fresh_ids(len(w.relations))
    lits = _register(engine, w, base)
    b = engine.bindings(w.binding_columns, w.num_positive)
    want = oracle.evaluate(w.relations, w.binding_columns, w.num_positive,
                           [l.as_tuple() for l in w.literals], bits=8, nthreads=8)
    np.testing.assert_array_equal(engine.evaluate_step(b, lits), want)
    np.testing.assert_array_equal(engine.evaluate_per_literal(b, lits), want)


@pytest.mark.parametrize("zipf", [False, True])
def test_single_literal_full_size(engine, zipf):
    """16M x 4 bindings, 4M-tuple relation: closed-form counts (bincount)."""
    w = workloads.single_literal(zipf=zipf)
    base = fresh_ids(1)
    lits = _register(engine, w, base)
    b = engine.bindings([dev(c) for c in w.binding_columns], w.num_positive)
    A = w.relations[0][0]
    cnt = np.bincount(A, minlength=w.domain).astype(np.int64)
    m = cnt[w.binding_columns[2]]
    P = w.num_positive
    want = np.array([[np.count_nonzero(m[:P]), np.count_nonzero(m[P:]), m[:P].sum(), m[P:].sum()]])
    np.testing.assert_array_equal(engine.evaluate_step(b, lits), want)
    np.testing.assert_array_equal(engine.evaluate_per_literal(b, lits), want)


@pytest.mark.parametrize("bits", [1, 3, 8, 9, 12, 14])
def test_evaluate_partition_bits_do_not_change_counts(engine, bits):
    """Single-pass (<= 8 bits) and two-pass binding partitions, tiled and
    untiled work items: identical counts."""
    from quickfoil_gb300 import _capi as C
    w = workloads.batched_step(n_bindings=300_000, num_relations=8, min_tuples=50,
                               max_tuples=200_000, num_literals=48, domain=20_000, seed=21)
    base = fresh_ids(len(w.relations))
    lits = _register(engine, w, base)
    b = engine.bindings(w.binding_columns, w.num_positive)
    want = brute_counts([None] * base + w.relations, w.binding_columns, w.num_positive, lits)
    try:
        engine.set_option(C.QFG_OPT_EVAL_BITS, bits)
        np.testing.assert_array_equal(engine.evaluate_step(b, lits), want)
    finally:
        engine.set_option(C.QFG_OPT_EVAL_BITS, 0)


@pytest.mark.parametrize("bits,pass1", [(12, 3), (12, 8), (14, 5), (14, 8), (16, 7), (16, 8)])
def test_evaluate_pass_split_does_not_change_counts(engine, bits, pass1):
    """The same partition bits split differently between the two passes
    (pass-1 bits; pass 2 takes the rest): identical counts."""
    from quickfoil_gb300 import _capi as C
    w = workloads.batched_step(n_bindings=300_000, num_relations=8, min_tuples=50,
                               max_tuples=200_000, num_literals=48, domain=20_000, seed=22)
    base = fresh_ids(len(w.relations))
    lits = _register(engine, w, base)
    b = engine.bindings(w.binding_columns, w.num_positive)
    want = brute_counts([None] * base + w.relations, w.binding_columns, w.num_positive, lits)
    try:
        engine.set_option(C.QFG_OPT_EVAL_BITS, bits)
        engine.set_option(C.QFG_OPT_PASS1_BITS, pass1)
        np.testing.assert_array_equal(engine.evaluate_step(b, lits), want)
    finally:
        engine.set_option(C.QFG_OPT_EVAL_BITS, 0)
        engine.set_option(C.QFG_OPT_PASS1_BITS, 0)


@pytest.mark.parametrize("offset", [0, 1, 3])
def test_partition_rounds_wide_and_unaligned(engine, offset):
    """5M binding rows: every partition CTA streams several 16K-row rounds.
    One literal group carries all eight columns (a literal binding every
    argument of an 8-ary relation), the label boundary is not a multiple of
    4 rows, and the binding columns are borrowed from device memory at an
    element offset (1 and 3: not 16-byte aligned, so every round is copied
    4 bytes at a time).  Counts equal the oracle's at the automatic, a
    small single-pass-adjacent and the widest partition settings."""
    from quickfoil_gb300 import _capi as C
    rng = np.random.default_rng(31 + offset)
    n, P, dom = 5_000_003, 1_234_567, 48
    B = [rng.integers(0, dom, n, dtype=np.int32) for _ in range(8)]
    B[0] = rng.integers(0, 300_000, n, dtype=np.int32)
    pick = rng.choice(n, 600_000, replace=False)
    noise = 80_000
    R8 = [np.concatenate([c[pick], rng.integers(0, dom, noise, dtype=np.int32)]) for c in B]
    R8[0][-noise:] = rng.integers(0, 300_000, noise, dtype=np.int32)
    R3 = [rng.integers(0, 300_000, 400_000, dtype=np.int32),
          rng.integers(0, dom, 400_000, dtype=np.int32),
          rng.integers(0, dom, 400_000, dtype=np.int32)]
    rels = [R8, R3]
    spec = [(0, list(range(8)), 0), (0, [0, 1, 2, -1, -1, -1, -1, 7], 0),
            (1, [0, 3, -1], 0), (1, [0, -1, 5], 0), (1, [0, -1, -1], 0)]
    want = oracle.evaluate(rels, B, P, spec, bits=8, nthreads=8)
    assert want[0, 0] > 0 and want[0, 1] > 0  # the 8-column literal covers rows of both labels
    base = fresh_ids(len(rels))
    for i, r in enumerate(rels):
        engine.register_relation(base + i, r)
    lits = [Literal(base + r, tuple(v), j) for r, v, j in spec]
    cols = []
    for c in B:
        t = torch.zeros(n + offset, dtype=torch.int32, device="cuda")
        t[offset:] = torch.from_numpy(c).cuda()
        cols.append(t[offset:])
    assert all((c.data_ptr() % 16 == 0) == (offset == 0) for c in cols)
    b = engine.bindings(cols, P)
    try:
        for bits, pass1 in ((0, 0), (9, 0), (16, 7)):
            engine.set_option(C.QFG_OPT_EVAL_BITS, bits)
            engine.set_option(C.QFG_OPT_PASS1_BITS, pass1)
            np.testing.assert_array_equal(engine.evaluate_step(b, lits), want)
    finally:
        engine.set_option(C.QFG_OPT_EVAL_BITS, 0)
        engine.set_option(C.QFG_OPT_PASS1_BITS, 0)
