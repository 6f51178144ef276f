"""The streamed evaluation mode (QFG_OPT_EVAL_MODE = 2: relation entries in a
shared-memory key table, binding rows streamed past it) against the oracle,
brute force and the reference's own counts, bit-exact (integer counts,
tolerance 0): small random cases with Zipf keys, the edge cases (empty
relation, P = 0 and P = n, repeated variables, literals whose further
arguments repeat the join variable), a medium step, a sweep of partition
bits and bits offsets, and the full-size 32M x 6 step against the
reference."""
import numpy as np
import pytest

import oracle
from quickfoil_gb300 import workloads
from quickfoil_gb300 import _capi as C
from quickfoil_gb300.engine import Literal
from tests import golden
from tests.brute import brute_counts

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

_next = [700_000]


def _register(engine, rels):
    base = _next[0]
    _next[0] += len(rels) + 10
    for i, r in enumerate(rels):
        engine.register_relation(base + i, r)
    return base


@pytest.fixture
def streamed(engine):
    engine.set_option(C.QFG_OPT_EVAL_MODE, 2)
    yield engine
    engine.set_option(C.QFG_OPT_EVAL_MODE, 0)
    engine.set_option(C.QFG_OPT_EVAL_BITS, 0)


@pytest.mark.parametrize("seed", range(6))
def test_streamed_small_random(streamed, seed):
    w = workloads.small_random(seed + 100, zipf=seed % 2 == 0, n_bindings=5000, num_literals=40)
    base = _register(streamed, w.relations)
    lits = [Literal(base + l.relation, l.vars, l.join_pos) for l in w.literals]
    b = streamed.bindings(w.binding_columns, w.num_positive)
    want = oracle.evaluate(w.relations, w.binding_columns, w.num_positive,
                           [l.as_tuple() for l in w.literals], bits=5)
    np.testing.assert_array_equal(streamed.evaluate_step(b, lits), want)
    b.close()


def test_streamed_edge_cases(streamed):
    rng = np.random.default_rng(1)
    B = [rng.integers(0, 10, 300).astype(np.int32) for _ in range(3)]
    rels = [[np.arange(100, 110, dtype=np.int32)],
            [np.array([1, 1, 1, 2, 3], dtype=np.int32), np.array([3, 3, 4, 5, 3], dtype=np.int32)],
            [np.zeros(0, dtype=np.int32), np.zeros(0, dtype=np.int32)],
            [rng.integers(0, 10, 50).astype(np.int32) for _ in range(3)]]
    base = _register(streamed, rels)
    lits = [Literal(0, (0,)), Literal(1, (1, 1)), Literal(1, (2, -1)), Literal(1, (-1, 0)),
            Literal(2, (0, 1)), Literal(1, (0, 0)), Literal(3, (0, 1, 1)), Literal(3, (0, 0, 2)),
            Literal(3, (2, 1, 0)), Literal(3, (1, -1, 1))]
    glits = [Literal(base + l.relation, l.vars, l.join_pos) for l in lits]
    for P in (0, 111, 300):
        b = streamed.bindings(B, P)
        np.testing.assert_array_equal(streamed.evaluate_step(b, glits), brute_counts(rels, B, P, lits))
        b.close()


def test_streamed_medium_step(streamed):
    w = workloads.batched_step(n_bindings=400_000, num_relations=12, min_tuples=100,
                               max_tuples=300_000, num_literals=64, domain=50_000, seed=9)
    base = _register(streamed, w.relations)
    lits = [Literal(base + l.relation, l.vars, l.join_pos) for l in w.literals]
    b = streamed.bindings(w.binding_columns, w.num_positive)
    want = oracle.evaluate(w.relations, w.binding_columns, w.num_positive,
                           [l.as_tuple() for l in w.literals], bits=8, nthreads=8)
    np.testing.assert_array_equal(streamed.evaluate_step(b, lits), want)
    b.close()


@pytest.mark.parametrize("bits", [0, 1, 6, 9, 13, 16])
def test_streamed_partition_bits_do_not_change_counts(streamed, bits):
    w = workloads.batched_step(n_bindings=300_000, num_relations=8, min_tuples=50,
                               max_tuples=200_000, num_literals=48, domain=20_000, seed=21)
    base = _register(streamed, w.relations)
    lits = [Literal(base + l.relation, l.vars, l.join_pos) for l in w.literals]
    b = streamed.bindings(w.binding_columns, w.num_positive)
    want = brute_counts([None] * base + w.relations, w.binding_columns, w.num_positive, lits)
    streamed.set_option(C.QFG_OPT_EVAL_BITS, bits)
    np.testing.assert_array_equal(streamed.evaluate_step(b, lits), want)
    b.close()


def test_streamed_full_size_step_matches_the_reference(streamed):
    lits, want, checksum = golden.batched_step_reference()
    w = workloads.batched_step()
    assert golden.input_checksum(w) == checksum
    base = _register(streamed, w.relations)
    glits = [Literal(base + l.relation, l.vars, l.join_pos) for l in lits]
    b = streamed.bindings(w.binding_columns, w.num_positive)
    np.testing.assert_array_equal(streamed.evaluate_step(b, glits), want)
    b.close()
    for i in range(len(w.relations)):
        streamed.release_relation(base + i)


def test_autotuner_records_a_mode(engine):
    w = workloads.batched_step(n_bindings=200_000, num_relations=6, min_tuples=100,
                               max_tuples=50_000, num_literals=24, domain=10_000, seed=31)
    base = _register(engine, w.relations)
    lits = [Literal(base + l.relation, l.vars, l.join_pos) for l in w.literals]
    b = engine.bindings(w.binding_columns, w.num_positive)
    want = engine.evaluate_step(b, lits)
    engine.autotune_step(b, lits)
    choice = engine.autotune_choice(200_000)
    assert choice["mode"] in ("tiled", "streamed")
    engine.set_option(C.QFG_OPT_AUTOTUNE, 1)
    try:
        np.testing.assert_array_equal(engine.evaluate_step(b, lits), want)
    finally:
        engine.set_option(C.QFG_OPT_AUTOTUNE, 0)
    b.close()
