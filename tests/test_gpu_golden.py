"""The GPU engine against golden fixtures produced by the reference's own code:
seeded evaluation cases, and the reference learner's kinship and Bongard-like
runs replayed call by call through the C ABI -- every Evaluate call (qfg_evaluate_group, the
drop-in for CandidateLiteralEvaluator::Evaluate), every binding-set extension
(qfg_extend_bindings, rows in the reference's order), and the reference score
of every candidate from GPU counts, with the added literal scoring best.
Identical counts at every call mean the unchanged learner, which decides from
those counts alone, makes the same choices and learns the same clauses."""
import numpy as np
import pytest

from quickfoil_gb300.engine import Literal
from tests import golden
from tests.test_golden import best_literals_by_step

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

_base = [200_000]


def _register(engine, rels):
    base = _base[0]
    _base[0] += len(rels) + 10
    for i, r in enumerate(rels):
        engine.register_relation(base + i, r)
    return base


def test_engine_matches_reference_counts(engine):
    for rels, B, P, lits, want in golden.eval_cases():
        base = _register(engine, rels)
        glits = [Literal(base + l.relation, l.vars, l.join_pos) for l in lits]
        b = engine.bindings(B, P)
        np.testing.assert_array_equal(engine.evaluate_step(b, glits), want)
        np.testing.assert_array_equal(engine.evaluate_per_literal(b, glits), want)
        b.close()


@pytest.mark.parametrize("name", ["kinship", "bongard"])
def test_learn_trace_replays_on_the_gpu(engine, name):
    rels, calls, _ = golden.learn_trace(name)
    base = _register(engine, rels)
    gpu_counts = {}
    for j, call in enumerate(calls):
        kind, key, cols, P, lits, result = call
        glits = [Literal(base + l.relation, l.vars, l.join_pos) for l in lits]
        b = engine.bindings(cols, P)
        if kind == "evaluate":
            got = engine.evaluate_group(b, key, glits)
            np.testing.assert_array_equal(got, result)
            gpu_counts[j] = got
        else:
            npos, nneg = key
            nb = engine.extend_bindings(b, glits[0], npos, nneg)
            out = nb.download()
            assert len(out) == len(result)
            for g, w in zip(out, result):
                np.testing.assert_array_equal(g, w)
            nb.close()
        b.close()
    index = {id(c): j for j, c in enumerate(calls)}
    steps = best_literals_by_step(calls, lambda ev: gpu_counts[index[id(ev)]])
    for lit, (npos, nneg), scored in steps:
        best = max(s for s, _, _ in scored)
        chosen = [s for s, l, c in scored if l == lit and c[2:] == (npos, nneg)]
        assert chosen and chosen[0] == pytest.approx(best, abs=1e-5)


def test_full_size_batched_step_matches_the_reference(engine):
    """32M x 6 bindings, 32 relations, 256 literals (199 distinct): every
    count equals the reference's own CandidateLiteralEvaluator output."""
    from quickfoil_gb300 import workloads
    lits, want, checksum = golden.batched_step_reference()
    w = workloads.batched_step()
    assert golden.input_checksum(w) == checksum
    base = _register(engine, w.relations)
    glits = [Literal(base + l.relation, l.vars, l.join_pos) for l in lits]
    b = engine.bindings(w.binding_columns, w.num_positive)
    np.testing.assert_array_equal(engine.evaluate_step(b, glits), want)
    pick = list(range(0, len(glits), 25))
    np.testing.assert_array_equal(engine.evaluate_per_literal(b, [glits[i] for i in pick]),
                                  want[pick])
    b.close()
    for i in range(len(w.relations)):
        engine.release_relation(base + i)
