"""The oracle against golden fixtures produced by the reference's own code
(tests/golden/make_golden.py): evaluation counts of seeded cases, and a full
replay of the reference learner's kinship and Bongard-like runs (every Evaluate call's counts,
every binding-set extension's rows in order, the score of every candidate and
the choice of the literal that was added)."""
import numpy as np
import pytest

import oracle
from quickfoil_gb300.scoring import literal_score
from tests import golden


def test_oracle_matches_reference_counts():
    for rels, B, P, lits, want in golden.eval_cases():
        got = oracle.evaluate(rels, B, P, [l.as_tuple() for l in lits], bits=5)
        np.testing.assert_array_equal(got, want)


def test_fixture_covers_the_edge_cases():
    cases = golden.eval_cases()
    Ps = {P for _, B, P, _, _ in cases}
    assert 0 in Ps
    assert any(P == len(B[0]) for _, B, P, _, _ in cases)
    assert any(not want.any() for *_, want in cases)  # a call without any join result
    assert any(len(l.vars) == 3 and sum(v >= 0 for v in l.vars) == 3
               for _, _, _, lits, _ in cases for l in lits)


def test_batched_step_fixture_matches_the_workload_generator():
    """The full-size batched step regenerates bit for bit (checksums of every
    column), and the oracle reproduces the reference's counts on a sample of
    its literals."""
    from quickfoil_gb300 import workloads
    lits, want, checksum = golden.batched_step_reference()
    w = workloads.batched_step()
    assert golden.input_checksum(w) == checksum
    assert list(dict.fromkeys(w.literals)) == lits
    pick = [i for i in range(len(lits)) if want[i].any()][:4] + \
           [i for i in range(len(lits)) if not want[i].any()][:1]
    got = oracle.evaluate(w.relations, w.binding_columns, w.num_positive,
                          [lits[i].as_tuple() for i in pick], bits=5)
    np.testing.assert_array_equal(got, want[pick])


def test_kinship_learns_the_planted_rule():
    _, _, clauses = golden.kinship()
    # uncle(X, Y) :- male(X), sibling(Z, X), parent(Z, Y)
    assert clauses == ["target(0, 1) :-  r1(0), r3(2, 0), r0(2, 1)"]


def test_bongard_learns_the_planted_rule():
    _, calls, clauses = golden.bongard()
    # pos(P) :- element(P, A), circle(A), inside(A, B), triangle(B)
    assert clauses == ["target(0) :-  r0(0, 1), r1(1), r4(1, 2), r2(2)"]
    assert sum(c[0] == "extend" for c in calls) == 3


def best_literals_by_step(calls, counts_of):
    """For every extension, the candidates evaluated on the same binding set
    before it, scored with the reference formula from counts_of(call)."""
    out = []
    pending = []
    for call in calls:
        if call[0] == "evaluate":
            pending.append(call)
        else:
            _, (npos, nneg), cols, P, (lit,), _ = call
            N = len(cols[0]) - P
            scored = []
            for ev in pending:
                for l, c in zip(ev[4], counts_of(ev)):
                    s = literal_score(c, P, N)
                    if s is not None:
                        scored.append((s, l, tuple(int(v) for v in c)))
            out.append((lit, (npos, nneg), scored))
            pending = []
    return out


@pytest.mark.parametrize("name", ["kinship", "bongard"])
def test_learn_trace_replays_on_the_oracle(name):
    rels, calls, _ = golden.learn_trace(name)
    o = oracle.Oracle(rels)
    for call in calls:
        kind, key, cols, P, lits, result = call
        if kind == "evaluate":
            got = o.evaluate(cols, P, [l.as_tuple() for l in lits], bits=5)
            np.testing.assert_array_equal(got, result)
        else:
            npos, nneg = key
            rel = rels[lits[0].relation]
            got = oracle.extend_bindings(cols, P, rel, lits[0].as_tuple(), npos, nneg)
            assert len(got) == len(result)
            for g, w in zip(got, result):
                np.testing.assert_array_equal(g, w)
    o.close()


@pytest.mark.parametrize("name", ["kinship", "bongard"])
def test_added_literals_have_the_best_reference_score(name):
    _, calls, _ = golden.learn_trace(name)
    steps = best_literals_by_step(calls, lambda ev: ev[5])
    assert steps
    for lit, (npos, nneg), scored in steps:
        best = max(s for s, _, _ in scored)
        chosen = [s for s, l, c in scored if l == lit and c[2:] == (npos, nneg)]
        assert chosen and chosen[0] == pytest.approx(best, abs=1e-5)


def test_oracle_after_semijoin_table_matches_the_reference():
    """BuildHashTableAfterSemiJoin restated (qf_oracle.c) against the
    reference's own tables: one chunk, 32768-row chunks with chunk-relative
    positions, short chunks, no or all bits set, seven keys."""
    cases = golden.after_semijoin_cases()
    assert any(chunk and len(keys[0]) > chunk for keys, _, chunk, *_ in cases)
    for keys, bits, chunk, nbt, want_b, want_n, want_m in cases:
        b, nx, m = oracle.build_hash_table_after_semijoin(keys, bits, chunk, nbt)
        assert m == want_m
        np.testing.assert_array_equal(b, want_b)
        np.testing.assert_array_equal(oracle.reachable_next(b, nx), want_n)
