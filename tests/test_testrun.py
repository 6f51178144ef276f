"""The test runner of learnt clauses (QuickFoilTestRunner::RunTest) on the
oracle: against the reference's own test runner (golden fixture: learnt
clauses of the kinship and Bongard tasks on mixed held-out test tables),
and the clause parser."""
import numpy as np

import oracle
from quickfoil_gb300 import workloads
from quickfoil_gb300.engine import Literal, parse_clause
from tests import golden


def _relations(name):
    return golden.learn_trace(name)[0]


def test_parse_clause_numbers_columns_as_the_binding_tables_grow():
    arity, body = parse_clause("target(0, 1) :-  r1(0), r3(2, 0), r0(2, 1)")
    assert arity == 2
    assert body == [Literal(1, (0,)), Literal(3, (-1, 0)), Literal(0, (2, 1))]
    arity, body = parse_clause("target(0) :-  r0(0, 1), r1(1), r4(1, 2), r2(2)")
    assert arity == 1
    assert body == [Literal(0, (0, -1)), Literal(1, (1,)), Literal(4, (1, -1)), Literal(2, (2,))]


def test_oracle_test_runner_matches_reference():
    runs = golden.test_runs()
    assert {r[0] for r in runs} == {"kinship", "bongard"}
    for name, clauses, tpos, tneg, want in runs:
        rels = _relations(name)
        parsed = [[(l.relation, l.vars) for l in parse_clause(c)[1]] for c in clauses]
        got = tuple(len(oracle.run_test(rels, parsed, t)[0]) for t in (tpos, tneg))
        assert got == want, name
        assert 0 < want[0] < len(tpos[0])  # neither all covered nor none


def test_oracle_test_runner_keeps_row_order_and_applies_clauses_in_turn():
    rels = _relations("kinship")
    clause = [(l.relation, l.vars) for l in
              parse_clause("target(0, 1) :-  r1(0), r3(2, 0), r0(2, 1)")[1]]
    t = workloads.kinship(seed=1, max_positive=10 ** 6, num_negative=300)
    test = t.target_columns
    left = oracle.run_test(rels, [clause], test)
    # every kept row is a row of the test table, in the same order
    idx = {(int(a), int(b)): i for i, (a, b) in enumerate(zip(*test))}
    order = [idx[(int(a), int(b))] for a, b in zip(*left)]
    assert order == sorted(order)
    assert len(left[0]) == 300
    # a second copy of the clause removes nothing more; an empty clause list nothing at all
    again = oracle.run_test(rels, [clause, clause], test)
    assert all(np.array_equal(a, b) for a, b in zip(again, left))
    assert all(np.array_equal(a, b) for a, b in zip(oracle.run_test(rels, [], test), test))
