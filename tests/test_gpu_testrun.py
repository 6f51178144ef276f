"""qfg_run_test (the device test runner, the drop-in for
QuickFoilTestRunner::RunTest) against the reference's own test runner
(golden fixture) and against the oracle's restatement on seeded clause
lists: uncovered counts and the uncovered rows in order."""
import numpy as np
import pytest

import oracle
from quickfoil_gb300 import workloads
from quickfoil_gb300.engine import Literal, parse_clause
from tests import golden

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

_ids = [1_200_000]


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).cuda()


def _register(engine, rels):
    base = _ids[0]
    _ids[0] += len(rels) + 10
    for i, r in enumerate(rels):
        engine.register_relation(base + i, r)
    return base


def _shift(clauses, base):
    return [[Literal(base + l.relation, l.vars) for l in body] for body in clauses]


def test_test_runner_matches_reference(engine):
    for name, clauses, tpos, tneg, want in golden.test_runs():
        rels = golden.learn_trace(name)[0]
        base = _register(engine, rels)
        parsed = [parse_clause(c)[1] for c in clauses]
        got = []
        for t in (tpos, tneg):
            n, rows = engine.run_test(_shift(parsed, base), [dev(c) for c in t], rows=True)
            want_rows = oracle.run_test(rels, [[(l.relation, l.vars) for l in b] for b in parsed], t)
            for g, w in zip(rows, want_rows):
                np.testing.assert_array_equal(g.cpu().numpy(), w)
            got.append(n)
        assert tuple(got) == want, name


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_test_runner_matches_oracle_on_random_clause_lists(engine, seed):
    """Clause lists of 1-3 clauses, each 1-3 body literals whose arguments
    bind test columns or the columns earlier literals introduced."""
    rng = np.random.default_rng(seed)
    w = workloads.small_random(seed, n_bindings=4000, ncols=2, max_tuples=3000, domain=60)
    rels = w.relations
    base = _register(engine, rels)
    test = [rng.integers(0, 60, 1500).astype(np.int32) for _ in range(2)]
    clauses = []
    for _ in range(int(rng.integers(1, 4))):
        body, ncols = [], 2
        for _ in range(int(rng.integers(1, 4))):
            r = int(rng.integers(0, len(rels)))
            vars_ = [int(rng.integers(0, ncols)) if rng.random() < 0.6 else -1
                     for _ in range(len(rels[r]))]
            if all(v < 0 for v in vars_):
                vars_[0] = int(rng.integers(0, ncols))
            body.append(Literal(r, tuple(vars_)))
            ncols += sum(1 for v in vars_ if v < 0)
        clauses.append(body)
    want = oracle.run_test(rels, [[(l.relation, l.vars) for l in b] for b in clauses], test)
    n, rows = engine.run_test(_shift(clauses, base), [dev(c) for c in test], rows=True)
    assert n == len(want[0])
    for g, wcol in zip(rows, want):
        np.testing.assert_array_equal(g.cpu().numpy(), wcol)


def test_test_runner_edge_cases(engine):
    rels = [[np.array([1, 2, 3], np.int32), np.array([4, 5, 6], np.int32)],
            [np.array([7], np.int32)]]
    base = _register(engine, rels)
    test = [np.array([1, 2, 9, 3], np.int32)]
    covers = [Literal(base, (0, -1))]                      # rows 1, 2, 3 covered
    nothing = [Literal(base + 1, (0,))]                    # covers none
    dead = [Literal(base, (0, -1)), Literal(base + 1, (1,))]  # extension then nothing
    assert engine.run_test([covers], [dev(test[0])]) == 1
    assert engine.run_test([nothing, dead], [dev(test[0])]) == 4
    assert engine.run_test([], [dev(test[0])]) == 4
    assert engine.run_test([covers], [dev(np.zeros(0, np.int32))]) == 0
