"""Graph replay and the serving loop against the direct batched step.

Integer counts, tolerance zero: a replayed graph, and a request served among
others, give exactly the counts of qfg_evaluate_step on the same inputs (and
those equal the oracle's)."""
import numpy as np
import pytest

import oracle
from quickfoil_gb300 import workloads
from quickfoil_gb300._capi import QFG_ERR_BUDGET, QfgError
from quickfoil_gb300.engine import Literal

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

_base = [500_000]


def _register(engine, w):
    base = _base[0]
    _base[0] += len(w.relations) + 10
    for i, r in enumerate(w.relations):
        engine.register_relation(base + i, r)
    return [Literal(base + l.relation, l.vars, l.join_pos) for l in dict.fromkeys(w.literals)]


def _dev_columns(cols):
    return [torch.from_numpy(np.ascontiguousarray(c, dtype=np.int32)).cuda() for c in cols]


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_graph_replay_equals_step_and_follows_refilled_bindings(engine, seed):
    w = workloads.small_random(seed, n_bindings=20000, max_tuples=5000, num_literals=40)
    lits = _register(engine, w)
    cols = _dev_columns(w.binding_columns)
    b = engine.bindings(cols, w.num_positive)
    counts = torch.zeros((len(lits), 4), dtype=torch.int64, device="cuda")
    want = engine.evaluate_step(b, lits)
    g = engine.step_graph(b, lits, counts.data_ptr())
    for _ in range(3):  # replays are idempotent: counts are re-zeroed inside
        g.launch()
        engine.synchronize()
        np.testing.assert_array_equal(counts.cpu().numpy(), want)
    # same binding set, new contents: the replay evaluates the new data
    rng = np.random.default_rng(100 + seed)
    new_cols = [rng.permutation(c) for c in w.binding_columns]
    torch.cuda.synchronize()
    for c, n in zip(cols, new_cols):
        c.copy_(torch.from_numpy(n))
    torch.cuda.synchronize()
    g.launch()
    engine.synchronize()
    b2 = engine.bindings([n for n in new_cols], w.num_positive)
    np.testing.assert_array_equal(counts.cpu().numpy(), engine.evaluate_step(b2, lits))
    g.close()
    b2.close()
    b.close()


def test_graph_of_an_empty_step(engine):
    b = engine.bindings([np.arange(10, dtype=np.int32)], 5)
    g = engine.step_graph(b, [], 0)
    g.launch()
    engine.synchronize()
    g.close()
    b.close()


def _requests(engine, seeds, sizes):
    reqs = []
    for seed, n in zip(seeds, sizes):
        w = workloads.small_random(seed, n_bindings=n, max_tuples=4000, num_literals=30)
        lits = _register(engine, w)
        b = engine.bindings(_dev_columns(w.binding_columns), w.num_positive)
        reqs.append((w, b, lits, engine.evaluate_step(b, lits)))
    return reqs


@pytest.mark.parametrize("slots,depth", [(1, 1), (3, 1), (8, 1), (1, 2), (2, 3)])
def test_served_requests_equal_direct_steps(engine, slots, depth):
    reqs = _requests(engine, range(10, 22), [500, 200000, 3000, 70000, 1, 40000, 9000, 120000,
                                             2500, 60000, 800, 30000])
    # the oracle pins the direct counts of two of them
    for w, b, lits, want in reqs[:2]:
        base = lits[0].relation - next(iter(dict.fromkeys(w.literals))).relation
        got = oracle.evaluate(w.relations, w.binding_columns, w.num_positive,
                              [(l.relation - base, l.vars, l.join_pos) for l in lits], bits=5)
        np.testing.assert_array_equal(want, got)
    srv = engine.server(slots=slots, depth=depth)
    ids = [srv.submit(b, lits) for _, b, lits, _ in reqs]
    seen = srv.poll()
    srv.result(ids[len(ids) // 2])
    seen += srv.poll()
    srv.drain()
    seen += srv.poll()
    assert sorted(seen) == sorted(ids)
    for rid, (_, _, _, want) in zip(ids, reqs):
        np.testing.assert_array_equal(srv.result(rid), want)
    st = srv.stats()
    assert st["completed"] == len(ids)
    assert 0 < st["p50_ms"] <= st["p99_ms"]
    assert 1 <= st["peak_in_flight"] <= slots * depth
    if slots * depth > 1:
        assert st["peak_in_flight"] > 1
    srv.close()
    for _, b, _, _ in reqs:
        b.close()


def test_server_refuses_a_request_over_its_budget(engine):
    (w, b, lits, want), = _requests(engine, [30], [50000])
    srv = engine.server(slots=2, hbm_budget=1)
    rid = srv.submit(b, lits)
    with pytest.raises(QfgError) as e:
        srv.result(rid)
    assert e.value.status == QFG_ERR_BUDGET
    assert rid in srv.poll()
    srv.close()
    # the engine itself is unaffected
    np.testing.assert_array_equal(engine.evaluate_step(b, lits), want)
    b.close()


def test_server_budget_serialises_requests(engine):
    reqs = _requests(engine, [40, 40, 40, 40], [100000, 100000, 100000, 100000])
    # a budget that fits one request's scratch but not two
    one = engine.step_scratch_bytes(reqs[0][1], reqs[0][2])
    srv = engine.server(slots=4, hbm_budget=int(one * 1.5))
    ids = [srv.submit(b, lits) for _, b, lits, _ in reqs]
    srv.drain()
    for rid, (_, _, _, want) in zip(ids, reqs):
        np.testing.assert_array_equal(srv.result(rid), want)
    assert srv.stats()["peak_in_flight"] == 1
    srv.close()
    for _, b, _, _ in reqs:
        b.close()


def test_cached_graphs_give_the_same_counts_and_follow_relation_changes(engine):
    from quickfoil_gb300._capi import QFG_OPT_USE_GRAPHS
    w = workloads.small_random(7, n_bindings=30000, max_tuples=6000, num_literals=40)
    lits = _register(engine, w)
    cols = _dev_columns(w.binding_columns)
    b = engine.bindings(cols, w.num_positive)
    want = engine.evaluate_step(b, lits)
    engine.set_option(QFG_OPT_USE_GRAPHS, 1)
    try:
        for _ in range(3):  # first call captures, the others replay
            np.testing.assert_array_equal(engine.evaluate_step(b, lits), want)
        # refilled in place: the replay reads the new contents
        new_cols = [np.random.default_rng(5).permutation(c) for c in w.binding_columns]
        torch.cuda.synchronize()
        for c, n in zip(cols, new_cols):
            c.copy_(torch.from_numpy(n))
        torch.cuda.synchronize()
        got = engine.evaluate_step(b, lits)
        engine.set_option(QFG_OPT_USE_GRAPHS, 0)
        np.testing.assert_array_equal(got, engine.evaluate_step(b, lits))
        engine.set_option(QFG_OPT_USE_GRAPHS, 1)
        # a relation registered again under the same id with other tuples
        rid = lits[0].relation
        rel = w.relations[rid - lits[0].relation + next(iter(dict.fromkeys(w.literals))).relation]
        engine.register_relation(rid, [np.asarray(c)[::-1].copy() + 1 for c in rel])
        got = engine.evaluate_step(b, lits)
        engine.set_option(QFG_OPT_USE_GRAPHS, 0)
        np.testing.assert_array_equal(got, engine.evaluate_step(b, lits))
    finally:
        engine.set_option(QFG_OPT_USE_GRAPHS, 0)
    b.close()


def test_autotuner_picks_bits_and_keeps_counts(engine):
    from quickfoil_gb300._capi import QFG_OPT_AUTOTUNE
    w = workloads.small_random(8, n_bindings=400_000, max_tuples=20000, num_literals=30)
    lits = _register(engine, w)
    b = engine.bindings(_dev_columns(w.binding_columns), w.num_positive)
    want = engine.evaluate_step(b, lits)
    bits, cbits, ms = engine.autotune_step(b, lits)
    assert ms > 0
    choice = engine.autotune_choice(400_000)
    if choice["mode"] == "tiled":
        assert 1 <= bits <= 16 and bits == choice["bits"]
        assert cbits == 0 if bits <= 8 else 7 <= cbits <= 8
    else:  # the streamed path won: its per-group bits offset
        assert choice["mode"] == "streamed" and bits == 0 and -1 <= cbits <= 2
    engine.set_option(QFG_OPT_AUTOTUNE, 1)
    try:
        np.testing.assert_array_equal(engine.evaluate_step(b, lits), want)
    finally:
        engine.set_option(QFG_OPT_AUTOTUNE, 0)
    b.close()


@pytest.mark.parametrize("slots,depth", [(2, 1), (1, 2)])
def test_served_request_waits_for_its_binding_upload(engine, slots, depth):
    """Binding sets uploaded from host memory right before submission: the
    request starts after the upload, and the next upload overlaps it.  With
    one slot of depth 2 the next request is queued behind the running one
    and each result is waited for before the one after it is submitted."""
    reqs = []
    for seed in (50, 51, 52):
        w = workloads.small_random(seed, n_bindings=300_000, max_tuples=8000, num_literals=30)
        lits = _register(engine, w)
        b = engine.bindings(w.binding_columns, w.num_positive)
        reqs.append((w, lits, engine.evaluate_step(b, lits)))
        b.close()
    srv = engine.server(slots=slots, depth=depth)
    ids, keep = [], []
    for i, (w, lits, want) in enumerate(reqs * 2):
        b = engine.bindings(w.binding_columns, w.num_positive)  # host upload on the context stream
        ids.append(srv.submit(b, lits))
        keep.append(b)
        if depth > 1 and i > 0:  # the pipelined pattern: result of the previous request
            np.testing.assert_array_equal(srv.result(ids[i - 1]), (reqs * 2)[i - 1][2])
    for rid, (_, _, want) in zip(ids, reqs * 2):
        np.testing.assert_array_equal(srv.result(rid), want)
    srv.close()
    for b in keep:
        b.close()
