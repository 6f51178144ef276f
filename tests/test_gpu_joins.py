"""GPU parity of the API-kept join operators against the oracle (bit-exact):
LeftSemiJoin / RightSemiJoin bit vectors and the label-aware binding-set
extension, including its row order."""
import numpy as np
import pytest

import oracle
from quickfoil_gb300 import QfgError
from quickfoil_gb300.engine import Literal
from tests.brute import brute_counts

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

_ids = [5000]


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).cuda()


@pytest.mark.parametrize("k", [1, 2, 3, 6])
@pytest.mark.parametrize("n_probe,n_build", [(0, 5), (5, 0), (1, 1), (777, 333), (100000, 3000),
                                             (64, 64), (65, 200000)])
def test_semijoins_exact(engine, k, n_probe, n_build):
    rng = np.random.default_rng(k * 7 + n_probe)
    probe = [rng.integers(0, 6, n_probe).astype(np.int32) for _ in range(k)]
    build = [rng.integers(0, 6, n_build).astype(np.int32) for _ in range(k)]
    for name, nrows in (("left", n_probe), ("right", n_build)):
        fn = engine.left_semijoin if name == "left" else engine.right_semijoin
        ofn = oracle.left_semijoin if name == "left" else oracle.right_semijoin
        if nrows == 0:
            continue
        bits, ones = fn([dev(c) for c in probe], [dev(c) for c in build])
        wbits, wones = ofn(probe, build)
        assert ones == wones
        np.testing.assert_array_equal(bits.cpu().numpy().view(np.uint64), wbits)


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("n_probe,n_build", [(300000, 9000), (9000, 300000), (40000, 30000),
                                             (30000, 40000)])
def test_semijoins_wide_domain(engine, k, n_probe, n_build):
    """Mostly missing keys (the bit filter rejects most probes) and repeated
    keys, with either side the larger one (the key set is built on the
    smaller side, whichever side gets the bits)."""
    rng = np.random.default_rng(1000 * k + n_probe)
    dom = {1: 60000, 2: 300, 3: 40}[k]
    probe = [rng.integers(-dom, dom, n_probe).astype(np.int32) for _ in range(k)]
    build = [rng.integers(-dom, dom, n_build).astype(np.int32) for _ in range(k)]
    for name in ("left", "right"):
        fn = engine.left_semijoin if name == "left" else engine.right_semijoin
        ofn = oracle.left_semijoin if name == "left" else oracle.right_semijoin
        bits, ones = fn([dev(c) for c in probe], [dev(c) for c in build])
        wbits, wones = ofn(probe, build)
        assert 0 < wones < (n_probe if name == "left" else n_build)
        assert ones == wones
        np.testing.assert_array_equal(bits.cpu().numpy().view(np.uint64), wbits)


def _extension_case(engine, B, P, R, lit):
    rid = _ids[0]
    _ids[0] += 1
    engine.register_relation(rid, R)
    c = brute_counts([R], B, P, [Literal(0, lit.vars, lit.join_pos)])[0]
    npos, nneg = int(c[2]), int(c[3])
    want = oracle.extend_bindings(B, P, R, (0, list(lit.vars), lit.join_pos), npos, nneg)
    b = engine.bindings(B, P)
    glit = Literal(rid, lit.vars, lit.join_pos)
    nb = engine.extend_bindings(b, glit, npos, nneg)
    got = nb.download()
    assert len(got) == len(want)
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g, w)
    with pytest.raises(QfgError):
        engine.extend_bindings(b, glit, npos + 1, nneg)
    return nb, glit


@pytest.mark.parametrize("case", range(6))
def test_extend_bindings_exact(engine, case):
    rng = np.random.default_rng(case)
    n, P = [60, 5000, 20000, 3000, 100, 40000][case], [20, 400, 2000, 3000, 0, 4000][case]
    nR = [10, 100000, 800, 50000, 7, 30000][case]
    dom = [5, 300, 50, 1000, 3, 2000][case]
    B = [rng.integers(0, dom, n).astype(np.int32) for _ in range(3)]
    R = [rng.integers(0, dom, nR).astype(np.int32) for _ in range(2)]
    lit = [Literal(0, (0, -1)), Literal(0, (1, 0)), Literal(0, (-1, 2)), Literal(0, (2, 2)),
           Literal(0, (0, -1)), Literal(0, (1, -1))][case]
    _extension_case(engine, B, P, R, lit)


def test_extension_feeds_next_step(engine):
    """The extended binding set stays on the device and feeds the next
    evaluation; its counts equal the oracle's on the downloaded columns."""
    rng = np.random.default_rng(11)
    B = [rng.integers(0, 40, 3000).astype(np.int32) for _ in range(2)]
    R = [rng.integers(0, 40, 500).astype(np.int32) for _ in range(2)]
    nb, glit = _extension_case(engine, B, 700, R, Literal(0, (0, -1)))
    cols = nb.download()
    rid = glit.relation
    lits = [Literal(rid, (2, 1)), Literal(rid, (2, -1)), Literal(rid, (-1, 0))]
    want = brute_counts({rid: R}, cols, nb.num_positive, lits)
    np.testing.assert_array_equal(engine.evaluate_step(nb, lits), want)


def test_after_semijoin_table_matches_reference_and_oracle(engine):
    """qfg_build_hash_table_after_semijoin against the reference's own tables
    (golden fixture) and the oracle, byte for byte: buckets, mask, and every
    next link (0 for positions never inserted, in both)."""
    from tests import golden
    for keys, bits, chunk, nbt, want_b, want_n, want_m in golden.after_semijoin_cases():
        dk = [dev(k) for k in keys]
        db = torch.from_numpy(bits.view(np.int64)).cuda()
        b, nx, m = engine.build_hash_table_after_semijoin(dk, db, chunk, nbt)
        b, nx = b.cpu().numpy(), nx.cpu().numpy()
        assert m == want_m
        np.testing.assert_array_equal(b, want_b)
        np.testing.assert_array_equal(oracle.reachable_next(b, nx), want_n)
        ob, onx, om = oracle.build_hash_table_after_semijoin(keys, bits, chunk, nbt)
        np.testing.assert_array_equal(b, ob)
        np.testing.assert_array_equal(nx, onx)


@pytest.mark.parametrize("n,k,dom,chunk", [(1, 1, 5, 0), (40000, 2, 20, 32768), (9000, 4, 3, 2000),
                                           (50000, 1, 1 << 30, 0)])
def test_after_semijoin_table_random_against_oracle(engine, n, k, dom, chunk):
    rng = np.random.default_rng(n + k)
    keys = [rng.integers(0, dom, n).astype(np.int32) for _ in range(k)]
    flags = rng.random(n) < 0.7
    words = np.zeros((n + 63) // 64, dtype=np.uint64)
    idx = np.nonzero(flags)[0]
    np.bitwise_or.at(words, idx >> 6, np.left_shift(np.uint64(1), (idx & 63).astype(np.uint64)))
    nbt = n if chunk <= 0 else max(chunk, 1)
    b, nx, m = engine.build_hash_table_after_semijoin([dev(c) for c in keys],
                                                      torch.from_numpy(words.view(np.int64)).cuda(),
                                                      chunk, nbt)
    ob, onx, om = oracle.build_hash_table_after_semijoin(keys, words, chunk, nbt)
    assert m == om
    np.testing.assert_array_equal(b.cpu().numpy(), ob)
    np.testing.assert_array_equal(nx.cpu().numpy(), onx)
