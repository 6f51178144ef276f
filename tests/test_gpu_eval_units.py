"""Evaluation units of the batched step against the oracle, at shapes that take
every branch of the evaluation kernel's work loop: items of many tiles (more
binding rows than a shared-memory tile holds), items whose relation entries
fill several 512-entry chunks and several evaluation units, partial last
chunks (entries shared by several threads, threads without an entry in a later
chunk), and a hot join key.  Integer counts, tolerance 0."""
import numpy as np
import pytest

import oracle
from quickfoil_gb300 import _capi as C
from quickfoil_gb300.engine import Literal

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

_BASE = 700_000


def _case(seed: int):
    rng = np.random.default_rng(seed)
    n, P, dom = 200_003, 61_001, 4_000
    # Join column: a hot key on a tenth of the rows, the rest uniform.
    j = rng.integers(0, dom, n, dtype=np.int32)
    j[rng.random(n) < 0.1] = 7
    B = [j, rng.integers(0, 40, n, dtype=np.int32), rng.integers(0, 40, n, dtype=np.int32),
         rng.integers(0, dom, n, dtype=np.int32)]
    # R0: many distinct (key, value) tuples a key; R1: two checked columns.
    R0 = [rng.integers(0, dom, 300_000, dtype=np.int32), rng.integers(0, 40, 300_000, dtype=np.int32)]
    R1 = [rng.integers(0, dom, 200_000, dtype=np.int32), rng.integers(0, 40, 200_000, dtype=np.int32),
          rng.integers(0, 40, 200_000, dtype=np.int32)]
    R2 = [rng.integers(0, dom, 50_000, dtype=np.int32)]
    rels = [R0, R1, R2]
    spec = [(0, [0, -1], 0), (0, [0, 1], 0), (0, [0, 2], 0), (1, [0, 1, 2], 0), (1, [0, 2, -1], 0),
            (1, [0, -1, 1], 0), (2, [0], 0), (0, [3, 1], 0), (2, [3], 0)]
    return rels, B, P, spec


@pytest.mark.parametrize("bits", [0, 2, 6])
def test_evaluation_units_match_the_oracle(engine, bits):
    rels, B, P, spec = _case(5)
    want = oracle.evaluate(rels, B, P, spec, bits=8, nthreads=8)
    assert want[:, 2:].min() > 0  # every literal joins
    for i, r in enumerate(rels):
        engine.register_relation(_BASE + i, r)
    lits = [Literal(_BASE + r, tuple(v), jp) for r, v, jp in spec]
    b = engine.bindings([torch.from_numpy(c).cuda() for c in B], P)
    try:
        engine.set_option(C.QFG_OPT_EVAL_BITS, bits)
        engine.set_option(C.QFG_OPT_EVAL_MODE, 1)
        np.testing.assert_array_equal(engine.evaluate_step(b, lits), want)
    finally:
        engine.set_option(C.QFG_OPT_EVAL_BITS, 0)
        engine.set_option(C.QFG_OPT_EVAL_MODE, 0)
        b.close()
        for i in range(len(rels)):
            engine.release_relation(_BASE + i)
