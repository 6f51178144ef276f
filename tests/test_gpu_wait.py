"""The bounded device-side wait of the batched evaluation kernel.

A tile of binding rows reaches shared memory by bulk copies that complete on
an mbarrier; the kernel polls that barrier at most QFG_OPT_WAIT_LIMIT times,
then flags the context, stops its CTA and the call returns QFG_ERR_TIMEOUT.
The test option QFG_OPT_TEST_WITHHOLD_COPIES makes the kernel announce tile
bytes without issuing any copy, so the wait runs out with nothing in flight
(no fault, no hang).  The next call on the same context must then be clean:
status OK and counts equal to the oracle's (integer counts, tolerance 0).
"""
import numpy as np
import pytest

import oracle
from quickfoil_gb300 import workloads
from quickfoil_gb300 import _capi as C
from quickfoil_gb300.engine import Literal

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_wait_that_runs_out_returns_timeout_and_context_stays_usable(engine):
    w = workloads.small_random(41, n_bindings=30000, max_tuples=4000, num_literals=24)
    base = 900_000
    for i, r in enumerate(w.relations):
        engine.register_relation(base + i, r)
    lits = [Literal(base + l.relation, l.vars, l.join_pos) for l in w.literals]
    want = oracle.evaluate(w.relations, w.binding_columns, w.num_positive,
                           [l.as_tuple() for l in w.literals], bits=5)
    b = engine.bindings([torch.from_numpy(c).cuda() for c in w.binding_columns], w.num_positive)
    try:
        engine.set_option(C.QFG_OPT_WAIT_LIMIT, 2000)
        engine.set_option(C.QFG_OPT_TEST_WITHHOLD_COPIES, 1)
        with pytest.raises(C.QfgError) as err:
            engine.evaluate_step(b, lits)
        assert err.value.status == C.QFG_ERR_TIMEOUT
        # Same context, copies issued again: a clean call with exact counts.
        engine.set_option(C.QFG_OPT_TEST_WITHHOLD_COPIES, 0)
        engine.set_option(C.QFG_OPT_WAIT_LIMIT, 1 << 26)
        np.testing.assert_array_equal(engine.evaluate_step(b, lits), want)
        np.testing.assert_array_equal(engine.evaluate_step(b, lits), want)
    finally:
        engine.set_option(C.QFG_OPT_TEST_WITHHOLD_COPIES, 0)
        engine.set_option(C.QFG_OPT_WAIT_LIMIT, 1 << 26)
        b.close()
        for i in range(len(w.relations)):
            engine.release_relation(base + i)
