"""BASELINE config 4 at full scale on the GPU: the reference learner's run on
the 1M-picture Bongard-like knowledge base (tests/golden/bongard_kb_trace.npz)
replayed through the C ABI with every binding set, example table and
compaction kept on the device (tests/learn_replay.py).  Every Evaluate call's
counts, every extension's output (column checksums), every coverage step's
count and covered positions equal the reference's (integers, tolerance 0);
so the learner, fed these results, selects the same literal at every step and
learns the same clauses.  Coverage is checked in the default set-membership
mode and in the reference-compatible mode (QFG_OPT_COVERAGE_COMPAT)."""
import pytest

from tests import learn_replay

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def own_engine():
    from quickfoil_gb300 import Engine
    torch.zeros(1, device="cuda")
    eng = Engine(0)
    yield eng
    eng.close()


@pytest.mark.parametrize("compat", [False, True])
def test_config4_learn_trace_replays_on_the_device(own_engine, compat):
    out = learn_replay.replay(own_engine, torch, compat=compat)
    assert out["calls"]["evaluate"] >= 5 and out["calls"]["extend"] >= 3
    assert out["calls"]["coverage"] >= 3
    assert out["reference_clauses"] == ["target(0) :-  r0(0, 1), r2(1), r4(2, 1), r1(2)"]
    print("config 4 replay:", out["calls"], "GPU s", out["gpu_seconds"],
          "reference s", out["reference_seconds"])
