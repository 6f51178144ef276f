"""The allocation-free radix partition, qfg_radix_partition_static.

It exists for callers that cannot let a library allocate device memory (a
host that owns all GPU memory through its own allocator, or a loop that
cannot afford the device synchronization of cudaMalloc / cudaFree); its only
working memory is a fixed array inside the library.  These tests call it
through the C ABI and require its output to equal that of the allocating
entry point, qfg_radix_partition, exactly (integer output, zero tolerance),
on two calls in a row, since the shared array keeps the previous call's
contents.  This file is collected last so a stop-at-first-failure run has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

from quickfoil_gb300 import Engine
from quickfoil_gb300 import _capi as C

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _static_partition(values, bits):
    lib = C.load()
    n = values.numel()
    tuples = torch.empty((max(n, 1), 2), dtype=torch.int32, device=values.device)
    offsets = torch.empty((1 << bits) + 1, dtype=torch.int64, device=values.device)
    err = ctypes.create_string_buffer(256)
    stream = torch.cuda.current_stream(values.device).cuda_stream
    rc = lib.qfg_radix_partition_static(stream, values.data_ptr(), n, bits, tuples.data_ptr(),
                                        offsets.data_ptr(), err, len(err))
    torch.cuda.synchronize()
    return rc, err.value.decode(), tuples[:n], offsets


@pytest.fixture(scope="module")
def own_engine():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.zeros(1, device="cuda")
    eng = Engine(0)
    eng.set_stream(torch.cuda.current_stream().cuda_stream)
    yield eng
    eng.close()


@pytest.mark.parametrize("bits,n", [(5, 1_000_000), (12, 300_000), (15, 2_000_000), (1, 17)])
def test_static_partition_equals_allocating_entry_point_twice(own_engine, bits, n):
    rng = np.random.default_rng(bits * 1000 + n)
    for call in range(2):  # the second call sees what the first left in the array
        vals = torch.from_numpy(rng.integers(-2**31, 2**31, n).astype(np.int32)).cuda()
        rc, err, tuples, offsets = _static_partition(vals, bits)
        assert rc == C.QFG_OK, err
        want_t, want_o = own_engine.radix_partition(vals, bits)
        torch.cuda.synchronize()
        assert torch.equal(offsets, want_o), f"offsets differ on call {call}"
        assert torch.equal(tuples, want_t), f"tuples differ on call {call}"


def test_static_partition_of_no_values_zeroes_the_offsets(own_engine):
    for call in range(2):
        vals = torch.empty(0, dtype=torch.int32, device="cuda")
        rc, err, _, offsets = _static_partition(vals, 7)
        assert rc == C.QFG_OK, err
        _, want_o = own_engine.radix_partition(vals, 7)
        torch.cuda.synchronize()
        assert torch.equal(offsets, torch.zeros_like(offsets))
        assert torch.equal(offsets, want_o), f"offsets differ on call {call}"


def test_static_partition_at_the_exact_scratch_limit(own_engine):
    # At 8 radix bits a warp chunk is 2048 values with 256 digit counts, and
    # the scan adds one word per 4096 counts: 4095 chunks fill the 2^20-word
    # array exactly (1 048 320 counts + 256 tile sums); one more value needs a
    # 4096th chunk and is refused.
    bits, n = 8, 4095 * 2048
    rng = np.random.default_rng(8)
    for call in range(2):
        vals = torch.from_numpy(rng.integers(-2**31, 2**31, n).astype(np.int32)).cuda()
        rc, err, tuples, offsets = _static_partition(vals, bits)
        assert rc == C.QFG_OK, err
        want_t, want_o = own_engine.radix_partition(vals, bits)
        torch.cuda.synchronize()
        assert torch.equal(offsets, want_o), f"offsets differ on call {call}"
        assert torch.equal(tuples, want_t), f"tuples differ on call {call}"
    rc, err, _, _ = _static_partition(torch.zeros(n + 1, dtype=torch.int32, device="cuda"), bits)
    assert rc == C.QFG_ERR_INVALID and "static scratch" in err


def test_static_partition_rejects_inputs_beyond_its_scratch():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    n = 40_000_000  # more than the static array can serve at 12 radix bits
    vals = torch.zeros(n, dtype=torch.int32, device="cuda")
    rc, err, _, _ = _static_partition(vals, 12)
    assert rc == C.QFG_ERR_INVALID
    assert "static scratch" in err
