"""Partition-range sharding of the batched step.

CPU tests: the shard function splits every literal's binding rows into
disjoint shards whose oracle counts add up to the full counts, checked in one
process and across a world of 2 gloo ranks that exchange only the int64 sum.
GPU test: the engine's shard option gives counts equal to the oracle on the
shard's rows, and the shards sum to the full step.
"""
import os
import socket

import numpy as np
import pytest

import oracle
from quickfoil_gb300 import sharding, workloads
from quickfoil_gb300.engine import Literal


def _shard_counts(w, bits, shard, count):
    """Oracle counts of one shard: every literal sees only the binding rows
    whose join key hashes into the shard's partition range."""
    out = np.zeros((len(w.literals), 4), dtype=np.int64)
    o = oracle.Oracle(w.relations)
    try:
        for i, lit in enumerate(w.literals):
            j = lit.vars[lit.join_pos]
            mask = sharding.shard_mask(w.binding_columns[j], bits, shard, count)
            cols = [c[mask] for c in w.binding_columns]
            npos = int(mask[:w.num_positive].sum())
            out[i] = o.evaluate(cols, npos, [lit.as_tuple()], bits=5)[0]
    finally:
        o.close()
    return out


def test_fmix32_known_values():
    # fmix32(0) = 0; the finalizer is a bijection on uint32.
    assert sharding.fmix32(np.array([0]))[0] == 0
    x = np.arange(1 << 16, dtype=np.int64)
    assert len(np.unique(sharding.fmix32(x))) == len(x)


@pytest.mark.parametrize("count", [2, 3, 5])
def test_shards_sum_to_full_counts(count):
    w = workloads.small_random(3, n_bindings=2000, num_literals=16)
    full = oracle.evaluate(w.relations, w.binding_columns, w.num_positive,
                           [l.as_tuple() for l in w.literals], bits=5)
    total = sum(_shard_counts(w, 6, s, count) for s in range(count))
    np.testing.assert_array_equal(total, full)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, result_path):
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        w = workloads.small_random(4, n_bindings=3000, num_literals=20)
        mine = torch.from_numpy(_shard_counts(w, 7, rank, world))
        dist.all_reduce(mine, op=dist.ReduceOp.SUM)
        if rank == 0:
            np.save(result_path, mine.numpy())
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_exchange_only_the_count_sum(tmp_path):
    import torch.multiprocessing as mp
    path = str(tmp_path / "counts.npy")
    mp.start_processes(_rank_main, args=(2, _free_port(), path), nprocs=2, join=True,
                       start_method="spawn")
    w = workloads.small_random(4, n_bindings=3000, num_literals=20)
    full = oracle.evaluate(w.relations, w.binding_columns, w.num_positive,
                           [l.as_tuple() for l in w.literals], bits=5)
    np.testing.assert_array_equal(np.load(path), full)


@pytest.mark.gpu
def test_engine_shards_match_oracle_and_sum(engine):
    from quickfoil_gb300 import _capi as C
    torch = pytest.importorskip("torch")
    w = workloads.batched_step(n_bindings=200_000, num_relations=6, min_tuples=100,
                               max_tuples=50_000, num_literals=24, domain=10_000, seed=31)
    base = 90_000
    for rid, cols in enumerate(w.relations):
        engine.register_relation(base + rid, cols)
    lits = [Literal(base + l.relation, l.vars, l.join_pos) for l in w.literals]
    b = engine.bindings(w.binding_columns, w.num_positive)
    full = engine.evaluate_step(b, lits)
    bits, count = 10, 3
    total = np.zeros_like(full)
    engine.set_option(C.QFG_OPT_EVAL_BITS, bits)
    try:
        for s in range(count):
            engine.set_option(C.QFG_OPT_SHARD_COUNT, count)
            engine.set_option(C.QFG_OPT_SHARD_INDEX, s)
            got = engine.evaluate_step(b, lits)
            np.testing.assert_array_equal(got, _shard_counts(w, bits, s, count))
            total += got
    finally:
        engine.set_option(C.QFG_OPT_SHARD_INDEX, 0)
        engine.set_option(C.QFG_OPT_SHARD_COUNT, 1)
        engine.set_option(C.QFG_OPT_EVAL_BITS, 0)
    np.testing.assert_array_equal(total, full)


def _gpu_rank_main(rank, world, port, result_path):
    """One rank of a 2-rank gloo world on the one GPU: its own engine
    (context), the shared step, its shard through sharding.evaluate_sharded;
    rank 0 keeps the summed counts.  The ranks' kernels never wait on each
    other: the only exchange is the host-side sum of the counters."""
    import torch
    import torch.distributed as dist
    from quickfoil_gb300 import Engine
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        torch.zeros(1, device="cuda")
        eng = Engine(0)
        w = workloads.batched_step(n_bindings=300_000, num_relations=8, min_tuples=100,
                                   max_tuples=80_000, num_literals=40, domain=20_000, seed=33)
        for rid, cols in enumerate(w.relations):
            eng.register_relation(rid, cols)
        b = eng.bindings(w.binding_columns, w.num_positive)
        got = sharding.evaluate_sharded(eng, b, w.literals)
        if rank == 0:
            np.save(result_path, got)
        b.close()
        eng.close()
    finally:
        dist.destroy_process_group()


@pytest.mark.gpu
def test_two_gloo_ranks_evaluate_shards_on_the_gpu(tmp_path):
    """sharding.evaluate_sharded on 2 gloo ranks, each a process with its own
    engine on the one GPU: the summed counts equal the oracle's full step."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import torch.multiprocessing as mp
    path = str(tmp_path / "gpu_counts.npy")
    mp.start_processes(_gpu_rank_main, args=(2, _free_port(), path), nprocs=2, join=True,
                       start_method="spawn")
    w = workloads.batched_step(n_bindings=300_000, num_relations=8, min_tuples=100,
                               max_tuples=80_000, num_literals=40, domain=20_000, seed=33)
    full = oracle.evaluate(w.relations, w.binding_columns, w.num_positive,
                           [l.as_tuple() for l in w.literals], bits=5)
    np.testing.assert_array_equal(np.load(path), full)
