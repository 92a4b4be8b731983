"""The multi-process path on the CPU: two gloo ranks, each integrating its own block of
samples of the same stream (first_sample = rank * N), merged with feyntrop_gb300.shard
and finalised once, against a single-process run over all 2N samples.

The per-shard sums come from the oracle's per-sample values here (no GPU in this
test); on GPUs the same merge runs on ft_integrate's moments (bench.py under torchrun).
"""
import json
import math
import os
import socket
import tempfile

import numpy as np
import pytest

PINS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_pins.json")))
N_PER_RANK = 20000


def shard_moments(inp, seed, first, count):
    """2K moment records of samples [first, first + count) from the oracle."""
    import oracle_lib as ol
    s = ol.Prepared(inp).samples(seed, first, count)
    ok = ~s["dropped"]
    K = s["R"].shape[1]
    out = []
    for j in range(K):
        for part in (np.real, np.imag):
            v = part(s["R"][ok, j])
            out.append([float(ok.sum()), math.fsum(v), 0.0, math.fsum(v * v), 0.0])
    return out


def _rank_main(rank, world, port, name, seed, result_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from feyntrop_gb300 import shard
        inp = PINS["cases"][name]["input"]
        K = inp["num_eps_terms"]

        def integrate(N, first_sample=0):
            return {"moments": shard_moments(inp, seed, first_sample, N)}

        import feyntrop_gb300 as ft
        real_only = not ft.subgraph_table(inp)[4]["deformed"]   # the plan's regime decision (host only)
        integral, _ = shard.integrate_sharded(integrate, N_PER_RANK, K, real_only, rank, world)
        if rank == 0:
            with open(result_path, "w") as f:
                json.dump(integral, f)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("name", ["C1_K4", "1L_3pt_mink", "1L_3pt_eucl"])
def test_two_gloo_ranks_equal_one_run_over_all_samples(name):
    mp = pytest.importorskip("torch.multiprocessing")
    import oracle_lib as ol
    seed = 5
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "merged.json")
        mp.start_processes(_rank_main, args=(2, free_port(), name, seed, path), nprocs=2, start_method="spawn")
        merged = json.load(open(path))
    inp = PINS["cases"][name]["input"]
    ref, kept, dropped = ol.Prepared(inp).integrate(2 * N_PER_RANK, seed, 1)
    for j in range(inp["num_eps_terms"]):
        (re, dre), (im, dim) = merged[j]
        assert abs(re - ref[j, 0]) <= 1e-12 * abs(ref[j, 0]) + 1e-15, (j, re, ref[j])
        assert abs(dre - ref[j, 1]) <= 1e-8 * ref[j, 1], (j, dre, ref[j])
        if ref[j, 3] == 0:
            assert im == 0 and dim == 0
        else:
            assert abs(im - ref[j, 2]) <= 1e-12 * abs(ref[j, 2]) + 1e-15
            assert abs(dim - ref[j, 3]) <= 1e-8 * ref[j, 3]


BATCH = ["C1_K4", "1L_3pt_mink", "1L_3pt_eucl"]   # three integrals, two topologies
BATCH_N = [15001, 12000, 9999]


def _batch_rank_main(rank, world, port, mode, result_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import feyntrop_gb300 as ft
        from feyntrop_gb300 import shard
        inputs = [PINS["cases"][n]["input"] for n in BATCH]
        Ks = [x["num_eps_terms"] for x in inputs]
        real_only = [not ft.subgraph_table(x)[4]["deformed"] for x in inputs]

        def run(mine, seeds, firsts):
            # this rank's part of the batch, from the oracle's per-sample values
            return [None if N is None else {"moments": shard_moments(x, s, f, N)}
                    for x, N, s, f in zip(inputs, mine, seeds, firsts)]

        integrals, _ = shard.batch_sharded(run, BATCH_N, Ks, real_only, rank, world, seeds=[3, 4, 5], mode=mode)
        if rank == 0:
            with open(result_path, "w") as f:
                json.dump(integrals, f)
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("mode", ["samples", "integrals"])
def test_sharded_batch_equals_one_run(mode):
    """A 3-integral, 2-topology batch over two gloo ranks (each rank its block of every
    integral's samples, or its share of the integrals), merged, against one run of every
    integral over all its samples."""
    mp = pytest.importorskip("torch.multiprocessing")
    import oracle_lib as ol
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "merged.json")
        mp.start_processes(_batch_rank_main, args=(2, free_port(), mode, path), nprocs=2, start_method="spawn")
        merged = json.load(open(path))
    for name, N, seed, got in zip(BATCH, BATCH_N, [3, 4, 5], merged):
        inp = PINS["cases"][name]["input"]
        ref, _, _ = ol.Prepared(inp).integrate(N, seed, 1)
        for j in range(inp["num_eps_terms"]):
            (re, dre), (im, dim) = got[j]
            assert abs(re - ref[j, 0]) <= 1e-12 * abs(ref[j, 0]) + 1e-15, (name, j, re, ref[j])
            assert abs(dre - ref[j, 1]) <= 1e-8 * ref[j, 1], (name, j, dre, ref[j])
            if ref[j, 3] == 0:
                assert im == 0 and dim == 0
            else:
                assert abs(im - ref[j, 2]) <= 1e-12 * abs(ref[j, 2]) + 1e-15


def test_split_samples_covers_the_range():
    from feyntrop_gb300 import shard
    for N in (0, 1, 7, 1000, 12345):
        for world in (1, 2, 3, 8):
            parts = [shard.split_samples(N, r, world) for r in range(world)]
            assert sum(c for _, c in parts) == N
            pos = 0
            for f, c in parts:
                assert f == pos
                pos += c


def test_merge_rejects_mismatched_shards():
    from feyntrop_gb300 import shard
    with pytest.raises(ValueError):
        shard.merge_moments([[[1, 0, 0, 0, 0]] * 2, [[1, 0, 0, 0, 0]] * 4])
    m = shard.merge_moments([[[2, 1.0, 1e-17, 3.0, 0.0]], [[3, 2.0, -1e-17, 4.0, 0.0]]])
    assert m == [[5, 3.0, 0.0, 7.0, 0.0]]
    assert shard.first_sample(3, 1000, offset=7) == 3007
