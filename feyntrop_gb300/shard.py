"""One integral over several processes (one per GPU): rank r of `world` integrates
samples [r*N, (r+1)*N) of the seed's single stream (ft_run_options.first_sample),
which the GPU path reaches exactly by skip-ahead, so `world` ranks together evaluate
the samples a single run over world*N would.  The only exchange is the merge of the
2K moment records (count, sum f, sum f^2 as hi/lo pairs, a few hundred bytes) on the
host, after which ft_finalize_moments applies the reference's formulas once
(srcs/stats.hpp:86-121 merges per-thread stats the same way).

Batches shard the same way (batch_sharded): every rank runs its own contiguous block
of every integral's samples (mode "samples"), or its own share of the integrals at
their full N (mode "integrals"); the per-integral moment records are gathered and
merged, so the merged batch equals one run of the whole batch on one GPU.
"""
import math

__all__ = ["first_sample", "merge_moments", "integrate_sharded", "split_samples", "batch_sharded"]


def first_sample(rank, samples_per_rank, offset=0):
    """Index of rank's first sample in the seed's stream."""
    return offset + rank * samples_per_rank


def merge_moments(per_rank):
    """Field-wise exact sums (math.fsum) of the moment records of several shards:
    per_rank[r] is a list of 2K records [n, s1_hi, s1_lo, s2_hi, s2_lo]."""
    if not per_rank:
        raise ValueError("no shards")
    n = len(per_rank[0])
    if any(len(m) != n for m in per_rank):
        raise ValueError("shards with different numbers of eps orders")
    return [[math.fsum(m[i][k] for m in per_rank) for k in range(5)] for i in range(n)]


def integrate_sharded(integrate, samples_per_rank, K, real_only, rank, world, group=None, offset=0, **kw):
    """Runs integrate(N, first_sample=..., **kw) -> result dict with "moments" on this
    rank's shard, gathers every rank's moments (torch.distributed, any backend) and
    returns (merged integral [[[re, dre], [im, dim]], ...], this rank's result)."""
    from . import finalize_moments
    r = integrate(samples_per_rank, first_sample=first_sample(rank, samples_per_rank, offset), **kw)
    moments = r["moments"]
    if world > 1:
        import torch.distributed as dist
        allm = [None] * world
        dist.all_gather_object(allm, moments, group=group)
        moments = merge_moments(allm)
    return finalize_moments(moments, K, real_only), r


def split_samples(N, rank, world):
    """(first, count) of rank's contiguous block of N samples: the first N % world
    ranks take one more."""
    base, extra = divmod(int(N), world)
    count = base + (1 if rank < extra else 0)
    return rank * base + min(rank, extra), count


def _zero_moments(K):
    return [[0.0, 0.0, 0.0, 0.0, 0.0] for _ in range(2 * K)]


def batch_sharded(run, Ns, Ks, real_only, rank, world, seeds=0, first_samples=0, mode="samples", group=None):
    """A batch of integrals over `world` ranks.  run(Ns, seeds, first_samples) runs the
    given integrals of this rank's batch (a list with None for an integral it skips)
    and returns their result dicts (each with "moments").  mode "samples": rank r runs
    its block [first + split_samples(N, r, world)] of every integral's samples; mode
    "integrals": integral i runs whole on rank i % world.  Returns (merged integrals,
    one per integral as [[[re, dre], [im, dim]], ...], merged moment records)."""
    from . import finalize_moments
    n = len(Ns)
    seeds = list(seeds) if isinstance(seeds, (list, tuple)) else [seeds] * n
    firsts = list(first_samples) if isinstance(first_samples, (list, tuple)) else [first_samples] * n
    mine_N, mine_first = [], []
    for i in range(n):
        if mode == "samples":
            f, c = split_samples(Ns[i], rank, world)
            mine_N.append(c if c > 0 else None)
            mine_first.append(firsts[i] + f)
        elif mode == "integrals":
            mine_N.append(Ns[i] if i % world == rank else None)
            mine_first.append(firsts[i])
        else:
            raise ValueError("mode must be 'samples' or 'integrals'")
    res = run(mine_N, seeds, mine_first)
    local = [r["moments"] if N is not None else _zero_moments(Ks[i])
             for i, (N, r) in enumerate(zip(mine_N, res))]
    if world > 1:
        import torch.distributed as dist
        allm = [None] * world
        dist.all_gather_object(allm, local, group=group)
    else:
        allm = [local]
    merged = [merge_moments([allm[r][i] for r in range(world)]) for i in range(n)]
    return [finalize_moments(m, Ks[i], real_only[i]) for i, m in enumerate(merged)], merged
