"""One integral over several processes (one per GPU): rank r of `world` integrates
samples [r*N, (r+1)*N) of the seed's single stream (ft_run_options.first_sample),
which the GPU path reaches exactly by skip-ahead, so `world` ranks together evaluate
the samples a single run over world*N would.  The only exchange is the merge of the
2K moment records (count, sum f, sum f^2 as hi/lo pairs, a few hundred bytes) on the
host, after which ft_finalize_moments applies the reference's formulas once
(srcs/stats.hpp:86-121 merges per-thread stats the same way).
"""
import math

__all__ = ["first_sample", "merge_moments", "integrate_sharded"]


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
