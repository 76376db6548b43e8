"""Corpus split across GPUs: one process per GPU, each holding a contiguous shard.

The reference splits its corpus into chunks, searches each chunk on its own
CUDA stream and merges the per-chunk top-k lists on the host
(src/cuknnBitonic.cu:550-589; mergeResBitonic, :381-417).  Across GPUs the
same structure has one real exchange step: every rank searches its shard for
the top-min(k, rows) of every query (indices made global by the shard's first
row), the ranks all-gather those Q x k (distance, index) lists, and each rank
merges them in rank order on its own device (knns_merge_topk, by (distance,
index)).  Every rank ends with the same answer, the one a single search over
the whole corpus gives: a (query, row) pair's distance does not depend on the
shard it sits in, and ties resolve by the lower global index on every path.

Queries, in the other split, need no exchange at all (replicas): that is what
the benchmark's default multi-GPU mode measures.

The collective is torch.distributed's all_gather on the group given (NCCL
between GPUs); the functions take the search and merge steps as parameters so
that the host logic can be exercised with CPU ranks (gloo) and stand-in steps.
"""
from __future__ import annotations

INT32_MAX = 2 ** 31 - 1


def shard_bounds(n: int, world: int, rank: int):
    """Rows [r0, r1) of rank `rank` in a balanced contiguous split of n rows over `world` ranks."""
    if world < 1 or not 0 <= rank < world or n < 0:
        raise ValueError("bad shard request")
    base, extra = divmod(n, world)
    r0 = rank * base + min(rank, extra)
    return r0, r0 + base + (1 if rank < extra else 0)


def sharded_search(shard, offset: int, queries, k: int, *, group=None, search=None, merge=None, **opts):
    """kNN of `queries` against the corpus whose rows [offset, offset + len(shard)) this rank holds.

    shard, queries: tensors on this rank's device (CUDA for the engine; any device the stand-in
    steps accept).  Every rank passes the same queries and k.  Returns (dist Q x k float32,
    idx Q x k int32 global row indices), identical on every rank.

    search(shard, queries, kb, **opts) -> (dist Q x kb, idx Q x kb local rows), default the
    engine's device search; merge(run_d, run_i, have, blk_d, blk_i, kb, k) -> (dist, idx) Q x k,
    default the engine's device merge.
    """
    import torch
    import torch.distributed as dist
    if search is None or merge is None:
        import cuknns
        search = search or (lambda c, q, kk, **o: cuknns.search(c, q, kk, **o))
        merge = merge or (lambda rd, ri, h, bd, bi, kb_, kk: cuknns.merge_topk(rd, ri, h, bd, bi, kb_, kk))
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    Q = queries.shape[0]
    rows = shard.shape[0]
    if offset < 0 or offset + rows > INT32_MAX:
        raise ValueError("global row indices must fit in int32")
    dev = queries.device
    kb = min(k, rows)
    # this rank's list, padded to k columns so that every rank contributes equal shapes
    d_loc = torch.full((Q, k), float("inf"), dtype=torch.float32, device=dev)
    i_loc = torch.full((Q, k), INT32_MAX, dtype=torch.int32, device=dev)
    if kb > 0 and Q > 0:
        d, i = search(shard, queries, kb, **opts)
        d_loc[:, :kb] = d
        i_loc[:, :kb] = i.to(torch.int32) + int(offset)
    if world == 1:
        return d_loc, i_loc
    counts = torch.tensor([kb], dtype=torch.int64, device=dev)
    all_counts = [torch.zeros_like(counts) for _ in range(world)]
    all_d = [torch.empty_like(d_loc) for _ in range(world)]
    all_i = [torch.empty_like(i_loc) for _ in range(world)]
    dist.all_gather(all_counts, counts, group=group)
    dist.all_gather(all_d, d_loc, group=group)
    dist.all_gather(all_i, i_loc, group=group)
    return merge_rank_lists(all_d, all_i, [int(c.item()) for c in all_counts], k, merge)


def merge_rank_lists(ds, idxs, counts, k: int, merge):
    """Merge per-rank lists (rank order; ds[r] / idxs[r] Q x k, first counts[r] columns real,
    global indices) into one Q x k list by (distance, index)."""
    have = counts[0]
    run_d, run_i = ds[0], idxs[0]
    for r in range(1, len(ds)):
        kr = counts[r]
        if kr == 0:
            continue
        run_d, run_i = merge(run_d, run_i, have, ds[r][:, :kr].contiguous(), idxs[r][:, :kr].contiguous(), kr, k)
        have = min(k, have + kr)
    return run_d, run_i
