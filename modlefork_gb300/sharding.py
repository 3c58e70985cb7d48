"""Multi-GPU runs: one process per GPU, cells (or perturbate windows) sharded across ranks.

A cell is a pure function of the configuration, the chromosome and its cell id (its seed is
Chromosome::hash of (seed, cell id), genome.cpp:317-335), so ranks share nothing while they
simulate.  A run partitions every chromosome's cell ids into contiguous ranges, one per rank,
and ends with one exact integer sum of each chromosome's band over the ranks (the reference's
worker threads add into one shared matrix instead, scheduler_simulate.cpp:229-256).  The
collective is torch.distributed's all_reduce on int64 counts: NCCL between GPUs, gloo on CPU.
"""

import numpy as np


def cell_range(ncells, world, rank):
    """Contiguous block of cell ids [lo, hi) of ``rank``: sizes differ by at most one."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    base, extra = divmod(int(ncells), int(world))
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard_tasks(seeds, targets, world, rank):
    """The slice of a chromosome's per-cell seeds and contact targets that ``rank`` runs."""
    lo, hi = cell_range(len(seeds), world, rank)
    return np.asarray(seeds)[lo:hi], np.asarray(targets)[lo:hi]


def allreduce_counts(values, device=None, group=None):
    """Exact sum over ranks of an integer array (bands are uint32, counters uint64); returns a
    numpy array of the input's dtype.  Counts travel as int64, so uint32 sums are exact."""
    import torch
    import torch.distributed as dist

    a = np.ascontiguousarray(values)
    t = torch.from_numpy(a.astype(np.int64))
    if device is not None:
        t = t.to(device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    out = t.cpu().numpy()
    if a.dtype == np.uint32 and (out.max(initial=0) > np.iinfo(np.uint32).max):
        raise OverflowError("a summed band count exceeds 2^32 - 1")
    return out.astype(a.dtype)


def allreduce_band_(band, group=None):
    """In-place exact sum over ranks of a uint32 band held as an int32 tensor (on the GPU with
    NCCL, on the CPU with gloo): two's-complement int32 addition wraps exactly as uint32
    addition does, so the result is the uint32 sum modulo 2^32, the reference's contacts_t
    arithmetic, without a round trip through host memory."""
    import torch
    import torch.distributed as dist

    if band.dtype != torch.int32:
        raise TypeError("the band must be an int32 view of the uint32 counts")
    dist.all_reduce(band, op=dist.ReduceOp.SUM, group=group)
    return band


def reduce_timing(ms, counters, device=None, group=None):
    """Max of the ranks' timed-region lengths and sums of their counters (dict of numbers)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    keys = sorted(counters)
    v = torch.tensor([float(counters[k]) for k in keys], dtype=torch.float64, device=device)
    dist.all_reduce(v, op=dist.ReduceOp.SUM, group=group)
    return float(t.item()), {k: float(x) for k, x in zip(keys, v.cpu().tolist())}


def simulate_chromosome_sharded(run_cells, chrom_task, world, rank, device=None, group=None):
    """Run this rank's share of one chromosome's cells with ``run_cells(seeds, targets, band)``
    (which adds contacts to ``band`` and returns the missed updates), then sum the bands and
    missed updates over the ranks; every rank returns the full chromosome's band."""
    seeds, targets = shard_tasks(chrom_task["seeds"], chrom_task["targets"], world, rank)
    band = np.zeros(chrom_task["nrows"] * chrom_task["ncols"], dtype=np.uint32)
    missed = run_cells(seeds, targets, band) if len(seeds) else 0
    band = allreduce_counts(band, device, group)
    missed = int(allreduce_counts(np.array([missed], dtype=np.uint64), device, group)[0])
    return band, missed


def shard_windows(planned, world, rank):
    """The contiguous block of the window queue (perturbate.plan_windows' (chrom, task) pairs,
    in task-id order) that ``rank`` simulates."""
    lo, hi = cell_range(len(planned), world, rank)
    return planned[lo:hi]


def gather_records(records, group=None):
    """Every rank's (task_id, bedpe line) records, merged in task-id order (records of one task
    keep their order); every rank returns the merged lines."""
    import torch.distributed as dist

    parts = [None] * dist.get_world_size(group)
    dist.all_gather_object(parts, list(records), group=group)
    merged = sorted((r for part in parts for r in part), key=lambda r: r[0])
    return [line for _, line in merged]


def perturbate_sharded(cfg, planned, feats1, feats2, ref_bands, world, rank, run_windows, block_size=9,
                       group=None):
    """modle perturbate over ranks: this rank simulates its block of the window queue with
    ``run_windows(cfg, planned_block)`` (perturbate.run_windows on a GPU), scores its windows,
    and the ranks exchange their records; each rank returns all records in task-id order.
    Window cells are independent, so only the records cross ranks."""
    from . import perturbate

    mine = shard_windows(planned, world, rank)
    recs = []
    for r in run_windows(cfg, mine):
        for line in perturbate.perturbate_records(cfg, feats1, feats2, ref_bands, [r], block_size):
            recs.append((r.task["task_id"], line))
    return gather_records(recs, group)
