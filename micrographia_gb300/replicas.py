"""Multi-GPU replicas. The MD path has no exchange step between GPUs, so N GPUs run independent
work: the same workload on every rank (plain and batched forms, weak scaling), or a request stream
dealt out by rank (serving). The only collectives aggregate the result: units summed and times
maxed over the ranks, frame latencies gathered. `pg` is `torch.distributed` after
`init_process_group` (NCCL on GPUs, gloo on CPU), or None for one process."""


def shard(items, rank, world):
    """Rank `rank`'s share of `items`: every `world`-th item from `rank` (request k to rank k mod N)."""
    return list(items)[rank::world]


def _device(pg):
    import torch

    return "cuda" if torch.cuda.is_available() and pg.get_backend() == "nccl" else "cpu"


def aggregate(pg, units, seconds):
    """(units summed over ranks, seconds maxed over ranks): the whole job's throughput is their ratio."""
    if pg is None:
        return float(units), float(seconds)
    import torch

    dev = _device(pg)
    u = torch.tensor([float(units)], dtype=torch.float64, device=dev)
    s = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    pg.all_reduce(u, op=pg.ReduceOp.SUM)
    pg.all_reduce(s, op=pg.ReduceOp.MAX)
    return float(u.item()), float(s.item())


def gather(pg, values):
    """Every rank's list of values, concatenated in rank order (on every rank)."""
    if pg is None:
        return list(values)
    out = [None] * pg.get_world_size()
    pg.all_gather_object(out, list(values))
    return [v for part in out for v in part]
