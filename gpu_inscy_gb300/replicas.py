"""Multi-process helpers: INSCY has no exchange step, so one process per GPU
either runs a replica of the workload or takes a shard of independent
datasets (the batched workload).  Only the timing is combined: the slowest
rank's time over the points all ranks processed."""


def shard(sizes, rank, world):
    """Indices of the datasets `rank` processes: largest first, each to the
    least-loaded rank (deterministic, identical on every rank)."""
    load = [0] * world
    owner = {}
    for i in sorted(range(len(sizes)), key=lambda i: (-sizes[i], i)):
        r = min(range(world), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += sizes[i]
    return [i for i in range(len(sizes)) if owner[i] == rank]


def combine(points_local, ms_local, group=None):
    """Whole-job throughput: (sum of points) / (max of per-rank times)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return points_local / (ms_local * 1e-3), ms_local
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(ms_local)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    pts = torch.tensor([float(points_local)], dtype=torch.float64, device=dev)
    dist.all_reduce(pts, op=dist.ReduceOp.SUM, group=group)
    return float(pts.item()) / (float(t.item()) * 1e-3), float(t.item())
