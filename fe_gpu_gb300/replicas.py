"""Replica runs for bench.py --gpus N: one process per GPU, each fitting its
own copy of the workload. The estimation of one specification has no exchange
step that would shard (row-sharding would all-reduce the G x C group sums of
every projection), so N GPUs run N independent fits: a barrier on both sides
of the timed region, the slowest rank's time, and the whole-job throughput =
the rows of all ranks / that time (weak scaling). No collective touches the
data path; the only collectives are the barrier and the max of the timings."""
import os

import torch


def dist_env():
    """(rank, world size, local rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(world: int, backend: str = "nccl") -> None:
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group(backend)


def barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int, device="cpu") -> float:
    """The largest x over the ranks (every rank gets it)."""
    if world <= 1:
        return float(x)
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, seconds: float, world: int) -> float:
    """Whole-job throughput: the units every rank processed over the slowest
    rank's time."""
    return world * units_per_rank / seconds


def finish(world: int) -> None:
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
