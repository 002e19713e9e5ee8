"""Several GPUs of one node run independent replicas of the loop (the loop
does not shard here: one domain per rank, weak scaling). This is the host
logic around a timed region: a barrier, the maximum of the per-rank times,
and the whole-job throughput from them. There is no collective on the data
path."""
import os


def comm(backend="nccl", device=0):
    """(world, rank, barrier, dmax, close) for the process group described by
    the torchrun environment (RANK, WORLD_SIZE, MASTER_ADDR, MASTER_PORT); a
    single process gets no-op functions."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world <= 1:
        return 1, 0, (lambda: None), (lambda x: x), (lambda: None)
    import torch
    import torch.distributed as dist

    dist.init_process_group(backend)
    rank = dist.get_rank()
    on_cpu = backend == "gloo"

    def barrier():
        if on_cpu:
            dist.barrier()
        else:
            dist.barrier(device_ids=[device])

    def dmax(x):
        t = torch.tensor([float(x)], dtype=torch.float64, device="cpu" if on_cpu else f"cuda:{device}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def close():
        dist.destroy_process_group()

    return world, rank, barrier, dmax, close


def job_throughput(units_per_rank, steps, world, t_max):
    """Units per second of the whole job: every rank processed
    units_per_rank x steps units, the job took the slowest rank's time."""
    return units_per_rank * steps * world / t_max
