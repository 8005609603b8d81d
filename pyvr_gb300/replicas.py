"""Replicas across GPUs: one independent server or renderer per process and
GPU, with no exchange on the data path (rays and requests are independent).
The only collectives are the timing barrier around a measured region, the
ranks' joint decision to repeat a measurement, and the final aggregation of
what every rank did."""

from __future__ import annotations


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1 else None


def barrier() -> None:
    """Line the ranks up before (and after) a timed region."""
    d = _dist()
    if d is not None:
        d.barrier()


def all_ok(flag: bool, device=None) -> bool:
    """True on every rank if the flag is true on every rank: a decision the
    ranks take together (e.g. whether a timed run is repeated), so that their
    collectives stay paired.  With one process, the flag itself."""
    d = _dist()
    if d is None:
        return bool(flag)
    import torch
    t = torch.tensor([1 if flag else 0], dtype=torch.int32, device=device)
    d.all_reduce(t, op=d.ReduceOp.MIN)
    return bool(t.item())


def job_rate(count: float, elapsed_s: float, device=None) -> float:
    """Whole-job rate of the replicas: the units all ranks completed divided
    by the longest rank's elapsed time (the job ends when its slowest rank
    does).  With one process, count / elapsed_s."""
    d = _dist()
    if d is None:
        return count / elapsed_s if elapsed_s > 0 else 0.0
    import torch
    c = torch.tensor([float(count)], dtype=torch.float64, device=device)
    e = torch.tensor([float(elapsed_s)], dtype=torch.float64, device=device)
    d.all_reduce(c, op=d.ReduceOp.SUM)
    d.all_reduce(e, op=d.ReduceOp.MAX)
    return c.item() / e.item() if e.item() > 0 else 0.0
