"""Replica runs on several GPUs of one node.

The STRUCTURE runs are independent chains, so several GPUs take replicas: one
process per GPU (launched by torchrun), each with its own copy of the dataset
and its own chains, and no data-path exchange. What crosses ranks is the
timing: a barrier on both sides of the timed region and the maximum of the
ranks' times, from which the whole-job throughput is the units all ranks
processed over that time.
"""
from __future__ import annotations

import os

import torch


def env() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str = "nccl") -> tuple[int, int, int]:
    rank, world, local = env()
    if world > 1 and not torch.distributed.is_initialized():
        torch.distributed.init_process_group(backend, init_method="env://")
    return rank, world, local


def _device():
    if torch.distributed.is_initialized() and torch.distributed.get_backend() == "nccl":
        return "cuda"
    return "cpu"


def barrier() -> None:
    if torch.distributed.is_initialized():
        torch.distributed.barrier()


def max_over_ranks(x: float) -> float:
    if not torch.distributed.is_initialized():
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float) -> float:
    if not torch.distributed.is_initialized():
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.SUM)
    return float(t.item())


def finish() -> None:
    if torch.distributed.is_initialized():
        torch.distributed.destroy_process_group()
