"""Replica bookkeeping for runs on several GPUs.

The path shards over independent (model, frequency, source batch) units with
no exchange step: the reference's frequency groups (elwave.f90:19-21,149).
Each rank factors its own frequency; the job's time is the slowest rank's.
"""
import torch


def rank_frequency(step, rank, freqs):
    """Frequency of a rank's step: ranks start at different frequencies."""
    return freqs[(step + rank) % len(freqs)]


def max_over_ranks(value, world, device="cpu"):
    """Largest value over the ranks (the job's time); identity for one rank."""
    if world <= 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, units_per_rank, seconds):
    """Whole-job throughput: every rank processes units_per_rank units."""
    return world * units_per_rank / seconds
