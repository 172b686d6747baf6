"""Batch-mode replicas: the configurations of one batched sweep partitioned
across processes (one GPU each), whole configurations per process, balanced
by their photon budgets.

A configuration's photons all stay on one process, so every configuration's
outputs come from exactly one process: the processes' results are gathered,
not summed.  (Splitting the photons of one configuration across processes is
the other replica mode, `Simulation.set_replica` / `xmi_gpu_set_replica`,
whose outputs are summed as the reference's MPI reduce does,
bin/xmimsim.c:396-413.)  The reference has no batched sweep on several
processes; its batch mode (src/xmi_batch.c:367-472) runs the configurations
one after another.
"""
from __future__ import annotations

from typing import Sequence


def photon_budget(spec) -> int:
    """Photon histories one xmi_main_msim of `spec` simulates: every
    continuous interval and every discrete line runs its own photon count
    (src/xmi_main.F90:240-858)."""
    return int(spec.n_photons_interval) * max(0, len(spec.continuous) - 1) + \
        int(spec.n_photons_line) * len(spec.discrete)


def partition_by_budget(budgets: Sequence[int], n_ranks: int) -> list[list[int]]:
    """Configuration indices of each of `n_ranks` processes.

    Longest processing time first: the configurations in decreasing budget
    (ties by index), each given to the process with the least budget so far
    (ties: the lowest rank); each process's list in increasing index, so a
    process runs its configurations in the sweep's order.  The result depends
    on the budgets alone, so every process computes the same partition
    without communication.  The largest load is at most 4/3 of the best
    possible one (Graham's bound for this greedy), hence at most
    4/3 * max(sum / n_ranks, largest budget)."""
    if n_ranks < 1:
        raise ValueError("n_ranks must be at least 1")
    if any(int(b) < 0 for b in budgets):
        raise ValueError("budgets must be non-negative")
    load = [0] * n_ranks
    parts: list[list[int]] = [[] for _ in range(n_ranks)]
    for i in sorted(range(len(budgets)), key=lambda i: (-int(budgets[i]), i)):
        r = min(range(n_ranks), key=lambda r: (load[r], r))
        parts[r].append(i)
        load[r] += int(budgets[i])
    return [sorted(p) for p in parts]


def rank_share(specs: Sequence, rank: int, n_ranks: int) -> list[int]:
    """Indices of the configurations process `rank` runs."""
    if not 0 <= rank < n_ranks:
        raise ValueError("rank out of range")
    return partition_by_budget([photon_budget(s) for s in specs], n_ranks)[rank]


def gather_by_config(parts: Sequence[Sequence[int]], results: Sequence[Sequence], n_configs: int) -> list:
    """Per-configuration results in sweep order from each process's results
    (in the order of its index list); every configuration exactly once."""
    out: list = [None] * n_configs
    seen = [False] * n_configs
    for idx, res in zip(parts, results):
        if len(idx) != len(res):
            raise ValueError("a process returned %d results for %d configurations" % (len(res), len(idx)))
        for i, r in zip(idx, res):
            if seen[i]:
                raise ValueError("configuration %d returned by two processes" % i)
            seen[i] = True
            out[i] = r
    if not all(seen):
        raise ValueError("configurations without a result: %s" % [i for i, s in enumerate(seen) if not s])
    return out
