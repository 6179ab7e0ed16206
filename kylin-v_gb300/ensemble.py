"""Independent chains over several GPUs.

A single chain's sweep is sequential, but independent chains (a disordered
ensemble, the perturbed runs of a finite-difference gradient) partition
across GPUs with no exchange step: one process per GPU, each advancing its
share of the chains with kv_sweep_batched, and the observables gathered on
rank 0's host at the end.  The reference runs such chains as separate
kln-tdvp processes (src/kln-tdvp.cpp:22-80), one chain each.
"""
from __future__ import annotations

from typing import Callable


def chain_cost(n_sites: int, D: int) -> float:
    """Estimate of a chain's work per sweep (sites x D^3)."""
    return float(n_sites) * float(D) ** 3


def shard(costs: list, world: int) -> list:
    """Chain indices per rank: longest first, each to the least-loaded rank
    (ties to the lower index / rank), so every chain is on exactly one rank and
    the split is the same in every process."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    out = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += costs[i]
    return [sorted(x) for x in out]


def gather(obj, rank: int, world: int):
    """List of every rank's `obj` on rank 0 (None elsewhere); host objects
    only, through torch.distributed's object gather."""
    if world == 1:
        return [obj]
    import torch.distributed as dist

    out = [None] * world if rank == 0 else None
    dist.gather_object(obj, out, dst=0)
    return out


def run_ensemble(members: list, costs: list, run: Callable, rank: int = 0, world: int = 1):
    """Run `run(indices)` -> {index: result} on this rank's share of the
    chains and return every chain's result, in chain order, on rank 0
    (None on the other ranks)."""
    mine = shard(costs, world)[rank]
    res = run([members[i] for i in mine], mine) if mine else {}
    parts = gather(res, rank, world)
    if rank != 0:
        return None
    merged = {}
    for p in parts:
        merged.update(p)
    if sorted(merged) != list(range(len(members))):
        raise RuntimeError("ensemble: a chain's result is missing after the gather")
    return [merged[i] for i in range(len(members))]


def tdvp_runner(steps: int, mode: int = 1, precision: int = 1, max_streams: int = 0, tol_svd: float = 1e-8,
                tol_exp: float = 1e-8, max_iter: int = 11, dt: float = 0.05, seed: int = 1234):
    """A `run` for run_ensemble on this process's GPU: members are
    (HolsteinChain, D); each chain starts from the seeded random MPS
    (seed + its index), all advance together by kv_sweep_batched, and the
    result per chain is its exciton populations after every step."""
    from . import holstein as H
    from . import kvgpu as G

    def run(chains, idx):
        ts, dens = [], []
        for (ch, D), i in zip(chains, idx):
            ts.append(G.TDVP(H.random_mps(ch, D, seed=seed + i), H.hamiltonian_mpo(ch), tol_svd, tol_exp, D,
                             max_iter, dt, precision))
            dens.append([[G.Tensor.from_host(x) for x in H.density_mpo(ch, j)] for j in ch.exciton_sites()])
        pops = {i: [] for i in idx}
        for _ in range(steps):
            G.sweep_batched(ts, mode, 1, max_streams)
            for t, d, i in zip(ts, dens, idx):
                s = t.sites()
                pops[i].append([G.expectation(s, x, s).real for x in d])
        return pops

    return run
