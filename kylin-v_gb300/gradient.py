"""Parameter gradients of Holstein TDVP observables by central differences,
the perturbed chains advanced together on the GPU.

The reference has no derivative code; its gradient of an observable with
respect to a Hamiltonian parameter is the central difference of two runs of
``kln-tdvp`` at theta +- h (one process each).  Here all 2k + 1 chains (the
base point and theta +- h along each of k parameters) share one initial MPS
and advance together through ``kv_sweep_batched``; the observables are read
on the device after every step.  Quantities (one-site TDVP, dt per step):

  msd    = sum_{t=1..steps} sum_i i * P_i(t), P_i = <psi(t)| n_i |psi(t)>, the
           exciton population of molecule i (0-based), an exciton
           mean-square-displacement proxy
  energy = <psi(T)| H(theta) |psi(T)> after the last step

For the differences to be smooth, nothing is truncated (tolSVD = 0,
maxD = D) and the Krylov recurrence stops at a residual of 1e-12 (tolExp),
so a change of the Krylov dimension between neighbouring parameters moves
the result by about 1e-12.  tolExp = 0 (a fixed dimension) is not smooth: on
the small local spaces at the chain ends the recurrence of
holstein/exponential.h:109-147 then runs past the exhaustion of the space
and normalises rounding noise into the basis, and the result moves by about
1e-4 between neighbouring parameters.
"""
from __future__ import annotations

import numpy as np

from . import holstein as H
from . import kvgpu as G

PARAMS = ("J", "omega", "g")


def holstein_chain(n_mol: int, cutoff: int, theta: dict, eps=None) -> H.HolsteinChain:
    """A one-mode chain with hopping J, frequency omega and coupling g on every
    molecule (the differentiation workload's model)."""
    return H.HolsteinChain(n_mol, [theta["omega"]], [[theta["g"]]] * n_mol, cutoff=cutoff, J=theta["J"], eps=eps)


def points(theta: dict, h: float, names=PARAMS) -> list:
    """The base point, then theta + h e_k and theta - h e_k for each name."""
    out = [dict(theta)]
    for k in names:
        for s in (1.0, -1.0):
            p = dict(theta)
            p[k] = theta[k] + s * h
            out.append(p)
    return out


def assemble(values: np.ndarray, h: float, names=PARAMS) -> dict:
    """Central differences from the values at points(...)."""
    return {k: float((values[1 + 2 * i] - values[2 + 2 * i]) / (2.0 * h)) for i, k in enumerate(names)}


def fd_gradient(n_mol: int, cutoff: int, D: int, theta: dict, steps: int = 10, dt: float = 0.05, h: float = 1e-5,
                max_iter: int = 11, tol_exp: float = 1e-12, precision: int = G.KV_FP64, seed: int = 1234,
                names=PARAMS, max_streams: int = 0) -> dict:
    """Values and central-difference gradients of msd and energy (module
    docstring) with respect to `names`; all chains on the GPU."""
    pts = points(theta, h, names)
    chains = [holstein_chain(n_mol, cutoff, p) for p in pts]
    mps = [G.Tensor.from_host(x) for x in H.random_mps(chains[0], D, seed=seed)]
    mpos = [[G.Tensor.from_host(x) for x in H.hamiltonian_mpo(c)] for c in chains]
    dens = [[G.Tensor.from_host(x) for x in H.density_mpo(chains[0], j)] for j in chains[0].exciton_sites()]
    ts = [G.TDVP(mps, w, 0.0, tol_exp, D, max_iter, dt, precision) for w in mpos]
    msd = np.zeros(len(ts))
    weights = np.arange(len(dens), dtype=float)
    device_ms = 0.0
    for _ in range(steps):
        device_ms += G.sweep_batched(ts, 1, 1, max_streams)
        for c, t in enumerate(ts):
            s = t.sites()
            msd[c] += float(np.dot(weights, [G.expectation(s, d, s).real for d in dens]))
    energy = np.zeros(len(ts))
    for c, t in enumerate(ts):
        s = t.sites()
        energy[c] = G.expectation(s, mpos[c], s).real
    return {"value": {"msd": float(msd[0]), "energy": float(energy[0])},
            "grad": {"msd": assemble(msd, h, names), "energy": assemble(energy, h, names)},
            "chains": len(ts), "device_ms": device_ms}
