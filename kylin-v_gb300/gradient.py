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
    ident = [G.Tensor.from_host(x) for x in H.identity_mpo(chains[0])]
    dens = [(j, G.Tensor.from_host(H.density_mpo(chains[0], j)[j])) for j in chains[0].exciton_sites()]
    ts = [G.TDVP(mps, w, 0.0, tol_exp, D, max_iter, dt, precision) for w in mpos]
    msd = np.zeros(len(ts))
    weights = np.arange(len(dens), dtype=float)
    device_ms = 0.0
    for _ in range(steps):
        device_ms += G.sweep_batched(ts, 1, 1, max_streams)
        for c, t in enumerate(ts):
            s = t.sites()
            msd[c] += float(np.dot(weights, [v.real for v in G.local_expectations(s, ident, dens)]))
    energy = np.zeros(len(ts))
    for c, t in enumerate(ts):
        s = t.sites()
        energy[c] = G.expectation(s, mpos[c], s).real
    return {"value": {"msd": float(msd[0]), "energy": float(energy[0])},
            "grad": {"msd": assemble(msd, h, names), "energy": assemble(energy, h, names)},
            "chains": len(ts), "device_ms": device_ms}


# ------------------------------------------------------------ reverse mode
def _energy_envs(mps_dev, W_dev, precision):
    """Left environments of <psi|H|psi>: envs[0] the boundary, envs[s+1] =
    env_sweep(envs[s], A_s, W_s) (holstein/product.h:505-521)."""
    from .kvio import BlockTensor

    envs = [G.Tensor.from_host(BlockTensor((1, -1, -1), [((0, 0, 0), np.ones((1, 1, 1), complex))]))]
    for a, w in zip(mps_dev, W_dev):
        envs.append(G.env_sweep(envs[-1], a, w, True, precision))
    return envs


def _energy_value(env_last):
    """<psi|H|psi> from the final environment, as kv_expectation reads it."""
    h = env_last.to_host()
    if not h.blocks:
        return 0.0, h
    q = h.blocks[0][0][0]
    return float(sum(a.ravel()[0].real for qn, a in h.blocks if a.size == 1 and qn == (q, 0, q))), h


def energy_forward(chain: H.HolsteinChain, mps, names=PARAMS, precision: int = G.KV_FP64):
    """E = <psi|H(theta)|psi> on the device, keeping what the reverse pass needs
    (the left environments and the parameter-linear MPO)."""
    W, dW = H.hamiltonian_mpo_param(chain, names)
    A = [t if isinstance(t, G.Tensor) else G.Tensor.from_host(t) for t in mps]
    Wd = [G.Tensor.from_host(w) for w in W]
    envs = _energy_envs(A, Wd, precision)
    e, last = _energy_value(envs[-1])
    return e, {"A": A, "W": Wd, "dW": dW, "envs": envs, "last": last, "names": names, "precision": precision}


def energy_backward(state) -> dict:
    """dE/dtheta from energy_forward's state: from the cotangent 1 of E the
    environment adjoints run backward (kv_adjoint_env), giving the cotangent
    W_bar_s of every MPO site; dE/dtheta_k = sum_s Re<W_bar_s, dW_k[s]>."""
    from .kvio import BlockTensor

    last, names, dW = state["last"], state["names"], state["dW"]
    q = last.blocks[0][0][0] if last.blocks else 0
    ebar = G.Tensor.from_host(BlockTensor(last.dirs, [(qn, (np.ones_like(a) if (a.size == 1 and qn == (q, 0, q))
                                                           else np.zeros_like(a))) for qn, a in last.blocks]))
    grad = {k: 0.0 for k in names}
    for s in reversed(range(len(state["A"]))):
        out = G.adjoint_env(state["envs"][s], state["A"][s], state["W"][s], True, ebar, state["precision"],
                            want=("env", "W"))
        wbar = out["W"].to_host().as_dict()
        for k in names:
            for qn, d in dW[k][s].blocks:
                b = wbar.get((tuple(qn), d.shape))
                if b is not None:
                    grad[k] += float(np.sum(np.conj(b) * d).real)
        ebar = out["env"]
    return grad


def energy_gradient_adjoint(chain: H.HolsteinChain, mps, names=PARAMS, precision: int = G.KV_FP64) -> dict:
    """E = <psi|H(theta)|psi> and dE/dtheta by reverse mode through the MPS
    contraction (energy_forward, energy_backward): the environment adjoints of
    kv_adjoint_env and the exact dW/dtheta of the parameter-linear MPO.

    One-site TDVP without truncation conserves <H> exactly (up to the Krylov
    tolerance), so this is also the gradient of <H> after any number of such
    steps from the same state -- the differentiation workload's energy
    quantity."""
    e, state = energy_forward(chain, mps, names, precision)
    return {"value": e, "grad": energy_backward(state)}


def torch_energy(chain_of_theta, names=PARAMS, precision: int = G.KV_FP64):
    """A torch.autograd.Function of theta (a float64 tensor, one entry per
    name): forward E = <psi|H(theta)|psi> on the GPU library (energy_forward),
    backward the reverse-mode pass (energy_backward) scaled by the incoming
    gradient.  ``chain_of_theta(dict)`` builds the chain; call as
    ``torch_energy(f, names).apply(theta, mps)``."""
    import torch

    class HolsteinEnergy(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta, mps):
            th = {k: float(v) for k, v in zip(names, theta.detach().cpu().tolist())}
            e, ctx.kv_state = energy_forward(chain_of_theta(th), mps, names, precision)
            return torch.tensor(e, dtype=torch.float64)

        @staticmethod
        def backward(ctx, g):
            grad = energy_backward(ctx.kv_state)
            ctx.kv_state = None
            return g * torch.tensor([grad[k] for k in names], dtype=torch.float64), None

    return HolsteinEnergy
