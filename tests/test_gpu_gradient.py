"""Central-difference parameter gradients (kylin_v_gb300.gradient): the GPU
routine, whose perturbed chains run together through kv_sweep_batched,
against the same differences formed from the oracle's one-site TDVP runs
(the reference's way of differentiating: one run per perturbed parameter)."""
import numpy as np
import pytest

import kvtest_util as U

U.load_package()
O = U.load_oracle()
from kylin_v_gb300 import gradient as GR  # noqa: E402
from kylin_v_gb300 import holstein as H  # noqa: E402

THETA = {"J": -1.0, "omega": 1.0, "g": 1.0}


def _oracle_fd(n_mol, cutoff, D, theta, steps, dt, h, seed=1234):
    pts = GR.points(theta, h)
    chains = [GR.holstein_chain(n_mol, cutoff, p) for p in pts]
    mps = H.random_mps(chains[0], D, seed=seed)
    dens = [H.density_mpo(chains[0], j) for j in chains[0].exciton_sites()]
    msd, energy = np.zeros(len(pts)), np.zeros(len(pts))
    for c, ch in enumerate(chains):
        mpo = H.hamiltonian_mpo(ch)
        t = O.Tdvp(mps, mpo, 0.0, 1e-12, D, 11, dt)
        for _ in range(steps):
            t.sweep(1)
            s = t.mps()
            msd[c] += sum(i * O.join(s, d, s).real for i, d in enumerate(dens))
        s = t.mps()
        energy[c] = O.join(s, mpo, s).real
    return {"value": {"msd": msd[0], "energy": energy[0]},
            "grad": {"msd": GR.assemble(msd, h), "energy": GR.assemble(energy, h)}}


def test_energy_difference_is_exact_at_time_zero():
    """<psi|H(theta)|psi> is affine in (J, omega, g) at a fixed state, so the
    central difference over zero steps equals <H(theta + e_k)> - <H(theta)>."""
    n_mol, cutoff, D = 3, 4, 8
    ref = _oracle_fd(n_mol, cutoff, D, THETA, 0, 0.05, 1e-3)
    mps = H.random_mps(GR.holstein_chain(n_mol, cutoff, THETA), D, seed=1234)
    e = lambda th: O.join(mps, H.hamiltonian_mpo(GR.holstein_chain(n_mol, cutoff, th)), mps).real  # noqa: E731
    for k in GR.PARAMS:
        unit = dict(THETA, **{k: THETA[k] + 1.0})
        assert abs(ref["grad"]["energy"][k] - (e(unit) - e(THETA))) < 1e-9, k


@pytest.mark.gpu
def test_fd_gradient_matches_oracle():
    from kylin_v_gb300 import kvgpu

    kvgpu.init(0)
    n_mol, cutoff, D, steps, dt, h = 3, 4, 8, 3, 0.05, 1e-5
    got = GR.fd_gradient(n_mol, cutoff, D, THETA, steps=steps, dt=dt, h=h)
    ref = _oracle_fd(n_mol, cutoff, D, THETA, steps, dt, h)
    assert got["chains"] == 7
    # the differences are converged in h: the same to 1e-6 at h = 1e-4
    ref4 = _oracle_fd(n_mol, cutoff, D, THETA, steps, dt, 1e-4)
    for q in ("msd", "energy"):
        for k in GR.PARAMS:
            assert abs(ref4["grad"][q][k] - ref["grad"][q][k]) < 1e-6 * max(1.0, abs(ref["grad"][q][k]))
    for q in ("msd", "energy"):
        assert abs(got["value"][q] - ref["value"][q]) < 1e-9 * max(1.0, abs(ref["value"][q])), q
        for k in GR.PARAMS:
            a, b = got["grad"][q][k], ref["grad"][q][k]
            assert abs(a - b) < 1e-5 * max(1.0, abs(b)), (q, k, a, b)


@pytest.mark.gpu
def test_adjoint_energy_gradient():
    """Reverse mode through the environment adjoints with the parameter-linear
    MPO: dE/dtheta equals the oracle's exact affine differences at a fixed
    state, equals the central differences of <H> after three one-site TDVP
    steps (which conserve it), and comes out of torch.autograd."""
    import torch

    from kylin_v_gb300 import kvgpu

    kvgpu.init(0)
    n_mol, cutoff, D = 3, 4, 8
    ch = GR.holstein_chain(n_mol, cutoff, THETA)
    mps = H.random_mps(ch, D, seed=1234)
    r = GR.energy_gradient_adjoint(ch, mps)
    e = lambda th: O.join(mps, H.hamiltonian_mpo(GR.holstein_chain(n_mol, cutoff, th)), mps).real  # noqa: E731
    assert abs(r["value"] - e(THETA)) < 1e-10
    for k in GR.PARAMS:
        exact = e(dict(THETA, **{k: THETA[k] + 1.0})) - e(THETA)
        assert abs(r["grad"][k] - exact) <= 1e-10 * max(1.0, abs(exact)), k
    fd = GR.fd_gradient(n_mol, cutoff, D, THETA, steps=3, dt=0.05, h=1e-5)
    for k in GR.PARAMS:
        assert abs(r["grad"][k] - fd["grad"]["energy"][k]) <= 1e-5 * max(1.0, abs(r["grad"][k])), k
    f = GR.torch_energy(lambda th: GR.holstein_chain(n_mol, cutoff, th))
    theta = torch.tensor([THETA[k] for k in GR.PARAMS], dtype=torch.float64, requires_grad=True)
    out = f.apply(theta, mps)
    out.backward()
    assert abs(out.item() - r["value"]) < 1e-12
    assert np.allclose(theta.grad.numpy(), [r["grad"][k] for k in GR.PARAMS], rtol=1e-12, atol=1e-12)
