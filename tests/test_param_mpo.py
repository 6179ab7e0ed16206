"""The parameter-linear Hamiltonian MPO (holstein.hamiltonian_mpo_param):
its derivative tensors sit on the Hamiltonian's own block list, the sites are
affine in each parameter (so dW/dtheta is exact), and the energy derivative
assembled from them equals the central difference of <psi|H(theta)|psi>
computed by the oracle.  CPU only."""
import numpy as np
import pytest

import kvtest_util as U

U.load_package()
from kylin_v_gb300 import holstein as H  # noqa: E402

NAMES = ("J", "omega_0", "omega_1", "g_0", "g_1", "eps")


def _chain(theta):
    """Two modes: mode k has frequency omega_k and coupling g_k on every molecule."""
    g = [[theta["g_0"], theta["g_1"]] for _ in range(3)]
    return H.HolsteinChain(3, [theta["omega_0"], theta["omega_1"]], g, cutoff=3, J=theta["J"],
                           eps=[0.1 + theta["eps"], -0.2 + theta["eps"], 0.3 + theta["eps"]])


THETA = {"J": -1.0, "omega_0": 1.0, "omega_1": 0.4, "g_0": 0.9, "g_1": 0.6, "eps": 0.0}


@pytest.mark.parametrize("name", NAMES)
def test_sites_affine_on_one_block_list(name):
    W, dW = H.hamiltonian_mpo_param(_chain(THETA), NAMES)
    step = 0.37
    W2 = H.hamiltonian_mpo(_chain(dict(THETA, **{name: THETA[name] + step})))
    for s in range(len(W)):
        assert [q for q, _ in W[s].blocks] == [q for q, _ in dW[name][s].blocks] == [q for q, _ in W2[s].blocks]
        for (_, a), (_, d), (_, a2) in zip(W[s].blocks, dW[name][s].blocks, W2[s].blocks):
            assert np.abs(a + step * d - a2).max() < 1e-14


def test_energy_derivative_from_dW_matches_central_difference():
    """dE/dtheta_k = sum_s <psi| H with site s replaced by dW_k[s] |psi>."""
    O = U.load_oracle()
    ch = _chain(THETA)
    mps = H.random_mps(ch, 10, seed=3)
    W, dW = H.hamiltonian_mpo_param(ch, NAMES)
    h = 1e-5
    for name in NAMES:
        exact = sum(O.join(mps, W[:s] + [dW[name][s]] + W[s + 1:], mps).real for s in range(len(W)))
        ep = O.join(mps, H.hamiltonian_mpo(_chain(dict(THETA, **{name: THETA[name] + h}))), mps).real
        em = O.join(mps, H.hamiltonian_mpo(_chain(dict(THETA, **{name: THETA[name] - h}))), mps).real
        fd = (ep - em) / (2 * h)
        assert abs(exact - fd) <= 1e-8 * max(1.0, abs(fd)), (name, exact, fd)
