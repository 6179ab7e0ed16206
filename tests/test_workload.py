"""Workload generators (host side): random MPS and Holstein MPOs."""
import numpy as np
import pytest

import kvtest_util as U

U.load_package()
from kylin_v_gb300 import holstein as H  # noqa: E402


@pytest.mark.parametrize("name", ["holstein-1site-L8", "holstein-2site-L32"])
def test_random_mps_is_normalised_right_canonical(name):
    ch, D, _ = H.config_chain(name)
    mps = H.random_mps(ch, D, seed=1234)
    assert len(mps) == ch.n_sites
    assert abs(mps[0].norm() - 1.0) < 1e-12
    for s in range(1, ch.n_sites):
        by = {}
        for q, a in mps[s].blocks:
            assert np.isfinite(a).all()
            assert q[0] + q[1] == q[2]  # U(1): left + physical = right
            by.setdefault(q[0], []).append(a[:, 0, :])
        for mats in by.values():
            m = np.concatenate(mats, axis=1)
            assert np.abs(m @ m.conj().T - np.eye(m.shape[0])).max() < 1e-12
    bonds = [sum(t.legs()[2].values()) for t in mps[:-1]]
    assert max(bonds) == D


def test_random_mps_is_seeded():
    ch, D, _ = H.config_chain("holstein-1site-L8")
    a, b = H.random_mps(ch, D, seed=5), H.random_mps(ch, D, seed=5)
    for x, y in zip(a, b):
        for (q1, m1), (q2, m2) in zip(x.blocks, y.blocks):
            assert q1 == q2 and np.array_equal(m1, m2)


def test_hamiltonian_mpo_bond_sectors():
    ch, _, _ = H.config_chain("holstein-2site-L32")
    mpo = H.hamiltonian_mpo(ch)
    # MPO bond dimension <= 7 (FSM states), charges in {-1, 0, 1}
    for t in mpo:
        legs = t.legs()
        assert set(legs[3]) <= {-1, 0, 1} and sum(legs[3].values()) <= 7
        for q, a in t.blocks:
            assert q[0] + q[1] == q[2] + q[3]
