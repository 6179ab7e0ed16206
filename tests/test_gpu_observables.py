"""Site observables on the device (kv_local_expectations): every exciton
population of a chain from one left and one right pass of identity
environments equals <psi|D_j|psi> of the full contraction (kv_expectation,
Operator::join with the reference's density MPO) for canonical, evolved and
non-canonical states, FP64."""
import os

import numpy as np
import pytest

import kvtest_util as U

U.load_package()
from kylin_v_gb300 import holstein as H  # noqa: E402
from kylin_v_gb300 import kvio  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from kylin_v_gb300 import kvgpu

    kvgpu.init(0)
    return kvgpu


def _chain(case):
    import sys

    sys.path.insert(0, U.GOLDEN)
    import make_golden as MG

    return MG.cases()[case]["chain"], U.manifest()[case]


@pytest.mark.parametrize("case", ["tiny1", "tiny2m", "l8c8d32"])
def test_local_expectations_equal_full_contractions(gpu, case):
    ch, ent = _chain(case)
    mps = H.random_mps(ch, ent["D"], seed=ent["seed"])
    mpo = H.hamiltonian_mpo(ch)
    ident = [gpu.Tensor.from_host(x) for x in H.identity_mpo(ch)]
    rng = np.random.default_rng(4)
    bent = [kvio.BlockTensor(t.dirs, [(q, a * (1.0 + 0.3 * rng.standard_normal(a.shape))) for q, a in t.blocks])
            for t in mps]
    t = gpu.TDVP(mps, mpo, 1e-8, 1e-8, ent["D"], 11, 0.05)
    t.one_site()
    for state in (mps, bent, t.sites()):
        sites = ch.exciton_sites()
        dens = [H.density_mpo(ch, j) for j in sites]
        ops = [(j, gpu.Tensor.from_host(d[j])) for j, d in zip(sites, dens)]
        got = gpu.local_expectations(state, ident, ops)
        for (j, _), d, v in zip(ops, dens, got):
            ref = gpu.expectation(state, [gpu.Tensor.from_host(x) for x in d], state)
            assert abs(v - ref) <= 1e-12 * max(1.0, abs(ref)), (j, v, ref)
