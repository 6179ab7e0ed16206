"""kv_sweep_batched: independent disordered chains advanced concurrently on
worker streams leave exactly the site tensors that a loop of single-chain
sweeps leaves (bit for bit, FP64 and mixed, one- and two-site), and its
argument checks return status codes."""
import numpy as np
import pytest

import kvtest_util as U

U.load_package()
from kylin_v_gb300 import holstein as H  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from kylin_v_gb300 import kvgpu

    kvgpu.init(0)
    return kvgpu


def _chains(n, seed=77):
    """Small members of the disordered ensemble: L in [3, 6], D in {8, 16, 24},
    eps ~ N(0, 0.5^2), omega = 1, g in [0.5, 1.5], cutoff 4."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        L = int(rng.integers(3, 7))
        D = int(rng.choice([8, 16, 24]))
        ch = H.HolsteinChain(L, [1.0], [[float(x)] for x in rng.uniform(0.5, 1.5, L)], cutoff=4,
                             eps=list(rng.normal(0.0, 0.5, L)))
        out.append((ch, D, H.random_mps(ch, D, seed=1234 + i), H.hamiltonian_mpo(ch)))
    return out


def _same(a, b):
    ha, hb = a.to_host(), b.to_host()
    if len(ha.blocks) != len(hb.blocks):
        return False
    return all(qa == qb and np.array_equal(xa, xb) for (qa, xa), (qb, xb) in zip(ha.blocks, hb.blocks))


@pytest.mark.parametrize("mode,prec", [(1, 0), (2, 0), (1, 1), (2, 1)])
def test_batched_equals_sequential(gpu, mode, prec):
    steps = 2
    cs = _chains(6)
    make = lambda: [gpu.TDVP(m, w, 1e-8, 1e-8, D, 11, 0.05, prec) for _, D, m, w in cs]  # noqa: E731
    seq, bat = make(), make()
    for t in seq:
        for _ in range(steps):
            t.two_site() if mode == 2 else t.one_site()
    ms = gpu.sweep_batched(bat, mode, steps, max_streams=3)
    assert ms > 0.0
    for i, (a, b) in enumerate(zip(seq, bat)):
        for j in range(a.ns):
            assert _same(a.site(j), b.site(j)), (i, j)
    # a second call on the same chains (plans now cached on the workers)
    for t in seq:
        t.two_site() if mode == 2 else t.one_site()
    gpu.sweep_batched(bat, mode, 1, max_streams=3)
    for a, b in zip(seq, bat):
        assert all(_same(a.site(j), b.site(j)) for j in range(a.ns))


def test_batched_more_streams_than_chains(gpu):
    cs = _chains(2, seed=5)
    seq = [gpu.TDVP(m, w, 1e-8, 1e-8, D, 11, 0.05) for _, D, m, w in cs]
    bat = [gpu.TDVP(m, w, 1e-8, 1e-8, D, 11, 0.05) for _, D, m, w in cs]
    for t in seq:
        t.one_site()
    gpu.sweep_batched(bat, 1, 1, max_streams=16)
    for a, b in zip(seq, bat):
        assert all(_same(a.site(j), b.site(j)) for j in range(a.ns))


def test_batched_errors(gpu):
    cs = _chains(2, seed=9)
    ts = [gpu.TDVP(m, w, 1e-8, 1e-8, D, 11, 0.05) for _, D, m, w in cs]
    with pytest.raises(gpu.KvError):
        gpu.sweep_batched(ts, 3, 1)
    with pytest.raises(gpu.KvError):
        gpu.sweep_batched([ts[0], ts[0]], 1, 1)
    with pytest.raises(gpu.KvError):
        gpu.sweep_batched(ts, 1, -1)
    assert gpu.sweep_batched([], 1, 1) == 0.0
    assert gpu.sweep_batched(ts, 1, 0) == 0.0


def test_batched_large_bond(gpu):
    """Chains at the benchmark's bond dimension (D = 128, where the two-site
    sectors reach 128 x 128 and the register-resident Jacobi runs) and D = 64,
    two-site mixed steps: batched equals sequential bit for bit."""
    chains = [(H.HolsteinChain(4, [1.0], [[1.0]] * 4, cutoff=8), 128),
              (H.HolsteinChain(3, [0.6], [[0.8]] * 3, cutoff=8, eps=[0.2, -0.1, 0.0]), 64)]
    host = [(H.random_mps(ch, D, seed=99 + i), H.hamiltonian_mpo(ch), D) for i, (ch, D) in enumerate(chains)]
    make = lambda: [gpu.TDVP(m, w, 1e-8, 1e-8, D, 11, 0.05, gpu.KV_MIXED_3M_DIGITS) for m, w, D in host]  # noqa: E731
    seq, bat = make(), make()
    for t in seq:
        for _ in range(2):
            t.two_site()
    gpu.sweep_batched(bat, 2, 2, max_streams=2)
    assert max(sum(s.to_host().legs()[2].values()) for s in seq[0].sites()[:-1]) == 128
    for i, (a, b) in enumerate(zip(seq, bat)):
        for j in range(a.ns):
            assert _same(a.site(j), b.site(j)), (i, j)


def test_batched_sa_equals_sequential(gpu):
    """SA-1TDVP sweeps (mode 3) through kv_sweep_batched leave the tensors a
    loop of single-chain SA sweeps leaves: each chain draws from its own seed
    stream, whichever worker runs it."""
    cs = _chains(4, seed=5)
    def make():
        ts = [gpu.TDVP(m, w, 1e-8, 1e-8, 2 * D, 11, 0.05, gpu.KV_MIXED_3M_DIGITS) for _, D, m, w in cs]
        for i, (t, (ch, _, _, _)) in enumerate(zip(ts, cs)):
            t.set_sa([4.0] * (ch.n_sites - 1), 11 + i)
        return ts
    seq, bat = make(), make()
    for t in seq:
        for _ in range(2):
            t.sweep(3)
    gpu.sweep_batched(bat, 3, 2, max_streams=3)
    assert sum(t.sa_added() for t in seq) > 0
    for i, (a, b) in enumerate(zip(seq, bat)):
        for j in range(a.ns):
            assert _same(a.site(j), b.site(j)), (i, j)
