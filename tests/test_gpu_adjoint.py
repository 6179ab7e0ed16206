"""kv_adjoint_heff / kv_adjoint_env against the oracle's forward maps.

For y = H_eff(L, W1, W2, R) psi, multilinear in its operands, the cotangent
xbar of each operand x must satisfy Re<ybar, y(x -> dx)> = Re<xbar, dx> for
every direction dx; the environment update is quadratic in A, so there the
left side is the central difference (f(A + h dA) - f(A - h dA)) / 2h, exact for
a quadratic.  The forward side runs on the CPU oracle, the cotangents on the
GPU; agreement to 1e-10 relative (FP64), 1e-7 (mixed)."""
import os

import numpy as np
import pytest

import kvtest_util as U

U.load_package()
O = U.load_oracle()
from kylin_v_gb300 import kvio  # noqa: E402
from kylin_v_gb300.kvio import BlockTensor  # noqa: E402

pytestmark = pytest.mark.gpu
G = U.GOLDEN
OPS = [(c, d) for c in ("tiny1", "tiny2m") for d in sorted(os.listdir(os.path.join(G, c))) if d.startswith("ops_site")]


@pytest.fixture(scope="module")
def gpu():
    from kylin_v_gb300 import kvgpu

    kvgpu.init(0)
    return kvgpu


def _rand_like(t, rng):
    return BlockTensor(t.dirs, [(q, rng.normal(size=a.shape) + 1j * rng.normal(size=a.shape)) for q, a in t.blocks])


def _axpy(x, s, y):
    """x + s*y (same block structure)"""
    return BlockTensor(x.dirs, [(q, a + s * b) for (q, a), (_, b) in zip(x.blocks, y.blocks)])


def _inner(x, y):
    """<x, y> over the blocks of y (x may hold more blocks)"""
    dx = {(q, a.shape): a for q, a in x.blocks}
    return sum(np.vdot(dx[(q, a.shape)], a) for q, a in y.blocks if (q, a.shape) in dx)


def _cases(case, d):
    mps, mpo = kvio.read_mps(f"{G}/{case}/in.mps"), kvio.read_mpo(f"{G}/{case}/H.mpo")
    rd = lambda n: kvio.read_kvt(f"{G}/{case}/{d}/{n}.kvt")  # noqa: E731
    i = int(d[len("ops_site"):])
    L, R, R2 = rd("envL"), rd("envR"), rd("envR2")
    A, W, W2 = mps[i], mpo[i], mpo[i + 1]
    mm = O.product(A, mps[i + 1], 1)
    heff = [(1, L, A, W, None, R), (2, L, mm, W, W2, R2), (0, rd("envL_next"), rd("svd21_V"), None, None, R)]
    return heff, (L, R, A, W)


@pytest.mark.parametrize("case,d", OPS)
@pytest.mark.parametrize("prec", [0, 1])
def test_adjoint_heff(gpu, case, d, prec):
    rng = np.random.default_rng(11)
    heff, _ = _cases(case, d)
    tol = 1e-10 if prec == 0 else 1e-7
    for nsite, L, psi, W1, W2, R in heff:
        scale = 0.025
        y = O.apply(nsite, L, psi, W1, W2, R)
        yb = _rand_like(y, rng)
        g = gpu.adjoint_heff(nsite, L, psi, W1, W2, R, yb, scale=scale, precision=prec)
        args = {"L": L, "psi": psi, "W1": W1, "W2": W2, "R": R}
        expect = {"psi", "L", "R"} | ({"W1"} if nsite >= 1 else set()) | ({"W2"} if nsite == 2 else set())
        assert set(g) == expect
        for k, xb in g.items():
            dx = _rand_like(args[k], rng)
            a2 = dict(args, **{k: dx})
            lhs = scale * _inner(yb, O.apply(nsite, a2["L"], a2["psi"], a2["W1"], a2["W2"], a2["R"])).real
            rhs = _inner(xb.to_host(), dx).real
            assert abs(lhs - rhs) <= tol * max(1.0, abs(lhs)), (nsite, k, lhs, rhs)


@pytest.mark.parametrize("case,d", OPS)
@pytest.mark.parametrize("l2r", [True, False])
def test_adjoint_env(gpu, case, d, l2r):
    rng = np.random.default_rng(12)
    _, (L, R, A, W) = _cases(case, d)
    env = L if l2r else R
    out = O.env_sweep(env, A, W, l2r)
    eb = _rand_like(out, rng)
    g = gpu.adjoint_env(env, A, W, l2r, eb)
    args = {"env": env, "A": A, "W": W}
    for k, xb in g.items():
        dx = _rand_like(args[k], rng)
        h = 0.5
        ap, am = dict(args), dict(args)
        ap[k], am[k] = _axpy(args[k], h, dx), _axpy(args[k], -h, dx)
        fp = O.env_sweep(ap["env"], ap["A"], ap["W"], l2r)
        fm = O.env_sweep(am["env"], am["A"], am["W"], l2r)
        lhs = (_inner(eb, fp) - _inner(eb, fm)).real / (2 * h)
        rhs = _inner(xb.to_host(), dx).real
        assert abs(lhs - rhs) <= 1e-10 * max(1.0, abs(lhs)), (k, lhs, rhs)


def test_adjoint_subset_and_errors(gpu):
    heff, _ = _cases("tiny1", sorted(d for _, d in OPS if _ == "tiny1")[0])
    nsite, L, psi, W1, W2, R = heff[0]
    yb = _rand_like(O.apply(nsite, L, psi, W1, W2, R), np.random.default_rng(1))
    g = gpu.adjoint_heff(nsite, L, psi, W1, W2, R, yb, want=("W1",))
    assert set(g) == {"W1"}
    with pytest.raises(gpu.KvError):  # rank of ybar does not match nsite
        gpu.adjoint_heff(2, L, psi, W1, W1, R, yb)
