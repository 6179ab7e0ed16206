"""Mixed-precision (tcgen05, 3M with TF32 hi/lo split, FP32 accumulation)
contractions against the FP64 path of the same library and against the
reference's golden vectors.  Tolerance relative to the largest output entry:
the split keeps ~22 mantissa bits (~2e-7); FP32 accumulation adds about
6e-8 * sqrt(K) for a sum of K products, so 3e-6 for the short contractions
of the fixtures and 1e-5 for the ~500-term sums of the synthetic product."""
import numpy as np
import pytest

import kvtest_util as U

U.load_package()
from kylin_v_gb300 import kvio  # noqa: E402

pytestmark = pytest.mark.gpu
G = U.GOLDEN
REL = 3e-6


@pytest.fixture(scope="module")
def gpu():
    from kylin_v_gb300 import kvgpu

    kvgpu.init(0)
    return kvgpu


def _rand_tensor(rng, dirs, blocks):
    return kvio.BlockTensor(tuple(dirs), [(q, rng.standard_normal(sh) + 1j * rng.standard_normal(sh))
                                          for q, sh in blocks])


def _rel(a, b):
    return U.tensor_diff(a, b) / max(U.tensor_scale(b), 1e-300)


def test_mixed_product_matches_fp64(gpu):
    rng = np.random.default_rng(7)
    # A: (x, k) legs; B: (k, y); several charge sectors, odd sizes, multi-pair outputs
    blocks_a, blocks_b = [], []
    for q in range(3):
        for s in range(2):
            blocks_a.append(((q, s, q + s), (37 + 50 * q, 1, 29 + 20 * s)))
    for q in range(3):
        for s in range(2):
            for t in range(2):
                blocks_b.append(((q + s, t, q + s + t), (29 + 20 * s, 1, 70 + 13 * t)))
    A = _rand_tensor(rng, (1, 1, -1), blocks_a)
    B = _rand_tensor(rng, (1, 1, -1), blocks_b)
    ref = gpu.product(A, B, 1, precision=gpu.KV_FP64).to_host()
    mix = gpu.product(A, B, 1, precision=gpu.KV_MIXED_TF32).to_host()
    assert _rel(mix, ref) < REL
    # conjugate-transposed A (env update form) and transposed B (apply form)
    C1 = gpu.product(A, A, 2, opA=gpu.OP_C, opB=gpu.OP_N, precision=gpu.KV_FP64).to_host()
    C2 = gpu.product(A, A, 2, opA=gpu.OP_C, opB=gpu.OP_N, precision=gpu.KV_MIXED_TF32).to_host()
    assert _rel(C2, C1) < REL
    Bf = kvio.BlockTensor((-1, -1, 1), B.blocks)  # legs contracted against B need opposite directions
    D1 = gpu.product(B, Bf, 2, opA=gpu.OP_N, opB=gpu.OP_T, precision=gpu.KV_FP64)
    D2 = gpu.product(B, Bf, 2, opA=gpu.OP_N, opB=gpu.OP_T, precision=gpu.KV_MIXED_TF32)
    assert _rel(D2.to_host(), D1.to_host()) < 1e-5  # ~500 products per output entry


@pytest.mark.parametrize("case,site", [("tiny1", 1), ("tiny1", 4), ("tiny2m", 2), ("tiny2m", 6)])
def test_mixed_heff_matches_reference(gpu, case, site):
    mps, mpo = kvio.read_mps(f"{G}/{case}/in.mps"), kvio.read_mpo(f"{G}/{case}/H.mpo")
    rd = lambda n: kvio.read_kvt(f"{G}/{case}/ops_site{site}/{n}.kvt")  # noqa: E731
    L, R, R2 = rd("envL"), rd("envR"), rd("envR2")
    h1 = gpu.heff_apply(1, L, mps[site], mpo[site], None, R, precision=gpu.KV_MIXED_TF32).to_host()
    assert _rel(h1, rd("h1")) < REL
    h2 = gpu.heff_apply(2, L, rd("mm"), mpo[site], mpo[site + 1], R2, precision=gpu.KV_MIXED_TF32).to_host()
    assert _rel(h2, rd("h2")) < REL
    e = gpu.env_sweep(R, mps[site], mpo[site], False, precision=gpu.KV_MIXED_TF32).to_host()
    assert _rel(e, rd("envR_prev")) < REL
    k2, _ = gpu.local_krylov(2, L, rd("mm"), mpo[site], mpo[site + 1], R2, 0.05, 11, 1e-8,
                             precision=gpu.KV_MIXED_TF32)
    assert _rel(k2.to_host(), rd("k2")) < 1e-5


@pytest.mark.parametrize("case,site", [("tiny1", 1), ("tiny1", 4), ("tiny2m", 2), ("tiny2m", 6)])
def test_mixed_svd(gpu, case, site):
    """FP32 Jacobi + FP64 polish: the kept factor is orthonormal to FP64
    precision, U.V equals the reference's to the FP32 subspace accuracy, and
    the kept dimensions match."""
    O = U.load_oracle()
    mps = kvio.read_mps(f"{G}/{case}/in.mps")
    rd = lambda n: kvio.read_kvt(f"{G}/{case}/ops_site{site}/{n}.kvt")  # noqa: E731
    D = U.manifest()[case]["D"]
    for src, r1, l2r in ((mps[site], 2, True), (mps[site], 1, False), (rd("mm"), 2, True), (rd("mm"), 2, False)):
        u, v, nk, nt = gpu.svd_impl(src, r1, l2r, 1e-8, D, precision=gpu.KV_MIXED_TF32)
        uo, vo, so, nto = O.svd(src, r1, l2r, 1e-8, D)
        assert nk == len(so) and nt == nto
        uh, vh = u.to_host(), v.to_host()
        assert uh.legs()[-1] == uo.legs()[-1]
        prod = gpu.product(u, v, 1).to_host()
        assert _rel(prod, O.product(uo, vo, 1)) < 1e-5
        iso = O.product(uh, uh, r1, O.OP_C, O.OP_N) if l2r else O.product(vh, vh, src.rank - r1, O.OP_N, O.OP_C)
        for _, a in iso.as_dict().items():
            assert np.abs(a - np.eye(a.shape[0])).max() < 1e-12
