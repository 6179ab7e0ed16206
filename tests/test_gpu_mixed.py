"""Mixed-precision contractions (tcgen05 FP16 digit products with exact
FP32 accumulation, kv_tc.cu) against the FP64 path of the same library and
against the reference's golden vectors.

Each real operand value is a 38-bit fixed-point integer relative to its
GEMM row's (A) or column's (B) largest entry, split into five base-256
digits; digit products of orders 0..4 are accumulated exactly.  The error of
an output entry is therefore below ~2^-33 of max|A_row| max|B_col| summed
over K, which for these inputs is < 5e-10 of the largest output entry (REL);
integer-valued inputs are reproduced bit for bit."""
import numpy as np
import pytest

import kvtest_util as U

U.load_package()
from kylin_v_gb300 import kvio  # noqa: E402

pytestmark = pytest.mark.gpu
G = U.GOLDEN
REL = 5e-10


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
    assert _rel(D2.to_host(), D1.to_host()) < REL


def _segmented_pair(rng, integer):
    """A (x, s, k) and B (s, k, y): each output block (x, y) sums six block
    pairs (one per s) of K = 90 .. 700 (beyond one 336-step drain), every
    pair rescaled by 2^u on A and 2^-u on B so the pairs' row and column
    exponents differ while the product does not change."""
    Ks = [90, 95, 400, 100, 700, 17]
    us = [0, 3, -4, 5, -2, 1]
    val = (lambda sh: rng.integers(-9, 10, sh) + 1j * rng.integers(-9, 10, sh)) if integer else \
        (lambda sh: rng.standard_normal(sh) + 1j * rng.standard_normal(sh))
    rows = {x: 2.0 ** rng.integers(-20, 21, 60 + 40 * x) for x in range(2)}  # per-row scales of A
    cols = {y: 2.0 ** rng.integers(-20, 21, 40 + 30 * y) for y in range(2)}  # per-column scales of B
    if integer:
        rows = {x: np.ones_like(v) for x, v in rows.items()}
        cols = {y: np.ones_like(v) for y, v in cols.items()}
    ablk, bblk = [], []
    for x in range(2):
        for s, (K, u) in enumerate(zip(Ks, us)):
            a = val((60 + 40 * x, 1, K)) * rows[x][:, None, None] * 2.0 ** u
            ablk.append(((x, s, s + x), a))
    for s, (K, u) in enumerate(zip(Ks, us)):
        for x in range(2):
            for y in range(2):
                b = val((1, K, 40 + 30 * y)) * cols[y][None, None, :] * 2.0 ** (-u)
                bblk.append(((s, s + x, y), b))
    A = kvio.BlockTensor((1, 1, 1), ablk)
    B = kvio.BlockTensor((-1, -1, 1), bblk)
    # the same product as conj-transposed A (legs s, k, x) and transposed B (legs y, s, k)
    At = kvio.BlockTensor((1, 1, -1), [((q[1], q[2], q[0]), np.conj(np.transpose(a, (1, 2, 0)))) for q, a in ablk])
    Bt = kvio.BlockTensor((1, 1, 1), [((q[2], q[0], q[1]), np.transpose(b, (2, 0, 1))) for q, b in bblk])
    return A, B, At, Bt, rows, cols


def test_mixed_product_exact_on_integers(gpu):
    rng = np.random.default_rng(11)
    A, B, At, Bt, _, _ = _segmented_pair(rng, integer=True)
    ref = gpu.product(A, B, 2, precision=gpu.KV_FP64).to_host().as_dict()
    mix = gpu.product(A, B, 2, precision=gpu.KV_MIXED_TF32).to_host().as_dict()
    mix_t = gpu.product(At, Bt, 2, opA=gpu.OP_C, opB=gpu.OP_T, precision=gpu.KV_MIXED_TF32).to_host().as_dict()
    assert set(ref) == set(mix) == set(mix_t) and len(ref) == 4
    for q in ref:
        assert np.array_equal(ref[q], mix[q])
        assert np.array_equal(ref[q], mix_t[q])


def test_mixed_product_row_column_dynamic_range(gpu):
    """Rows of A and columns of B spanning 2^+-20: the error of every entry is
    small relative to its own row and column scale, not the block's."""
    rng = np.random.default_rng(12)
    A, B, At, Bt, rows, cols = _segmented_pair(rng, integer=False)
    ref = gpu.product(A, B, 2, precision=gpu.KV_FP64).to_host().as_dict()
    for P in (gpu.product(A, B, 2, precision=gpu.KV_MIXED_TF32),
              gpu.product(At, Bt, 2, opA=gpu.OP_C, opB=gpu.OP_T, precision=gpu.KV_MIXED_TF32)):
        mix = P.to_host().as_dict()
        for q, r in ref.items():
            x, y = q[0][0], q[0][1]  # as_dict keys are (charges, shape)
            sc = rows[x][:, None] * cols[y][None, :]
            r2 = r.reshape(sc.shape) / sc
            m2 = mix[q].reshape(sc.shape) / sc
            assert np.abs(m2 - r2).max() < REL * np.abs(r2).max()


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
    assert _rel(k2.to_host(), rd("k2")) < 1e-7


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


@pytest.mark.parametrize("l2r", [True, False])
def test_mixed_svd_sector_scales_and_ranks(gpu, l2r):
    """Charge sectors of very different norms (1 down to 1e-30, and an exactly
    zero one) and numerical ranks, tall and wide, in one tensor, nothing
    truncated (cutoff 0): every singular value above the mixed path's floor
    (1e-6 of its sector's largest) is kept, and U.V reproduces each block to
    1e-5 of that block's own scale."""
    rng = np.random.default_rng(7)
    # rank-3 tensor (l, s, r) with dirs (+1, +1, -1); one block per charge sector
    specs = [(40, 24, 1.0, 24), (24, 40, 1e-5, 10), (64, 64, 1e-12, 30), (30, 50, 1e-18, 5),
             (20, 20, 1e-30, 20), (16, 16, 0.0, 16)]
    blocks, expect = [], 0
    for q, (m, n, scale, rank) in enumerate(specs):
        x = (rng.standard_normal((m, rank)) + 1j * rng.standard_normal((m, rank))) @ \
            np.diag(np.logspace(0, -4, rank)) @ (rng.standard_normal((rank, n)) + 1j * rng.standard_normal((rank, n)))
        x *= scale
        sv = np.linalg.svd(x, compute_uv=False)
        if scale > 0:
            expect += int((sv > 2e-6 * sv[0]).sum())
        blocks.append(((q, 0, q), x.reshape(m, 1, n)))
    t = kvio.BlockTensor((1, 1, -1), blocks)
    u, v, nk, nt = gpu.svd_impl(t, 2 if l2r else 1, l2r, 0.0, 10000, precision=gpu.KV_MIXED_TF32)
    assert nt == sum(min(m, n) for m, n, _, _ in specs)
    assert nk >= expect
    prod = gpu.product(u, v, 1).to_host().as_dict()
    for (qn, a) in blocks:
        if not np.abs(a).max() > 0:
            continue
        b = prod.get((qn, a.shape))
        assert b is not None, qn
        assert np.abs(a - b).max() <= 1e-5 * np.abs(a).max(), qn
