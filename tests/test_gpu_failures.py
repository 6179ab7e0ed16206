"""Failure paths of the C ABI, each in a form that faults nothing on the GPU:
non-finite inputs (made on the host) end in KV_ENONFINITE, malformed block
lists and arguments in KV_EINVAL / KV_EMISMATCH, and a tensor-core GEMM whose
copies are withheld (kv_debug_gemm_stall: its first bounded wait runs out
with nothing in flight) in KV_ETIMEOUT.  After every failure the next normal
call succeeds and matches the oracle."""
import ctypes
import os

import numpy as np
import pytest

import kvtest_util as U

U.load_package()
from kylin_v_gb300 import kvio  # noqa: E402

pytestmark = pytest.mark.gpu
G_DIR = os.path.join(U.GOLDEN, "tiny1")
EINVAL, ENONFINITE, ETIMEOUT, EMISMATCH = -1, -4, -5, -7


@pytest.fixture(scope="module")
def gpu():
    from kylin_v_gb300 import kvgpu

    kvgpu.init(0)
    return kvgpu


@pytest.fixture(scope="module")
def site():
    mps = kvio.read_mps(os.path.join(G_DIR, "in.mps"))
    mpo = kvio.read_mpo(os.path.join(G_DIR, "H.mpo"))
    d = os.path.join(G_DIR, "ops_site4")
    return dict(mps=mps, mpo=mpo, L=kvio.read_kvt(os.path.join(d, "envL.kvt")),
                R=kvio.read_kvt(os.path.join(d, "envR.kvt")), A=mps[4], W=mpo[4])


def _with_nan(t):
    blocks = [(q, a.copy()) for q, a in t.blocks]
    blocks[0][1].flat[0] = np.nan
    return kvio.BlockTensor(t.dirs, blocks)


def _code(e):
    return e.value.code


def _check_recovered(gpu, site):
    """A normal FP64 and mixed call right after a failure: both match the oracle."""
    O = U.load_oracle()
    ref = O.product(site["A"], site["mps"][5], 1)
    for prec, tol in ((gpu.KV_FP64, 1e-12), (gpu.KV_MIXED_3M_DIGITS, 1e-7)):
        out = gpu.product(site["A"], site["mps"][5], 1, precision=prec).to_host()
        assert U.tensor_diff(out, ref) <= tol * U.tensor_scale(ref)


@pytest.mark.parametrize("prec", [0, 1])
def test_nan_in_psi_is_nonfinite(gpu, site, prec):
    s = site
    with pytest.raises(gpu.KvError) as e:
        gpu.local_krylov(1, s["L"], _with_nan(s["A"]), s["W"], None, s["R"], 0.05, 11, 1e-8, precision=prec)
    assert _code(e) == ENONFINITE
    _check_recovered(gpu, site)


@pytest.mark.parametrize("prec", [0, 1])
def test_nan_in_environment_is_nonfinite(gpu, site, prec):
    s = site
    with pytest.raises(gpu.KvError) as e:
        gpu.local_krylov(1, _with_nan(s["L"]), s["A"], s["W"], None, s["R"], 0.05, 11, 1e-8, precision=prec)
    assert _code(e) == ENONFINITE
    _check_recovered(gpu, site)


def test_nan_operand_of_mixed_product_is_nonfinite(gpu, site):
    """The digit slicer has no fixed-point code for Inf/NaN: it flags the row."""
    with pytest.raises(gpu.KvError) as e:
        gpu.product(_with_nan(site["A"]), site["mps"][5], 1, precision=gpu.KV_MIXED_3M_DIGITS)
    assert _code(e) == ENONFINITE and "Inf or NaN" in str(e.value)
    _check_recovered(gpu, site)


@pytest.mark.parametrize("prec", [0, 1])
def test_nan_in_svd_input_is_nonfinite(gpu, site, prec):
    with pytest.raises(gpu.KvError) as e:
        gpu.svd_impl(_with_nan(site["A"]), 2, True, 1e-8, 8, precision=prec)
    assert _code(e) == ENONFINITE
    _check_recovered(gpu, site)


def _create(L, rank, dirs, shapes, qns):
    out = ctypes.c_void_p()
    nb = len(shapes) // max(1, rank)
    rc = L.kv_tensor_create(rank, (ctypes.c_int * max(1, len(dirs)))(*dirs), nb,
                            (ctypes.c_int * max(1, len(shapes)))(*shapes), (ctypes.c_int * max(1, len(qns)))(*qns),
                            None, ctypes.byref(out))
    if rc == 0:
        L.kv_tensor_free(out)
    return rc


def test_malformed_block_lists_are_rejected(gpu, site):
    L = gpu.lib()
    assert _create(L, 3, [1, 1, -1], [2, 1, 3], [0, 0, 0]) == 0
    assert _create(L, 3, [1, 2, -1], [2, 1, 3], [0, 0, 0]) == EINVAL      # direction not +-1
    assert _create(L, 3, [1, 1, -1], [2, 0, 3], [0, 0, 0]) == EINVAL      # empty leg
    assert _create(L, 3, [1, 1, -1], [2, -1, 3], [0, 0, 0]) == EINVAL     # negative extent
    assert _create(L, 7, [1] * 7, [1] * 7, [0] * 7) == EINVAL             # rank above 6
    assert _create(L, 0, [], [], []) == EINVAL                            # rank 0
    out = ctypes.c_void_p()
    rc = L.kv_tensor_create(3, (ctypes.c_int * 3)(1, 1, -1), -2, None, None, None, ctypes.byref(out))
    assert rc == EINVAL                                                   # negative block count
    assert b"" != L.kv_last_error()
    _check_recovered(gpu, site)


def test_bad_arguments_are_rejected(gpu, site):
    s = site
    A = gpu.Tensor.from_host(s["A"])
    B = gpu.Tensor.from_host(s["mps"][5])
    # contracted legs whose directions do not pair: A's last leg (-1) against
    # the right environment's first leg (-1)
    with pytest.raises(gpu.KvError) as e:
        gpu.product(A, gpu.Tensor.from_host(s["R"]), 1)
    assert _code(e) == EMISMATCH
    with pytest.raises(gpu.KvError) as e:
        gpu.product(A, B, 3)          # contracts every leg: no output leg
    assert _code(e) == EINVAL
    with pytest.raises(gpu.KvError) as e:
        gpu.product(A, B, 1, precision=9)
    assert _code(e) == EINVAL
    with pytest.raises(gpu.KvError) as e:
        gpu.svd_impl(A, 0, True, 1e-8, 8)
    assert _code(e) == EINVAL
    with pytest.raises(gpu.KvError) as e:
        gpu.local_krylov(1, s["L"], s["A"], s["W"], None, s["R"], 0.05, 40, 1e-8)  # Krylov dimension above 32
    assert _code(e) == EINVAL
    with pytest.raises(gpu.KvError) as e:
        gpu.TDVP(s["mps"][:1], s["mpo"][:1], 1e-8, 1e-8, 8, 11, 0.05)
    assert _code(e) == EINVAL
    t = gpu.TDVP(s["mps"], s["mpo"], 1e-8, 1e-8, 8, 11, 0.05)
    with pytest.raises(gpu.KvError) as e:
        t.sweep(5)
    assert _code(e) == EINVAL
    _check_recovered(gpu, site)


def test_withheld_copies_time_out_and_the_next_call_succeeds(gpu, site):
    """Every bounded mbarrier wait of the tensor-core GEMM gives up after its
    limit; with copies withheld the MMA warp's first wait runs out before any
    copy or MMA is in flight, the kernel frees its tensor memory, and the call
    reports KV_ETIMEOUT.  The GEMM then runs normally again."""
    L = gpu.lib()
    gpu.check(L.kv_debug_gemm_stall(1))
    try:
        with pytest.raises(gpu.KvError) as e:
            gpu.product(site["A"], site["mps"][5], 1, precision=gpu.KV_MIXED_3M_DIGITS)
        assert _code(e) == ETIMEOUT
    finally:
        gpu.check(L.kv_debug_gemm_stall(0))
    _check_recovered(gpu, site)
    # a whole mixed sweep afterwards
    t = gpu.TDVP(site["mps"], site["mpo"], 1e-8, 1e-8, 8, 11, 0.05, gpu.KV_MIXED_3M_DIGITS)
    t.two_site()
