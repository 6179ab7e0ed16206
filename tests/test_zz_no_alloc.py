"""kv_expectation_noalloc: the allocation-free variant of kv_expectation.

It serves callers that cannot let the library allocate GPU memory (an
application owning all device memory through its own allocator, or a
latency-critical loop): all of its scratch lives in one fixed static device
array.  Called through the C ABI twice in a row, it must give the same
<a|W|b> as the existing entry point, to the FP64 tolerance the other GPU tests
use.  This file is collected last so a failure here never hides another
test's result; it passes alone in a fresh process as well."""
import ctypes
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


def _pool(G, reset):
    cur, high = ctypes.c_longlong(), ctypes.c_longlong()
    G.check(G.lib().kv_debug_pool_usage(int(reset), ctypes.byref(cur), ctypes.byref(high)))
    return cur.value, high.value


def _call(G, fn, bra, mpo, ket):
    ns = len(bra)
    arr = lambda hs: (ctypes.c_void_p * ns)(*[h.ptr for h in hs])  # noqa: E731
    re, im = ctypes.c_double(), ctypes.c_double()
    G.check(fn(ns, arr(bra), arr(mpo), arr(ket), ctypes.byref(re), ctypes.byref(im)))
    return complex(re.value, im.value)


@pytest.mark.parametrize("case", ["tiny1", "tiny2m", "l8c8d32"])
def test_noalloc_matches_existing_entry_point(gpu, case):
    G = gpu
    if case == "l8c8d32":
        ch, D, _ = H.config_chain("holstein-1site-L8")
        mps, mpo = H.random_mps(ch, D, seed=1234), H.hamiltonian_mpo(ch)
    else:
        g = os.path.join(U.GOLDEN, case)
        mps, mpo = kvio.read_mps(os.path.join(g, "in.mps")), kvio.read_mpo(os.path.join(g, "H.mpo"))
    a = [G.Tensor.from_host(t) for t in mps]
    w = [G.Tensor.from_host(t) for t in mpo]
    L = G.lib()
    ref = _call(G, L.kv_expectation, a, w, a)
    first = _call(G, L.kv_expectation_noalloc, a, w, a)
    before, _ = _pool(G, reset=True)
    second = _call(G, L.kv_expectation_noalloc, a, w, a)  # the scratch keeps the first call's contents
    after, high = _pool(G, reset=False)
    # nothing was taken from the device's memory pool during the second call
    assert after == before and high == before, (before, after, high)
    for v in (first, second):
        assert abs(v - ref) <= 1e-12 * max(1.0, abs(ref))
    # and on a second, different operator (the density of the first exciton site)
    if case != "tiny2m":
        ch = H.HolsteinChain(3, [1.0], [[1.0], [0.8], [1.2]], cutoff=4, eps=[0.1, -0.2, 0.3]) if case == "tiny1" \
            else H.config_chain("holstein-1site-L8")[0]
        d0 = [G.Tensor.from_host(t) for t in H.density_mpo(ch, 0)]
        r2 = _call(G, L.kv_expectation, a, d0, a)
        assert abs(_call(G, L.kv_expectation_noalloc, a, d0, a) - r2) <= 1e-12 * max(1.0, abs(r2))


def test_noalloc_rejects_oversized_input(gpu):
    """An input whose first environment (3000 x 1 x 3000 complex, 144 MB)
    exceeds the 64 MiB scratch fails with KV_ENOMEM and a clear message."""
    G = gpu
    rng = np.random.default_rng(0)
    big = 3000
    a0 = kvio.BlockTensor((1, 1, -1), [((0, 0, 0), rng.standard_normal((1, 1, big)) + 0j)])
    a1 = kvio.BlockTensor((1, 1, -1), [((0, 0, 0), rng.standard_normal((big, 1, 1)) + 0j)])
    w = kvio.BlockTensor((1, 1, -1, -1), [((0, 0, 0, 0), np.ones((1, 1, 1, 1), complex))])
    a = [G.Tensor.from_host(t) for t in (a0, a1)]
    ws = [G.Tensor.from_host(w), G.Tensor.from_host(w)]
    with pytest.raises(G.KvError) as e:
        _call(G, G.lib().kv_expectation_noalloc, a, ws, a)
    assert e.value.code == -3 and "64 MiB" in str(e.value)
    # the existing entry point computes it; the no-alloc one still works afterwards
    ref = _call(G, G.lib().kv_expectation, a, ws, a)
    amp = np.sum(a0.blocks[0][1].ravel() * a1.blocks[0][1].ravel())  # the state is one amplitude
    assert abs(ref - abs(amp) ** 2) < 1e-9 * abs(ref)


def test_noalloc_bond_dimension_128_fits(gpu):
    """The scratch is set by the largest site, not by the chain length: a
    15-site chain of the two-site benchmark's local structure (D = 128, MPO
    bond dimension 7, local dimension 16) fits the 64 MiB array."""
    G = gpu
    ch, D, _ = H.config_chain("holstein-2site-L32")
    ch = H.HolsteinChain(3, ch.omega, ch.g[:3], ch.cutoff, ch.J, ch.eps[:3])
    mps, mpo = H.random_mps(ch, D, seed=1234), H.hamiltonian_mpo(ch)
    a = [G.Tensor.from_host(t) for t in mps]
    w = [G.Tensor.from_host(t) for t in mpo]
    ref = _call(G, G.lib().kv_expectation, a, w, a)
    for _ in range(2):
        assert abs(_call(G, G.lib().kv_expectation_noalloc, a, w, a) - ref) <= 1e-12 * max(1.0, abs(ref))


def test_noalloc_task_lists_beyond_scratch_leave_no_pending_error(gpu):
    """A contraction whose output fits the scratch but whose GEMM task lists do
    not (800 000 one-element blocks): KV_ENOMEM, and the arena views are
    cleared on the way out, so no arena address reaches cudaFreeAsync and the
    next calls of both entry points succeed."""
    G = gpu
    L = G.lib()
    n = 800_000
    shapes = np.ones((n, 3), dtype=np.int32)
    qns = np.zeros((n, 3), dtype=np.int32)
    qns[:, 2] = np.arange(n, dtype=np.int32)
    data = np.zeros(2 * n)
    data[::2] = 1.0
    ip = ctypes.POINTER(ctypes.c_int)
    t = ctypes.c_void_p()
    G.check(L.kv_tensor_create(3, (ctypes.c_int * 3)(1, 1, -1), n, shapes.ctypes.data_as(ip),
                               qns.ctypes.data_as(ip), data.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                               ctypes.byref(t)))
    big = G.Tensor(t.value)
    w = G.Tensor.from_host(kvio.BlockTensor((1, 1, -1, -1), [((0, 0, 0, 0), np.ones((1, 1, 1, 1), complex))]))
    with pytest.raises(G.KvError) as e:
        _call(G, L.kv_expectation_noalloc, [big], [w], [big])
    assert e.value.code == -3 and "64 MiB" in str(e.value)
    g = os.path.join(U.GOLDEN, "tiny1")
    mps, mpo = kvio.read_mps(os.path.join(g, "in.mps")), kvio.read_mpo(os.path.join(g, "H.mpo"))
    a = [G.Tensor.from_host(x) for x in mps]
    ws = [G.Tensor.from_host(x) for x in mpo]
    ref = _call(G, L.kv_expectation, a, ws, a)
    assert abs(_call(G, L.kv_expectation_noalloc, a, ws, a) - ref) <= 1e-12 * max(1.0, abs(ref))
