"""ctypes wrapper of the CPU restatement oracle (oracle/kv_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline leg as the checker.  Tensors cross the boundary as
``BlockTensor`` objects (kylin_v_gb300.kvio) and are copied into oracle handles.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libkvoracle.so")
OP_N, OP_T, OP_C = 111, 112, 113

_lib = None


def build(force: bool = False) -> str:
    """Compile the restatement with the committed Makefile (g++, scipy's OpenBLAS)."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
            os.path.join(HERE, "kv_oracle.cpp")):
        subprocess.run(["make", "-C", HERE, "port"], check=True, stdout=subprocess.DEVNULL)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp, ip, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
        L.kvo_last_error.restype = ctypes.c_char_p
        L.kvo_tensor_new.argtypes = [ctypes.c_int, ip, ctypes.c_int, ip, ip, dp, ctypes.POINTER(vp)]
        L.kvo_tensor_info.argtypes = [vp, ip, ip, ctypes.POINTER(ctypes.c_longlong)]
        L.kvo_tensor_get.argtypes = [vp, ip, ip, ip, dp]
        L.kvo_tensor_free.argtypes = [vp]
        L.kvo_tensor_free.restype = None
        L.kvo_product.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]
        L.kvo_apply.argtypes = [ctypes.c_int, vp, vp, vp, vp, vp, ctypes.POINTER(vp)]
        L.kvo_env_sweep.argtypes = [vp, vp, vp, ctypes.c_int, ctypes.POINTER(vp)]
        L.kvo_local_krylov.argtypes = [ctypes.c_int, vp, vp, vp, vp, vp, ctypes.c_double, ctypes.c_int,
                                       ctypes.c_double, ctypes.c_int, ip, ctypes.POINTER(vp)]
        L.kvo_svd.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                              ctypes.POINTER(vp), ctypes.POINTER(vp), dp, ip, ip]
        L.kvo_tdvp_new.argtypes = [ctypes.c_int, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.c_double,
                                   ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                   ctypes.POINTER(vp)]
        L.kvo_tdvp_sweep.argtypes = [vp, ctypes.c_int]
        L.kvo_tdvp_set_sa.argtypes = [vp, dp, ctypes.c_int, ctypes.c_ulonglong]
        L.kvo_tdvp_window.argtypes = [vp, ctypes.c_int, ctypes.c_int, dp]
        L.kvo_tdvp_site.argtypes = [vp, ctypes.c_int, ctypes.POINTER(vp)]
        L.kvo_tdvp_free.argtypes = [vp]
        L.kvo_tdvp_free.restype = None
        L.kvo_flops.argtypes = [ctypes.c_int]
        L.kvo_flops.restype = ctypes.c_double
        L.kvo_join.argtypes = [ctypes.c_int, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp), dp, dp]
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise RuntimeError("oracle: " + lib().kvo_last_error().decode())


class _H:
    """Owned oracle tensor handle."""

    def __init__(self, ptr):
        self.ptr = ptr

    def __del__(self):
        if self.ptr and _lib is not None:
            _lib.kvo_tensor_free(self.ptr)
            self.ptr = None


def to_handle(t) -> _H:
    L = lib()
    rank = t.rank
    nb = len(t.blocks)
    dirs = (ctypes.c_int * rank)(*t.dirs)
    shapes = np.array([s for _, a in t.blocks for s in a.shape], dtype=np.int32)
    qns = np.array([q for qn, _ in t.blocks for q in qn], dtype=np.int32)
    data = np.concatenate([a.ravel() for _, a in t.blocks]) if nb else np.zeros(1, complex)
    data = np.ascontiguousarray(data, dtype=np.complex128)
    out = ctypes.c_void_p()
    _check(L.kvo_tensor_new(rank, dirs, nb, shapes.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                            qns.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                            data.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(out)))
    return _H(out.value)


def from_handle(h):
    from kylin_v_gb300.kvio import BlockTensor  # the package is registered by the caller

    L = lib()
    ptr = h.ptr if isinstance(h, _H) else h
    rank, nb, ne = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
    L.kvo_tensor_info(ptr, ctypes.byref(rank), ctypes.byref(nb), ctypes.byref(ne))
    r, n = rank.value, nb.value
    dirs = (ctypes.c_int * r)()
    shapes = np.zeros(max(1, n * r), np.int32)
    qns = np.zeros(max(1, n * r), np.int32)
    data = np.zeros(max(1, ne.value), np.complex128)
    L.kvo_tensor_get(ptr, dirs, shapes.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                     qns.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                     data.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    blocks = []
    off = 0
    for b in range(n):
        sh = tuple(int(x) for x in shapes[b * r:(b + 1) * r])
        sz = int(np.prod(sh))
        blocks.append((tuple(int(x) for x in qns[b * r:(b + 1) * r]), data[off:off + sz].reshape(sh).copy()))
        off += sz
    return BlockTensor(tuple(dirs), blocks)


def _owned(ptr_holder) -> _H:
    return _H(ptr_holder.value)


def product(a, b, nc, ta=OP_N, tb=OP_N):
    out = ctypes.c_void_p()
    ha, hb = to_handle(a), to_handle(b)
    _check(lib().kvo_product(ha.ptr, hb.ptr, nc, ta, tb, ctypes.byref(out)))
    return from_handle(_owned(out))


def apply(nsite, L, psi, W1, W2, R):
    hs = [to_handle(x) if x is not None else None for x in (L, psi, W1, W2, R)]
    out = ctypes.c_void_p()
    _check(lib().kvo_apply(nsite, *[h.ptr if h else None for h in hs], ctypes.byref(out)))
    return from_handle(_owned(out))


def env_sweep(env, A, W, l2r):
    he, ha, hw = to_handle(env), to_handle(A), to_handle(W)
    out = ctypes.c_void_p()
    _check(lib().kvo_env_sweep(he.ptr, ha.ptr, hw.ptr, int(l2r), ctypes.byref(out)))
    return from_handle(_owned(out))


def local_krylov(nsite, L, psi, W1, W2, R, dt, max_iter, tol, reverse=False):
    hs = [to_handle(x) if x is not None else None for x in (L, psi, W1, W2, R)]
    out = ctypes.c_void_p()
    it = ctypes.c_int()
    _check(lib().kvo_local_krylov(nsite, *[h.ptr if h else None for h in hs], dt, max_iter, tol,
                                  int(reverse), ctypes.byref(it), ctypes.byref(out)))
    return from_handle(_owned(out)), it.value


def svd(A, r1, l2r, tol, max_dim):
    ha = to_handle(A)
    U, V = ctypes.c_void_p(), ctypes.c_void_p()
    nk, nt = ctypes.c_int(), ctypes.c_int()
    sv = np.zeros(sum(a.size for _, a in A.blocks) + 1)
    _check(lib().kvo_svd(ha.ptr, r1, int(l2r), tol, max_dim, ctypes.byref(U), ctypes.byref(V),
                         sv.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(nk), ctypes.byref(nt)))
    return from_handle(_owned(U)), from_handle(_owned(V)), sv[:nk.value].copy(), nt.value


class Tdvp:
    """The reference TDVP sweep driver (holstein/tdvp.h) on the CPU restatement."""

    def __init__(self, mps, mpo, tol_svd, tol_exp, max_dim, max_iter, dt):
        ns = len(mps)
        self._hm = [to_handle(t) for t in mps]
        self._ho = [to_handle(t) for t in mpo]
        arr_m = (ctypes.c_void_p * ns)(*[h.ptr for h in self._hm])
        arr_o = (ctypes.c_void_p * ns)(*[h.ptr for h in self._ho])
        out = ctypes.c_void_p()
        _check(lib().kvo_tdvp_new(ns, arr_m, arr_o, tol_svd, tol_exp, max_dim, max_iter, dt, ctypes.byref(out)))
        self.ptr = out.value
        self.ns = ns

    def window(self, i0, n) -> float:
        """Seconds for n two-site local updates of the left-to-right pass from
        site i0, on a copy of the state advanced (once) to i0."""
        sec = ctypes.c_double()
        _check(lib().kvo_tdvp_window(self.ptr, i0, n, ctypes.byref(sec)))
        return sec.value

    def sweep(self, mode):
        """mode 0: one global-Krylov step, 1: one_site, 2: two_site, 3: sa_site
        (widths and seed from set_sa)."""
        _check(lib().kvo_tdvp_sweep(self.ptr, mode))

    def set_sa(self, betas, seed):
        """SA-1TDVP widths per bond (betaSet of holstein/tdvp.h:343-358) and
        the seed of the generator every SA draw comes from."""
        b = (ctypes.c_double * len(betas))(*[float(x) for x in betas])
        _check(lib().kvo_tdvp_set_sa(self.ptr, b, len(betas), int(seed)))

    def mps(self):
        out = []
        for i in range(self.ns):
            h = ctypes.c_void_p()
            _check(lib().kvo_tdvp_site(self.ptr, i, ctypes.byref(h)))
            out.append(from_handle(_owned(h)))
        return out

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.kvo_tdvp_free(self.ptr)
            self.ptr = None


def flops(reset=True) -> float:
    """Complex-GEMM flops (8*M*N*K, the reference's zgemm calls) since the last reset."""
    return lib().kvo_flops(int(reset))


def join(a, w, b) -> complex:
    """<a|W|b> (Operator::join, holstein/operator.h:178-198)."""
    ns = len(a)
    ha, hw, hb = [to_handle(t) for t in a], [to_handle(t) for t in w], [to_handle(t) for t in b]
    mk = lambda hs: (ctypes.c_void_p * ns)(*[h.ptr for h in hs])
    re, im = ctypes.c_double(), ctypes.c_double()
    _check(lib().kvo_join(ns, mk(ha), mk(hw), mk(hb), ctypes.byref(re), ctypes.byref(im)))
    return complex(re.value, im.value)
