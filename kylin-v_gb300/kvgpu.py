"""ctypes binding of libkvgpu.so (C ABI in include/kvgpu.h).

There is no CPU fallback: if the library is missing or no CUDA device is
present, :func:`lib` / :func:`init` raise.  Tensors are exchanged as
:class:`~kylin_v_gb300.kvio.BlockTensor` (complex128 blocks, reference order).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .kvio import BlockTensor

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libkvgpu.so")

KV_FP64 = 0
KV_MIXED_3M_DIGITS = 1  # 3M products of fixed-point FP16 digits on the tensor cores (include/kvgpu.h)
KV_MIXED_TF32 = KV_MIXED_3M_DIGITS  # other names of the same mode
KV_MIXED_3M_TF32 = KV_MIXED_3M_DIGITS
KV_MIXED_3M_BF16X3 = KV_MIXED_3M_DIGITS
KV_MIXED_GEMM = 2  # tensor-core contractions, FP64 SVD
KV_MIXED_SVD = 3   # FP64 contractions, mixed SVD
OP_N, OP_T, OP_C = 111, 112, 113
MODULES = ("Evl-0", "Evl-1", "Evl-2", "SVD", "Update", "Sweep")

EXPORTS = (
    "kv_init", "kv_shutdown", "kv_last_error", "kv_version", "kv_tensor_create", "kv_tensor_info",
    "kv_tensor_download", "kv_tensor_free", "kv_product", "kv_heff_apply", "kv_env_update", "kv_lanczos_expm",
    "kv_svd_truncate", "kv_tdvp_create", "kv_tdvp_sweep", "kv_tdvp_site", "kv_tdvp_stats", "kv_tdvp_free",
    "kv_expectation", "kv_profile", "kv_profile_read", "kv_counters", "kv_expectation_noalloc",
    "kv_tdvp_host_stats", "kv_canonicalize", "kv_sweep_batched", "kv_adjoint_heff", "kv_adjoint_env",
    "kv_debug_gemm_stall", "kv_debug_pool_usage", "kv_svd_stats", "kv_krylov_stats", "kv_tdvp_set_sa",
    "kv_tdvp_svs", "kv_profile_read_lanczos", "kv_profile_read_mix", "kv_tdvp_window", "kv_local_expectations",
)


class KvError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"kvgpu error {code}: {msg}")
        self.code = code


_lib = None


def lib():
    """Load libkvgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        L = ctypes.CDLL(LIB_PATH)
        vp = ctypes.c_void_p
        ip = ctypes.POINTER(ctypes.c_int)
        dp = ctypes.POINTER(ctypes.c_double)
        pvp = ctypes.POINTER(vp)
        L.kv_last_error.restype = ctypes.c_char_p
        L.kv_init.argtypes = [ctypes.c_int]
        L.kv_tensor_create.argtypes = [ctypes.c_int, ip, ctypes.c_int, ip, ip, dp, pvp]
        L.kv_tensor_info.argtypes = [vp, ip, ip, ctypes.POINTER(ctypes.c_longlong)]
        L.kv_tensor_download.argtypes = [vp, ip, ip, ip, dp]
        L.kv_tensor_free.argtypes = [vp]
        L.kv_product.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, pvp]
        L.kv_heff_apply.argtypes = [ctypes.c_int, vp, vp, vp, vp, vp, ctypes.c_double, ctypes.c_int, pvp]
        L.kv_env_update.argtypes = [ctypes.c_int, vp, vp, vp, ctypes.c_int, pvp]
        L.kv_lanczos_expm.argtypes = [ctypes.c_int, vp, vp, vp, vp, vp, ctypes.c_double, ctypes.c_int,
                                      ctypes.c_double, ctypes.c_int, ctypes.c_int, pvp, ip]
        L.kv_svd_truncate.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                      pvp, pvp, ip, ip]
        L.kv_tdvp_create.argtypes = [ctypes.c_int, pvp, pvp, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_double, ctypes.c_int, pvp]
        L.kv_tdvp_sweep.argtypes = [vp, ctypes.c_int]
        L.kv_tdvp_window.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        L.kv_tdvp_site.argtypes = [vp, ctypes.c_int, pvp]
        L.kv_tdvp_stats.argtypes = [vp, dp, dp, dp, dp]
        L.kv_tdvp_host_stats.argtypes = [vp, dp, dp, ctypes.POINTER(ctypes.c_longlong), dp]
        L.kv_profile.argtypes = [ctypes.c_int]
        L.kv_profile_read.argtypes = [dp, dp, ctypes.POINTER(ctypes.c_longlong)]
        L.kv_profile_read_lanczos.argtypes = [dp, dp, ctypes.POINTER(ctypes.c_longlong)]
        L.kv_profile_read_mix.argtypes = [dp, dp, ctypes.POINTER(ctypes.c_longlong)]
        L.kv_counters.argtypes = [ctypes.POINTER(ctypes.c_longlong)]
        L.kv_tdvp_free.argtypes = [vp]
        L.kv_expectation.argtypes = [ctypes.c_int, pvp, pvp, pvp, dp, dp]
        L.kv_canonicalize.argtypes = [ctypes.c_int, pvp, ctypes.c_double, ctypes.c_int, ctypes.c_int, pvp]
        L.kv_expectation_noalloc.argtypes = [ctypes.c_int, pvp, pvp, pvp, dp, dp]
        L.kv_local_expectations.argtypes = [ctypes.c_int, pvp, pvp, ctypes.c_int, ip, pvp, dp, dp]
        L.kv_sweep_batched.argtypes = [ctypes.c_int, pvp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
        L.kv_adjoint_heff.argtypes = [ctypes.c_int, vp, vp, vp, vp, vp, ctypes.c_double, vp, ctypes.c_int,
                                      pvp, pvp, pvp, pvp, pvp]
        L.kv_adjoint_env.argtypes = [ctypes.c_int, vp, vp, vp, vp, ctypes.c_int, pvp, pvp, pvp]
        L.kv_debug_gemm_stall.argtypes = [ctypes.c_int]
        ll = ctypes.POINTER(ctypes.c_longlong)
        L.kv_svd_stats.argtypes = [ctypes.c_int, ll, ll, ll, ll, ip]
        L.kv_krylov_stats.argtypes = [ctypes.c_int, ll, ll, ll]
        L.kv_tdvp_set_sa.argtypes = [vp, dp, ctypes.c_int, ctypes.c_ulonglong, ll]
        L.kv_tdvp_svs.argtypes = [vp, ip, ll, ip, dp]
        L.kv_debug_pool_usage.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_longlong),
                                          ctypes.POINTER(ctypes.c_longlong)]
        _lib = L
    return _lib


def check(rc: int):
    if rc != 0:
        raise KvError(rc, lib().kv_last_error().decode())


def init(device: int = 0):
    check(lib().kv_init(device))


class Tensor:
    """Owned device tensor handle."""

    def __init__(self, ptr: int):
        self.ptr = ptr

    @classmethod
    def from_host(cls, t: BlockTensor) -> "Tensor":
        L = lib()
        rank, nb = t.rank, len(t.blocks)
        dirs = (ctypes.c_int * rank)(*t.dirs)
        shapes = np.array([s for _, a in t.blocks for s in a.shape] or [0], dtype=np.int32)
        qns = np.array([q for qn, _ in t.blocks for q in qn] or [0], dtype=np.int32)
        data = np.ascontiguousarray(np.concatenate([a.ravel() for _, a in t.blocks]) if nb else np.zeros(1),
                                    dtype=np.complex128)
        out = ctypes.c_void_p()
        check(L.kv_tensor_create(rank, dirs, nb, shapes.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                 qns.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                 data.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(out)))
        return cls(out.value)

    @classmethod
    def from_pinned(cls, t: BlockTensor, data_ptr: int) -> "Tensor":
        """Like from_host, with the block data read from a caller-owned host
        buffer (e.g. pinned memory) at data_ptr (complex128, block order)."""
        L = lib()
        rank, nb = t.rank, len(t.blocks)
        dirs = (ctypes.c_int * rank)(*t.dirs)
        shapes = np.array([s for _, a in t.blocks for s in a.shape] or [0], dtype=np.int32)
        qns = np.array([q for qn, _ in t.blocks for q in qn] or [0], dtype=np.int32)
        out = ctypes.c_void_p()
        check(L.kv_tensor_create(rank, dirs, nb, shapes.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                 qns.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                 ctypes.cast(data_ptr, ctypes.POINTER(ctypes.c_double)), ctypes.byref(out)))
        return cls(out.value)

    def info(self):
        r, nb, ne = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
        check(lib().kv_tensor_info(self.ptr, ctypes.byref(r), ctypes.byref(nb), ctypes.byref(ne)))
        return r.value, nb.value, ne.value

    def to_host(self) -> BlockTensor:
        r, nb, ne = self.info()
        dirs = (ctypes.c_int * r)()
        shapes = np.zeros(max(1, nb * r), np.int32)
        qns = np.zeros(max(1, nb * r), np.int32)
        data = np.zeros(max(1, ne), np.complex128)
        check(lib().kv_tensor_download(self.ptr, dirs, shapes.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                       qns.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                       data.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        blocks, off = [], 0
        for b in range(nb):
            sh = tuple(int(x) for x in shapes[b * r:(b + 1) * r])
            sz = int(np.prod(sh))
            blocks.append((tuple(int(x) for x in qns[b * r:(b + 1) * r]), data[off:off + sz].reshape(sh).copy()))
            off += sz
        return BlockTensor(tuple(dirs), blocks)

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.kv_tensor_free(self.ptr)
            self.ptr = None


def _t(x):
    if x is None:
        return None
    return x if isinstance(x, Tensor) else Tensor.from_host(x)


def _p(x):
    return x.ptr if x is not None else None


def product(A, B, nc, opA=OP_N, opB=OP_N, precision=KV_FP64) -> Tensor:
    """product<N1,N2,nc> (holstein/product.h:61-201)."""
    A, B = _t(A), _t(B)
    out = ctypes.c_void_p()
    check(lib().kv_product(A.ptr, B.ptr, nc, opA, opB, precision, ctypes.byref(out)))
    return Tensor(out.value)


def heff_apply(nsite, L, psi, W1, W2, R, scale=1.0, precision=KV_FP64) -> Tensor:
    """apply_zero / apply_single / apply_double (holstein/product.h:478-553)."""
    hs = [_t(x) for x in (L, psi, W1, W2, R)]
    out = ctypes.c_void_p()
    check(lib().kv_heff_apply(nsite, *[_p(h) for h in hs], scale, precision, ctypes.byref(out)))
    return Tensor(out.value)


def env_sweep(env, A, W, left2right, precision=KV_FP64) -> Tensor:
    """env_sweep (holstein/product.h:488-503)."""
    env, A, W = _t(env), _t(A), _t(W)
    out = ctypes.c_void_p()
    check(lib().kv_env_update(int(left2right), env.ptr, A.ptr, W.ptr, precision, ctypes.byref(out)))
    return Tensor(out.value)


HEFF_GRADS = ("psi", "L", "W1", "W2", "R")


def adjoint_heff(nsite, L, psi, W1, W2, R, ybar, scale=1.0, precision=KV_FP64, want=HEFF_GRADS) -> dict:
    """Cotangents of heff_apply's operands for the output cotangent ybar
    (kv_adjoint_heff); `want` names the ones to compute."""
    hs = [_t(x) for x in (L, psi, W1, W2, R, ybar)]
    present = {"psi": True, "L": True, "W1": nsite >= 1, "W2": nsite == 2, "R": True}
    outs = {k: ctypes.c_void_p() for k in HEFF_GRADS if k in want and present[k]}
    refs = [ctypes.byref(outs[k]) if k in outs else None for k in HEFF_GRADS]
    check(lib().kv_adjoint_heff(nsite, *[_p(h) for h in hs[:5]], scale, hs[5].ptr, precision, *refs))
    return {k: Tensor(v.value) for k, v in outs.items()}


def adjoint_env(env, A, W, left2right, out_bar, precision=KV_FP64, want=("env", "A", "W")) -> dict:
    """Cotangents of env_sweep's operands for the output cotangent out_bar (kv_adjoint_env)."""
    env, A, W, ob = _t(env), _t(A), _t(W), _t(out_bar)
    outs = {k: ctypes.c_void_p() for k in ("env", "A", "W") if k in want}
    refs = [ctypes.byref(outs[k]) if k in outs else None for k in ("env", "A", "W")]
    check(lib().kv_adjoint_env(int(left2right), env.ptr, A.ptr, W.ptr, ob.ptr, precision, *refs))
    return {k: Tensor(v.value) for k, v in outs.items()}


def local_krylov(nsite, L, psi, W1, W2, R, dt, max_iter, tol, reverse=False, precision=KV_FP64):
    """local_krylov<Rank> (holstein/exponential.h:92-190); returns (tensor, Krylov dimension)."""
    hs = [_t(x) for x in (L, psi, W1, W2, R)]
    out = ctypes.c_void_p()
    it = ctypes.c_int()
    check(lib().kv_lanczos_expm(nsite, *[_p(h) for h in hs], dt, max_iter, tol, int(reverse), precision,
                                ctypes.byref(out), ctypes.byref(it)))
    return Tensor(out.value), it.value


def svd_impl(A, r1, left2right, tol, max_dim, precision=KV_FP64):
    """svd_impl<R1,R2> (holstein/svd.h:296-440); returns (U, V, n_kept, n_total)."""
    A = _t(A)
    U, V = ctypes.c_void_p(), ctypes.c_void_p()
    nk, nt = ctypes.c_int(), ctypes.c_int()
    check(lib().kv_svd_truncate(A.ptr, r1, int(left2right), tol, max_dim, precision, ctypes.byref(U),
                                ctypes.byref(V), ctypes.byref(nk), ctypes.byref(nt)))
    return Tensor(U.value), Tensor(V.value), nk.value, nt.value


def expectation(bra, mpo, ket) -> complex:
    """<bra|W|ket> (Operator::join, holstein/operator.h:178-198)."""
    ns = len(bra)
    hb, hw, hk = [_t(x) for x in bra], [_t(x) for x in mpo], [_t(x) for x in ket]
    arr = lambda hs: (ctypes.c_void_p * ns)(*[h.ptr for h in hs])  # noqa: E731
    re, im = ctypes.c_double(), ctypes.c_double()
    check(lib().kv_expectation(ns, arr(hb), arr(hw), arr(hk), ctypes.byref(re), ctypes.byref(im)))
    return complex(re.value, im.value)


def canonicalize(mps, tol_svd=0.0, max_dim=1000, precision=KV_FP64) -> list:
    """State::canonicalize (holstein/state.h:166-185): L->R then R->L SVD
    sweeps; returns new site tensors with the orthogonality centre on site 0."""
    ns = len(mps)
    hs = [_t(x) for x in mps]
    outs = (ctypes.c_void_p * ns)()
    check(lib().kv_canonicalize(ns, (ctypes.c_void_p * ns)(*[h.ptr for h in hs]), tol_svd, max_dim, precision, outs))
    return [Tensor(outs[i]) for i in range(ns)]


def profile(enable: bool):
    """Bracket every grouped-GEMM launch with CUDA events (instrumentation)."""
    check(lib().kv_profile(int(enable)))


def _profile_read_bytes(fn) -> dict:
    ms, b, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
    check(fn(ctypes.byref(ms), ctypes.byref(b), ctypes.byref(n)))
    return {"ms": ms.value, "bytes": b.value, "launches": n.value}


def profile_read_lanczos() -> dict:
    """Profiled Lanczos steps since the last read: device ms, algorithmic bytes, launches."""
    return _profile_read_bytes(lib().kv_profile_read_lanczos)


def profile_read_mix() -> dict:
    """Profiled MPO mixings of the sweep since the last read: device ms, algorithmic bytes, launches."""
    return _profile_read_bytes(lib().kv_profile_read_mix)


def profile_read() -> dict:
    ms, fl, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
    check(lib().kv_profile_read(ctypes.byref(ms), ctypes.byref(fl), ctypes.byref(n)))
    return {"gemm_ms": ms.value, "gemm_ref_flops": fl.value, "gemm_launches": n.value}


def svd_stats(reset: bool = True) -> dict:
    """Charge sectors through the block SVD since the last reset: count,
    columns, ranks kept by the mixed path's QR reduction, Jacobi sweeps."""
    v = [ctypes.c_longlong() for _ in range(4)]
    mx = ctypes.c_int()
    check(lib().kv_svd_stats(int(reset), *[ctypes.byref(x) for x in v], ctypes.byref(mx)))
    n = max(1, v[0].value)
    return {"sectors": v[0].value, "mean_columns": v[1].value / n, "mean_rank": v[2].value / n,
            "mean_sweeps": v[3].value / n, "max_sweeps": mx.value}


def krylov_stats(reset: bool = True) -> dict:
    """local_krylov calls since the last reset, Lanczos iterations issued per
    call and the mean Krylov dimension reached."""
    v = [ctypes.c_longlong() for _ in range(3)]
    check(lib().kv_krylov_stats(int(reset), *[ctypes.byref(x) for x in v]))
    n = max(1, v[0].value)
    return {"calls": v[0].value, "issued_per_call": v[1].value / n, "mean_dimension": v[2].value / n}


def launches() -> int:
    n = ctypes.c_longlong()
    check(lib().kv_counters(ctypes.byref(n)))
    return n.value


def local_expectations(mps, ident_mpo, ops) -> list:
    """<psi|O|psi> for each (site, MPO tensor) in ops, O the identity elsewhere
    (kv_local_expectations): all from one left and one right pass."""
    ms = [_t(x) for x in mps]
    ws = [_t(x) for x in ident_mpo]
    os_ = [_t(t) for _, t in ops]
    ns, no = len(ms), len(ops)
    arr = lambda hs: (ctypes.c_void_p * max(1, len(hs)))(*[h.ptr for h in hs])  # noqa: E731
    sites = (ctypes.c_int * max(1, no))(*[s for s, _ in ops])
    re, im = (ctypes.c_double * max(1, no))(), (ctypes.c_double * max(1, no))()
    check(lib().kv_local_expectations(ns, arr(ms), arr(ws), no, sites, arr(os_), re, im))
    return [complex(re[k], im[k]) for k in range(no)]


def expectation_noalloc(bra, mpo, ket) -> complex:
    """<bra|W|ket> like :func:`expectation`, with every intermediate in the
    library's fixed 64 MiB device scratch array (no GPU allocation)."""
    ns = len(bra)
    hb, hw, hk = [_t(x) for x in bra], [_t(x) for x in mpo], [_t(x) for x in ket]
    arr = lambda hs: (ctypes.c_void_p * ns)(*[h.ptr for h in hs])  # noqa: E731
    re, im = ctypes.c_double(), ctypes.c_double()
    check(lib().kv_expectation_noalloc(ns, arr(hb), arr(hw), arr(hk), ctypes.byref(re), ctypes.byref(im)))
    return complex(re.value, im.value)


class TDVP:
    """TDVP sweep driver (holstein/tdvp.h:34-385) on the device."""

    def __init__(self, mps, mpo, tol_svd, tol_exp, max_dim, max_iter, dt, precision=KV_FP64):
        ns = len(mps)
        self._m = [_t(x) for x in mps]
        self._o = [_t(x) for x in mpo]
        self.mpo = self._o
        arr = lambda hs: (ctypes.c_void_p * ns)(*[h.ptr for h in hs])  # noqa: E731
        out = ctypes.c_void_p()
        check(lib().kv_tdvp_create(ns, arr(self._m), arr(self._o), tol_svd, tol_exp, max_dim, max_iter, dt,
                                   precision, ctypes.byref(out)))
        self.ptr = out.value
        self.ns = ns
        self._m = None  # the driver holds its own copies

    def global_krylov(self):
        """One step of total_start's global-Krylov stage (holstein/krylov.h:199-283)."""
        check(lib().kv_tdvp_sweep(self.ptr, 0))

    def sweep(self, mode: int):
        """mode 0: global_krylov, 1: one_site, 2: two_site, 3: sa_site (set_sa first)."""
        check(lib().kv_tdvp_sweep(self.ptr, mode))

    def set_sa(self, betas, seed: int):
        """SA-1TDVP widths per bond (betaSet, holstein/tdvp.h:343-358) and the
        seed of the stream every SA draw's generator is seeded from."""
        b = (ctypes.c_double * max(1, len(betas)))(*[float(x) for x in betas])
        check(lib().kv_tdvp_set_sa(self.ptr, b, len(betas), int(seed), None))

    def svs(self) -> list:
        """Kept singular values (descending) of every two-site split since the
        last call (the SVS record of holstein/svd.h:390-402), then cleared."""
        nr, nv = ctypes.c_int(), ctypes.c_longlong()
        check(lib().kv_tdvp_svs(self.ptr, ctypes.byref(nr), ctypes.byref(nv), None, None))
        counts = (ctypes.c_int * max(1, nr.value))()
        vals = (ctypes.c_double * max(1, nv.value))()
        check(lib().kv_tdvp_svs(self.ptr, None, None, counts, vals))
        out, k = [], 0
        for i in range(nr.value):
            out.append([vals[k + j] for j in range(counts[i])])
            k += counts[i]
        return out

    def sa_added(self) -> int:
        """States the SA splits of the last SA sweep added."""
        n = ctypes.c_longlong()
        check(lib().kv_tdvp_set_sa(self.ptr, None, 0, 0, ctypes.byref(n)))
        return n.value

    def window(self, i0: int, n: int):
        """n timed two-site local updates of the left-to-right pass from site
        i0 (the pass is advanced there first, untimed)."""
        check(lib().kv_tdvp_window(self.ptr, i0, n))

    def one_site(self):
        check(lib().kv_tdvp_sweep(self.ptr, 1))

    def two_site(self):
        check(lib().kv_tdvp_sweep(self.ptr, 2))

    def site(self, i) -> Tensor:
        out = ctypes.c_void_p()
        check(lib().kv_tdvp_site(self.ptr, i, ctypes.byref(out)))
        return Tensor(out.value)

    def sites(self) -> list:
        return [self.site(i) for i in range(self.ns)]

    def stats(self) -> dict:
        """Last sweep: per-module device ms, sweep device ms, reference flops
        (all zgemms) and the product<> part run by the grouped GEMM."""
        ms = (ctypes.c_double * len(MODULES))()
        sw, fl, fg = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(lib().kv_tdvp_stats(self.ptr, ms, ctypes.byref(sw), ctypes.byref(fl), ctypes.byref(fg)))
        return {"modules_ms": dict(zip(MODULES, list(ms))), "sweep_ms": sw.value, "ref_flops": fl.value,
                "gemm_ref_flops": fg.value}

    def host_stats(self) -> dict:
        """Last sweep, host side: per-module and sweep wall-clock ms, H_eff
        plans built (plan-cache misses) and the host ms spent building them."""
        ms = (ctypes.c_double * len(MODULES))()
        sw, pm = ctypes.c_double(), ctypes.c_double()
        nb = ctypes.c_longlong()
        check(lib().kv_tdvp_host_stats(self.ptr, ms, ctypes.byref(sw), ctypes.byref(nb), ctypes.byref(pm)))
        return {"modules_ms": dict(zip(MODULES, list(ms))), "sweep_ms": sw.value, "plans_built": nb.value,
                "plan_ms": pm.value}

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.kv_tdvp_free(self.ptr)
            self.ptr = None


def sweep_batched(chains, mode: int, steps: int = 1, max_streams: int = 0) -> float:
    """Advance independent chains (TDVP objects) by `steps` time steps of
    `mode` concurrently (kv_sweep_batched); returns the device ms."""
    n = len(chains)
    arr = (ctypes.c_void_p * max(1, n))(*[c.ptr for c in chains])
    ms = ctypes.c_double()
    check(lib().kv_sweep_batched(n, arr, mode, steps, max_streams, ctypes.byref(ms)))
    return ms.value
