// FP64 Lanczos kernels for local_krylov (holstein/exponential.h:92-190).
//
// All Krylov vectors share one block layout, so overlaps and updates are flat
// vector operations.  Reductions are two-level and deterministic: each kernel
// writes one partial per CTA (fixed grid, fixed order) and the next kernel
// reduces those partials in a fixed order before using the value, fused with
// the update that needs it (classical Gram-Schmidt in the reference's order:
// beta against v_{k-1} first, then alpha against v_k, then the norm).
#include <cooperative_groups.h>
#include <mutex>
#include "kv_internal.h"
#include "kv_jacobi.cuh"

namespace kv {

namespace {

constexpr int KT = 256;
constexpr double kMaxTridiagNorm = 1e5;  // largest ||T||_1 the Taylor sub-stepping accepts

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

// GB300's FP64 unit issues two thread-operations per clock per SM, so the
// vector kernels below are bound by their FP64 operation count and latency:
// products are accumulated with fused multiply-adds (two a component), and a
// block's warp sums are combined by a shuffle tree instead of one thread.

// s + conj(x) y, two fused multiply-adds a component
__device__ __forceinline__ double2 cdotc_acc(double2 s, double2 x, double2 y) {
    s.x = fma(x.x, y.x, fma(x.y, y.y, s.x));
    s.y = fma(x.x, y.y, fma(-x.y, y.x, s.y));
    return s;
}

// h - c x
__device__ __forceinline__ double2 csub_mul(double2 h, double2 c, double2 x) {
    h.x = fma(-c.x, x.x, fma(c.y, x.y, h.x));
    h.y = fma(-c.x, x.y, fma(-c.y, x.x, h.y));
    return h;
}

// s + c x
__device__ __forceinline__ double2 cmul_acc(double2 s, double2 c, double2 x) {
    s.x = fma(c.x, x.x, fma(-c.y, x.y, s.x));
    s.y = fma(c.x, x.y, fma(c.y, x.x, s.y));
    return s;
}

// s + |h|^2
__device__ __forceinline__ double norm2_acc(double s, double2 h) { return fma(h.x, h.x, fma(h.y, h.y, s)); }

// lane 0 receives the sum of the warp's first W values (a shuffle tree)
template <int W = 32>
__device__ __forceinline__ double2 warp_sum0(double2 v) {
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) {
        v.x += __shfl_down_sync(0xffffffffu, v.x, o);
        v.y += __shfl_down_sync(0xffffffffu, v.y, o);
    }
    return v;
}

// the block's sum, returned to every thread; a fixed order of adds
__device__ double2 block_sum(double2 v) {
    constexpr int NW = KT / 32;
    static_assert(NW <= 32 && (NW & (NW - 1)) == 0, "warp count a power of two");
    __shared__ double2 red[NW];
    __shared__ double2 out;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    v = warp_sum0(v);
    __syncthreads();  // a previous call's readers of red are done
    if (lane == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        double2 s = lane < NW ? red[lane] : make_double2(0.0, 0.0);
        s = warp_sum0<NW>(s);
        if (lane == 0) out = s;
    }
    __syncthreads();
    return out;
}

// every CTA reduces the same partial array in the same order
__device__ double2 reduce_partials(const double2 *parts, int nparts) {
    int i = threadIdx.x;
    double2 v = i < nparts ? parts[i] : make_double2(0.0, 0.0);
    for (i += KT; i < nparts; i += KT) v = cadd(v, parts[i]);
    return block_sum(v);
}

__global__ void __launch_bounds__(KT) k_norm_part(const double2 *x, int64_t n, double2 *parts) {
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)KT + threadIdx.x; i < n; i += (int64_t)gridDim.x * KT)
        s = norm2_acc(s, x[i]);
    double2 r = block_sum(make_double2(s, 0.0));
    if (threadIdx.x == 0) parts[blockIdx.x] = r;
}

// the host-mapped stop flag: visible to the host once the kernel has finished
__device__ __forceinline__ void raise_stop(int *stop) {
    if (stop) {
        *reinterpret_cast<volatile int *>(stop) = 1;
        __threadfence_system();
    }
}

__global__ void __launch_bounds__(KT) k_start(KrylovState *st, const double2 *psi, double2 *v0, int64_t n,
                                              const double2 *parts, int nparts, int *stop) {
    const double nrm = sqrt(reduce_partials(parts, nparts).x);
    const bool bad = !isfinite(nrm) || nrm == 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->psi_norm = nrm;
        st->err[0] = 1.0;
        st->done = bad ? 1 : 0;
        st->iters = 0;
        st->status = bad ? KV_ENONFINITE : KV_OK;
        if (bad) raise_stop(stop);
    }
    const double inv = bad ? 0.0 : 1.0 / nrm;
    for (int64_t i = blockIdx.x * (int64_t)KT + threadIdx.x; i < n; i += (int64_t)gridDim.x * KT)
        v0[i] = make_double2(psi[i].x * inv, psi[i].y * inv);
}

// parts[b] = sum conj(x) y
__global__ void __launch_bounds__(KT) k_dot_part(const KrylovState *st, const double2 *x, const double2 *y,
                                                 int64_t n, double2 *parts) {
    if (st->done) return;
    double2 s = make_double2(0.0, 0.0);
    for (int64_t i = blockIdx.x * (int64_t)KT + threadIdx.x; i < n; i += (int64_t)gridDim.x * KT)
        s = cdotc_acc(s, x[i], y[i]);
    double2 r = block_sum(s);
    if (threadIdx.x == 0) parts[blockIdx.x] = r;
}

// c = reduce(pin) (= overlap(v, hv) = <hv|v>);  hv -= c v on [0, n_sub) (v is
// zero beyond);  pout[b] = sum_{i < n_dot} conj(hv) w  (w == nullptr: sum |hv|^2).
// slot receives c.
__global__ void __launch_bounds__(KT) k_sub(KrylovState *st, double2 *hv, const double2 *v, const double2 *w,
                                            int64_t n_sub, int64_t n_dot, const double2 *pin, double2 *pout,
                                            int nparts, double2 *slot) {
    if (st->done) return;
    const double2 c = reduce_partials(pin, nparts);
    if (blockIdx.x == 0 && threadIdx.x == 0) *slot = c;
    double2 s = make_double2(0.0, 0.0);
    for (int64_t i = blockIdx.x * (int64_t)KT + threadIdx.x; i < n_dot; i += (int64_t)gridDim.x * KT) {
        double2 h = hv[i];
        if (i < n_sub) {
            h = csub_mul(h, c, v[i]);
            hv[i] = h;
        }
        if (w) s = cdotc_acc(s, h, w[i]);
        else s.x = norm2_acc(s.x, h);
    }
    double2 r = block_sum(s);
    if (threadIdx.x == 0) pout[blockIdx.x] = r;
}

// nrm = sqrt(reduce(pin)); err[k+1] = err[k] nrm; stop test; vnext = hv / nrm
__device__ __forceinline__ void normalize_body(KrylovState *st, const double2 *hv, double2 *vnext, int64_t n,
                                               const double2 *pin, int nparts, int k, double tol, int max_iter,
                                               int *stop) {
    const double nrm = sqrt(reduce_partials(pin, nparts).x);
    const double e = st->err[k] * nrm;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->err[k + 1] = e;
        if (!isfinite(nrm)) {
            st->status = KV_ENONFINITE;
            st->done = 1;
            st->iters = k + 1;
            raise_stop(stop);
        } else if (e <= tol || k + 1 >= max_iter - 1) {
            st->done = 1;
            st->iters = k + 1;
            raise_stop(stop);
        }
    }
    if (!(nrm > 0.0) || !isfinite(nrm)) return;
    const double inv = 1.0 / nrm;
    for (int64_t i = blockIdx.x * (int64_t)KT + threadIdx.x; i < n; i += (int64_t)gridDim.x * KT)
        vnext[i] = make_double2(hv[i].x * inv, hv[i].y * inv);
}

__global__ void __launch_bounds__(KT) k_normalize(KrylovState *st, const double2 *hv, double2 *vnext, int64_t n,
                                                  const double2 *pin, int nparts, int k, double tol, int max_iter,
                                                  int *stop) {
    if (st->done) return;
    normalize_body(st, hv, vnext, n, pin, nparts, k, tol, max_iter, stop);
}

// One Lanczos iteration after hv = (dt/2) H v_k, as one cooperative launch of
// the same grid the separate kernels use (k_dot_part, k_sub, k_sub,
// k_normalize), with a grid barrier where they end: the partial sums, their
// fixed-order reductions and so every result are the same bits.
__global__ void __launch_bounds__(KT) k_lanczos_step(KrylovState *st, int k, double2 *hv, const double2 *vprev,
                                                     const double2 *vk, double2 *vnext, int64_t n_prev, int64_t n_k,
                                                     int64_t n_next, double2 *P0, double2 *P1, int nparts, double tol,
                                                     int max_iter, int *stop) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    // read once, before the first barrier: this launch sets it only after the last one
    if (*reinterpret_cast<volatile int *>(&st->done)) return;  // uniform over the grid
    const int64_t i0 = blockIdx.x * (int64_t)KT + threadIdx.x, di = (int64_t)gridDim.x * KT;
    if (k > 0) {
        double2 s = make_double2(0.0, 0.0);
        for (int64_t i = i0; i < n_prev; i += di) s = cdotc_acc(s, hv[i], vprev[i]);
        double2 r = block_sum(s);
        if (threadIdx.x == 0) P0[blockIdx.x] = r;
        grid.sync();
        const double2 c = reduce_partials(P0, nparts);
        if (blockIdx.x == 0 && threadIdx.x == 0) st->beta[k - 1] = c;
        s = make_double2(0.0, 0.0);
        for (int64_t i = i0; i < n_k; i += di) {
            double2 h = hv[i];
            if (i < n_prev) {
                h = csub_mul(h, c, vprev[i]);
                hv[i] = h;
            }
            s = cdotc_acc(s, h, vk[i]);
        }
        r = block_sum(s);
        if (threadIdx.x == 0) P1[blockIdx.x] = r;
    } else {
        double2 s = make_double2(0.0, 0.0);
        for (int64_t i = i0; i < n_k; i += di) s = cdotc_acc(s, hv[i], vk[i]);
        const double2 r = block_sum(s);
        if (threadIdx.x == 0) P1[blockIdx.x] = r;
    }
    grid.sync();
    {
        const double2 c = reduce_partials(P1, nparts);
        if (blockIdx.x == 0 && threadIdx.x == 0) st->alpha[k] = c;
        double2 s = make_double2(0.0, 0.0);
        for (int64_t i = i0; i < n_next; i += di) {
            double2 h = hv[i];
            if (i < n_k) {
                h = csub_mul(h, c, vk[i]);
                hv[i] = h;
            }
            s.x = norm2_acc(s.x, h);
        }
        const double2 r = block_sum(s);
        if (threadIdx.x == 0) P0[blockIdx.x] = r;
    }
    grid.sync();
    normalize_body(st, hv, vnext, n_next, P0, nparts, k, tol, max_iter, stop);
}

// T = tridiag(Re alpha, beta upper); c = exp(img T) e0 with img = -i (forward)
// or +i (reverse).  The reference forms the same vector as
// Z exp(img Lambda) Z^H e0 from a dense eigendecomposition
// (holstein/exponential.h:163-183).  Here it is summed directly: m sub-steps
// with ||T/m||_1 <= 1, each a Taylor series of exp(img T/m) applied to the
// vector (terms t_k = img T t_{k-1} / (m k), stopping once a term falls below
// 1e-18 of the sum), so no term is larger than the vector it is added to.
// One warp; lane i holds component i and takes its neighbours' components
// by shuffles, so a term costs a few FP64 instructions per lane.  FP64.
__device__ __forceinline__ double2 shfl_down2(double2 v) {
    return make_double2(__shfl_down_sync(0xFFFFFFFFu, v.x, 1), __shfl_down_sync(0xFFFFFFFFu, v.y, 1));
}

__device__ __forceinline__ double2 shfl_up2(double2 v) {
    return make_double2(__shfl_up_sync(0xFFFFFFFFu, v.x, 1), __shfl_up_sync(0xFFFFFFFFu, v.y, 1));
}

__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}

__global__ void __launch_bounds__(32) k_tridiag_exp(KrylovState *st, int reverse) {
    static_assert(kMaxKrylov <= 32, "one lane per Krylov vector");
    const int lane = threadIdx.x;
    const int n = st->iters;
    if (n <= 0) return;
    if (st->status != KV_OK) {  // a non-finite Lanczos norm: no coefficients
        if (lane < n) st->coef[lane] = make_double2(nan(""), 0.0);
        return;
    }
    const bool on = lane < n;
    const double a = on ? st->alpha[lane].x : 0.0;
    const double2 zero = make_double2(0.0, 0.0);
    const double2 bu = (lane + 1 < n) ? st->beta[lane] : zero;  // T[lane][lane + 1]
    double2 bl = (on && lane >= 1) ? st->beta[lane - 1] : zero;  // T[lane][lane - 1] = conj(beta)
    bl.y = -bl.y;
    const double rs = warp_max(fabs(a) + sqrt(bu.x * bu.x + bu.y * bu.y) + sqrt(bl.x * bl.x + bl.y * bl.y));
    // the sub-step count is ceil(||T||_1): a norm beyond kMaxTridiagNorm (far
    // above any dt * H_eff of a physical chain) is reported as non-finite
    // instead of looping over that many steps
    if (!(rs <= kMaxTridiagNorm)) {
        if (on) st->coef[lane] = make_double2(nan(""), 0.0);
        if (lane == 0) st->status = KV_ENONFINITE;
        return;
    }
    const int m = max(1, (int)ceil(rs));
    const double sg = reverse ? 1.0 : -1.0;
    double2 y = make_double2(lane == 0 ? 1.0 : 0.0, 0.0);
    for (int step = 0; step < m; ++step) {
        double2 term = y, acc = y;
        for (int k = 1; k < 64; ++k) {
            const double2 up = shfl_down2(term);  // component lane + 1 (bu = 0 past the end)
            const double2 dn = shfl_up2(term);    // component lane - 1 (bl = 0 on lane 0)
            const double tr = a * term.x + (bu.x * up.x - bu.y * up.y) + (bl.x * dn.x - bl.y * dn.y);
            const double ti = a * term.y + (bu.x * up.y + bu.y * up.x) + (bl.x * dn.y + bl.y * dn.x);
            const double f = sg / ((double)m * k);  // term <- i f T term
            term = make_double2(-f * ti, f * tr);
            acc.x += term.x;
            acc.y += term.y;
            const double tm = warp_max(fabs(term.x) + fabs(term.y));
            const double am = warp_max(fabs(acc.x) + fabs(acc.y));
            if (tm <= 1e-18 * am) break;
        }
        y = acc;
    }
    if (on) st->coef[lane] = y;
}

__global__ void __launch_bounds__(KT) k_combine(const KrylovState *st, double2 *const *V, double2 *out,
                                                KrylovLens nl) {
    const int m = st->iters;
    if (m <= 0) return;
    const int64_t n = nl.n[m - 1];
    for (int64_t i = blockIdx.x * (int64_t)KT + threadIdx.x; i < n; i += (int64_t)gridDim.x * KT) {
        double2 acc = make_double2(0.0, 0.0);
        for (int j = 0; j < m; ++j) {
            if (i >= nl.n[j]) continue;
            acc = cmul_acc(acc, st->coef[j], V[j][i]);
        }
        out[i] = acc;
    }
}

__global__ void k_store_norm2(const double2 *parts, int nparts, double *result) {
    double2 s = reduce_partials(parts, nparts);
    if (threadIdx.x == 0) *result = s.x;
}

}  // namespace

int reduce_parts() { return std::max(1, std::min(512, 2 * ctx().num_sms)); }

void krylov_start(KrylovState *st, const double2 *psi, double2 *v0, int64_t n, double2 *parts, int *stop) {
    const int np = reduce_parts();
    k_norm_part<<<np, KT, 0, ctx().stream>>>(psi, n, parts);
    counted();
    k_start<<<np, KT, 0, ctx().stream>>>(st, psi, v0, n, parts, np, stop);
    counted();
    KV_CUDA(cudaGetLastError());
}

// Whether the fused step fits one co-resident wave on this device (checked
// once per device).  The fused step runs only on the main context's stream:
// kernels of one stream never overlap, so its grid barrier waits on no
// other launch of this library.
static bool lanczos_step_fused(int device, int np) {
    static std::mutex mu;
    static int ok[64] = {};  // 0 unknown, 1 yes, -1 no
    if (device < 0 || device >= 64) return false;
    std::lock_guard<std::mutex> lk(mu);
    if (ok[device] == 0) {
        int coop = 0, per_sm = 0, sms = 0;
        KV_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device));
        KV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        KV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lanczos_step, KT, 0));
        ok[device] = (coop && (int64_t)per_sm * sms >= np) ? 1 : -1;
    }
    return ok[device] > 0;
}

void krylov_step(KrylovState *st, int k, double2 *hv, const double2 *vprev, const double2 *vk, double2 *vnext,
                 const KrylovLens &nl, double2 *parts, double tol, int max_iter, int *stop) {
    int np = reduce_parts();
    double2 *P0 = parts, *P1 = parts + np;
    cudaStream_t s = ctx().stream;
    int64_t n_prev = k > 0 ? nl.n[k - 1] : 0, n_k = nl.n[k], n_next = nl.n[k + 1];
    if (&ctx() == &main_ctx() && lanczos_step_fused(ctx().device, np)) {
        void *args[] = {&st, &k, &hv, &vprev, &vk, &vnext, &n_prev, &n_k, &n_next, &P0, &P1, &np, &tol, &max_iter,
                        &stop};
        KV_CUDA(cudaLaunchCooperativeKernel((const void *)k_lanczos_step, dim3(np), dim3(KT), args, 0, s));
        counted();
        return;
    }
    if (k > 0) {
        k_dot_part<<<np, KT, 0, s>>>(st, hv, vprev, n_prev, P0);
        counted();
        k_sub<<<np, KT, 0, s>>>(st, hv, vprev, vk, n_prev, n_k, P0, P1, np, &st->beta[k - 1]);
        counted();
    } else {
        k_dot_part<<<np, KT, 0, s>>>(st, hv, vk, n_k, P1);
        counted();
    }
    k_sub<<<np, KT, 0, s>>>(st, hv, vk, nullptr, n_k, n_next, P1, P0, np, &st->alpha[k]);
    counted();
    k_normalize<<<np, KT, 0, s>>>(st, hv, vnext, n_next, P0, np, k, tol, max_iter, stop);
    counted();
    KV_CUDA(cudaGetLastError());
}

void tridiag_exp(KrylovState *st, int reverse) {
    k_tridiag_exp<<<1, 32, 0, ctx().stream>>>(st, reverse);
    counted();
    KV_CUDA(cudaGetLastError());
}

void krylov_finish(KrylovState *st, double2 *const *dV, double2 *out, const KrylovLens &nl, int reverse) {
    k_tridiag_exp<<<1, 32, 0, ctx().stream>>>(st, reverse);
    counted();
    k_combine<<<reduce_parts(), KT, 0, ctx().stream>>>(st, dV, out, nl);
    counted();
    KV_CUDA(cudaGetLastError());
}

void vec_norm2(const double2 *x, int64_t n, double2 *parts, double *result) {
    const int np = reduce_parts();
    k_norm_part<<<np, KT, 0, ctx().stream>>>(x, n, parts);
    counted();
    k_store_norm2<<<1, KT, 0, ctx().stream>>>(parts, np, result);
    counted();
    KV_CUDA(cudaGetLastError());
}

}  // namespace kv
