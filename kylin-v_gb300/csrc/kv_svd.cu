// Device block SVD for svd_impl (holstein/svd.h:296-440) and the SA-1TDVP
// split (holstein/svd.h:443-614).
//
// Each charge sector's dense matrix is gathered as T (p x q, column-major;
// T = A or T = A^H) and factorised by one CTA:
//  * FP64 mode: T tall (p >= q), one-sided (Hestenes) Jacobi with round-robin
//    ordering and accumulated rotations (k_svd_jacobi), sorted by descending
//    singular value (k_svd_finalize);
//  * mixed mode: T oriented so the wanted singular vectors are its columns, a
//    pivoted Householder reduction of its rows to the numerical rank, then
//    FP32 one-sided Jacobi on the rank-r factor, all in shared memory
//    (k_svd_qrj, the Jacobi with the columns in registers); sectors beyond
//    shared memory take the same reduction on an L2-resident workspace
//    (k_svd_qr_g) and the global-memory Jacobi (k_svd_jacobi_w).  The FP64
//    rebuild of the kept factor (k_svd_extract, k_col_norm2, k_chol,
//    k_trsm_rows with the FP64 GEMM) runs after the host's truncation.
// The host applies the reference's global truncation and the scatter kernel
// writes the kept columns into the U and S.V^H block tensors; the SA split's
// new directions come from k_sa_basis / k_sa_subtract / k_sa_scatter.
#include <mutex>
#include "kv_internal.h"
#include "kv_jacobi.cuh"
#include "kv_svd.h"

namespace kv {

namespace {

constexpr int ST = 256;

__global__ void __launch_bounds__(256) k_svd_gather(const SvdGather *__restrict__ g, const SvdSector *__restrict__ secs,
                                                    const double2 *__restrict__ A, double2 *__restrict__ T) {
    const SvdGather d = g[blockIdx.x];
    const SvdSector s = secs[d.sector];
    const int64_t n = (int64_t)d.nrows * d.ncols;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
        const int i = (int)(e / d.ncols), j = (int)(e % d.ncols);
        double2 v = A[d.blk_off + e];
        if (!s.transposed) T[s.t_off + (d.row_off + i) + (int64_t)(d.col_off + j) * s.p] = v;
        else { v.y = -v.y; T[s.t_off + (d.col_off + j) + (int64_t)(d.row_off + i) * s.p] = v; }
    }
}

template <class R>
struct Cx;
template <>
struct Cx<double> { using T = double2; };
template <>
struct Cx<float> { using T = float2; };

template <class R>
__device__ __forceinline__ void warp_sum3(R &a, R &b, R &cr, R &ci) {
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        cr += __shfl_xor_sync(0xffffffffu, cr, o);
        ci += __shfl_xor_sync(0xffffffffu, ci, o);
    }
}

// One CTA per sector, NT threads.  status[sector] = sweeps used (negative:
// no convergence within max_sweeps).
template <class R, int NT>
__global__ void __launch_bounds__(NT) k_svd_jacobi(const SvdSector *__restrict__ secs, typename Cx<R>::T *__restrict__ T,
                                                   typename Cx<R>::T *__restrict__ V, int *status, int max_sweeps,
                                                   R tol) {
    using C = typename Cx<R>::T;
    const SvdSector s = secs[blockIdx.x];
    const int p = s.p, q = s.q;
    C *t = T + s.t_off;
    C *v = V + s.v_off;
    for (int64_t e = threadIdx.x; e < (int64_t)q * q; e += NT) {
        C one;
        one.x = (e % q) == (e / q) ? R(1) : R(0);
        one.y = R(0);
        v[e] = one;
    }
    __syncthreads();
    const int qe = q + (q & 1);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = NT / 32;
    __shared__ int rotated;
    int sweep = 0;
    bool converged = (q < 2);
    for (; sweep < max_sweeps && !converged; ++sweep) {
        if (threadIdx.x == 0) rotated = 0;
        __syncthreads();
        for (int r = 0; r < qe - 1; ++r) {
            for (int pi = warp; pi < qe / 2; pi += nw) {
                int c0, c1;
                kvj::tournament_pair(qe, r, pi, c0, c1);
                if (c1 >= q) continue;
                C *x = t + (int64_t)c0 * p, *y = t + (int64_t)c1 * p;
                R a = 0, b = 0, cr = 0, ci = 0;
                for (int i = lane; i < p; i += 32) {
                    C xi = x[i], yi = y[i];
                    a += xi.x * xi.x + xi.y * xi.y;
                    b += yi.x * yi.x + yi.y * yi.y;
                    cr += xi.x * yi.x + xi.y * yi.y;
                    ci += xi.x * yi.y - xi.y * yi.x;
                }
                warp_sum3<R>(a, b, cr, ci);
                kvj::Rot<R> rot;
                if (!kvj::make_rotation<R>(a, b, cr, ci, tol, rot)) continue;
                if (lane == 0) rotated = 1;
                for (int i = lane; i < p; i += 32) {
                    C xi = x[i], yi = y[i];
                    kvj::rotate_pair(rot, xi.x, xi.y, yi.x, yi.y);
                    x[i] = xi;
                    y[i] = yi;
                }
                C *vx = v + (int64_t)c0 * q, *vy = v + (int64_t)c1 * q;
                for (int i = lane; i < q; i += 32) {
                    C xi = vx[i], yi = vy[i];
                    kvj::rotate_pair(rot, xi.x, xi.y, yi.x, yi.y);
                    vx[i] = xi;
                    vy[i] = yi;
                }
            }
            __syncthreads();
        }
        converged = (rotated == 0);
        __syncthreads();
    }
    if (threadIdx.x == 0) status[blockIdx.x] = converged ? sweep : -sweep;
}

// Mixed mode: one-sided Jacobi in FP32 without accumulated rotations.  T is
// oriented so that the singular vectors wanted afterwards are its own columns
// (they converge to sigma_j w_j); T stays in shared memory when p*q <=
// smem_elems.  Each column pair of a round is handled by a group of G lanes
// (G = 16: two pairs per warp; a group's 16 consecutive rows are one full
// pass over the shared-memory banks).  Columns below 1e-7 of ||T||_F are
// numerically zero in FP32 and are not rotated (this also lets wide T, q > p,
// converge: its q - p surplus columns go to zero).
//
// EPL > 0 (columns of at most G * EPL rows; the launch picks 2, 4 or 8 from
// its longest column): each lane keeps its EPL elements
// of the pair in registers between the dot product and the rotation, and the
// complex arithmetic runs as packed FP32 pairs (fma.rn.f32x2: the real and
// imaginary parts in one instruction).
template <int NT, int G, int EPL>
__global__ void __launch_bounds__(NT) k_svd_jacobi_w(const SvdSector *__restrict__ secs, float2 *__restrict__ T,
                                                     int *status, int max_sweeps, float tol, int smem_elems) {
    extern __shared__ float2 sT[];
    __shared__ int rotated;
    __shared__ float red[NT / 32];
    __shared__ float nrm[kJacobiMaxQ];  // |column|^2, recomputed every sweep, updated per rotation
    const SvdSector s = secs[blockIdx.x];
    const int p = s.p, q = s.q;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = NT / 32;
    const int gl = threadIdx.x % G, grp = threadIdx.x / G, ngrp = NT / G;
    const unsigned gmask = (G == 32) ? 0xFFFFFFFFu : (((1u << G) - 1u) << (lane & ~(G - 1)));
    float2 *g = T + s.t_off;
    const int64_t n = (int64_t)p * q;
    const bool in_smem = n <= smem_elems;
    float2 *t = in_smem ? sT : g;
    float fro = 0.f;
    for (int64_t e = threadIdx.x; e < n; e += NT) {
        const float2 v = g[e];
        if (in_smem) sT[e] = v;
        fro += v.x * v.x + v.y * v.y;
    }
    for (int o = 16; o > 0; o >>= 1) fro += __shfl_xor_sync(0xffffffffu, fro, o);
    if (lane == 0) red[warp] = fro;
    __syncthreads();
    float tot = 0.f;
    for (int w = 0; w < nw; ++w) tot += red[w];
    const float zt = 1e-14f * tot;  // (1e-7 ||T||_F)^2
    const int qe = q + (q & 1), m1 = qe - 1;
    int sweep = 0;
    bool converged = (q < 2);
    for (; sweep < max_sweeps && !converged; ++sweep) {
        for (int j = warp; j < q; j += nw) {
            float a = 0.f;
            for (int i = lane; i < p; i += 32) {
                const float2 x = t[(int64_t)j * p + i];
                a += x.x * x.x + x.y * x.y;
            }
            for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
            if (lane == 0) nrm[j] = a;
        }
        if (threadIdx.x == 0) rotated = 0;
        __syncthreads();
        for (int r = 0; r < m1; ++r) {
            for (int pi = grp; pi < qe / 2; pi += ngrp) {
                // round-robin pairing (position 0 fixed, the rest rotate by r)
                int c0 = 0, c1;
                if (pi > 0) { c0 = pi - 1 + r; if (c0 >= m1) c0 -= m1; ++c0; }
                c1 = qe - 2 - pi + r; if (c1 >= m1) c1 -= m1; ++c1;
                if (c0 > c1) { const int x = c0; c0 = c1; c1 = x; }
                if (c1 >= q) continue;  // uniform within the group
                const float a = nrm[c0], b = nrm[c1];
                if (!(a > zt) || !(b > zt)) continue;
                float2 *x = t + (int64_t)c0 * p, *y = t + (int64_t)c1 * p;
                float cr = 0, ci = 0;
                float2 xv[EPL > 0 ? EPL : 1], yv[EPL > 0 ? EPL : 1];
                if constexpr (EPL > 0) {
                    // (sum xr yr, sum xi yi) and (sum xr yi, sum xi yr)
                    float2 a1 = make_float2(0.f, 0.f), a2 = make_float2(0.f, 0.f);
#pragma unroll
                    for (int k = 0; k < EPL; ++k) {
                        const int i = gl + k * G;
                        xv[k] = i < p ? x[i] : make_float2(0.f, 0.f);
                        yv[k] = i < p ? y[i] : make_float2(0.f, 0.f);
                        a1 = __ffma2_rn(xv[k], yv[k], a1);
                        a2 = __ffma2_rn(xv[k], make_float2(yv[k].y, yv[k].x), a2);
                    }
                    cr = a1.x + a1.y;
                    ci = a2.x - a2.y;
                } else {
                    for (int i = gl; i < p; i += G) {
                        const float2 xi = x[i], yi = y[i];
                        cr += xi.x * yi.x + xi.y * yi.y;
                        ci += xi.x * yi.y - xi.y * yi.x;
                    }
                }
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1) {
                    cr += __shfl_xor_sync(gmask, cr, o, G);
                    ci += __shfl_xor_sync(gmask, ci, o, G);
                }
                // the rotation of kvj::make_rotation, keeping tan(theta) for the norm update:
                // the new squared norms are a - tan |c| and b + tan |c|
                const float ac = sqrtf(cr * cr + ci * ci);
                if (!(ac > tol * sqrtf(a * b))) continue;
                const float z = (b - a) / (2.f * ac);
                const float tn = copysignf(1.f, z) / (fabsf(z) + sqrtf(1.f + z * z));
                kvj::Rot<float> rot;
                rot.cs = 1.f / sqrtf(1.f + tn * tn);
                const float sn = tn * rot.cs;
                rot.s_re = sn * cr / ac;
                rot.s_im = sn * ci / ac;
                if (gl == 0) {
                    rotated = 1;
                    nrm[c0] = a - tn * ac;
                    nrm[c1] = b + tn * ac;
                }
                if constexpr (EPL > 0) {
                    // x' = cs x - s_re y - s_im (yi, -yr),  y' = cs y + s_re x + s_im (-xi, xr)
                    const float2 cs2 = make_float2(rot.cs, rot.cs), sr2 = make_float2(rot.s_re, rot.s_re);
                    const float2 msr2 = make_float2(-rot.s_re, -rot.s_re), pm = make_float2(-rot.s_im, rot.s_im);
#pragma unroll
                    for (int k = 0; k < EPL; ++k) {
                        const int i = gl + k * G;
                        const float2 xo = xv[k], yo = yv[k];
                        float2 nx = __fmul2_rn(cs2, xo);
                        nx = __ffma2_rn(msr2, yo, nx);
                        nx = __ffma2_rn(pm, make_float2(yo.y, yo.x), nx);
                        float2 ny = __fmul2_rn(cs2, yo);
                        ny = __ffma2_rn(sr2, xo, ny);
                        ny = __ffma2_rn(pm, make_float2(xo.y, xo.x), ny);
                        if (i < p) {
                            x[i] = nx;
                            y[i] = ny;
                        }
                    }
                } else {
                    for (int i = gl; i < p; i += G) {
                        float2 xi = x[i], yi = y[i];
                        kvj::rotate_pair(rot, xi.x, xi.y, yi.x, yi.y);
                        x[i] = xi;
                        y[i] = yi;
                    }
                }
            }
            __syncthreads();
        }
        converged = (rotated == 0);
        __syncthreads();
    }
    if (in_smem)
        for (int64_t e = threadIdx.x; e < n; e += NT) g[e] = sT[e];
    if (threadIdx.x == 0) status[blockIdx.x] = converged ? sweep : -sweep;
}

// One-sided Jacobi on the r columns of the row-major block sw (p rows, row
// stride ldw) by a CTA of 512 threads: round-robin pairs, one group of GJ
// lanes a pair, tolerance tol2 on the squared cosine, columns with norm^2 at
// or below zt left alone.  With E > 0 each lane holds its E elements of both
// columns (rows gjl + k GJ; p <= E GJ) in registers between the dot product
// and the rotation; E == 0 loops over the rows.  The caller picks GJ from r so
// that the r/2 pairs of a round keep most of the 16 warps busy.  cn: [r]
// scratch.  Returns the sweeps used, negative if max_sweeps ran out.
template <int GJ, int E>
__device__ __forceinline__ int qrj_jacobi(float2 *sw, int ldw, int p, int r, float *cn, int *rotated,
                                          int max_sweeps, float tol2, float zt) {
    constexpr int NT = 512, NW = NT / 32;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int gj = tid / GJ, gjl = tid % GJ, ngj = NT / GJ;
    const unsigned jmask = GJ == 32 ? 0xFFFFFFFFu : (((1u << GJ) - 1u) << (lane & ~(GJ - 1)));
    const int qe = r + (r & 1), m1 = qe - 1;
    int sweep = 0;
    bool converged = r < 2;
    for (; sweep < max_sweeps && !converged; ++sweep) {
        for (int j = warp; j < r; j += NW) {
            float a = 0.f;
            for (int i = lane; i < p; i += 32) {
                const float2 x = sw[i * ldw + j];
                a += x.x * x.x + x.y * x.y;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xFFFFFFFFu, a, o);
            if (lane == 0) cn[j] = a;
        }
        if (tid == 0) *rotated = 0;
        __syncthreads();
        for (int rr = 0; rr < m1; ++rr) {
            for (int pi = gj; pi < qe / 2; pi += ngj) {
                int c0 = 0, c1;
                if (pi > 0) { c0 = pi - 1 + rr; if (c0 >= m1) c0 -= m1; ++c0; }
                c1 = qe - 2 - pi + rr; if (c1 >= m1) c1 -= m1; ++c1;
                if (c0 > c1) { const int x = c0; c0 = c1; c1 = x; }
                if (c1 >= r) continue;  // group-uniform from here on
                const float a = cn[c0], b = cn[c1];
                if (!(a > zt) || !(b > zt)) continue;
                float cr = 0.f, ci = 0.f;
                float2 xv[E > 0 ? E : 1], yv[E > 0 ? E : 1];
                if constexpr (E > 0) {
                    // two accumulator pairs (even / odd k) halve the dependent
                    // chain where registers allow (E <= 8)
                    float2 a1 = make_float2(0.f, 0.f), a2 = a1, a3 = a1, a4 = a1;
#pragma unroll
                    for (int kk = 0; kk < E; ++kk) {
                        const int i = gjl + kk * GJ;
                        xv[kk] = i < p ? sw[i * ldw + c0] : make_float2(0.f, 0.f);
                        yv[kk] = i < p ? sw[i * ldw + c1] : make_float2(0.f, 0.f);
                        const float2 ys = make_float2(yv[kk].y, yv[kk].x);
                        if ((kk & 1) && E <= 8) {
                            a3 = __ffma2_rn(xv[kk], yv[kk], a3);
                            a4 = __ffma2_rn(xv[kk], ys, a4);
                        } else {
                            a1 = __ffma2_rn(xv[kk], yv[kk], a1);
                            a2 = __ffma2_rn(xv[kk], ys, a2);
                        }
                    }
                    cr = (a1.x + a3.x) + (a1.y + a3.y);
                    ci = (a2.x + a4.x) - (a2.y + a4.y);
                } else {
                    for (int i = gjl; i < p; i += GJ) {
                        const float2 xi = sw[i * ldw + c0], yi = sw[i * ldw + c1];
                        cr += xi.x * yi.x + xi.y * yi.y;
                        ci += xi.x * yi.y - xi.y * yi.x;
                    }
                }
#pragma unroll
                for (int o = GJ / 2; o > 0; o >>= 1) {
                    cr += __shfl_xor_sync(jmask, cr, o, GJ);
                    ci += __shfl_xor_sync(jmask, ci, o, GJ);
                }
                // |c|^2 <= tol^2 a b: the pair is orthogonal to the tolerance
                const float ac2 = cr * cr + ci * ci;
                if (!(ac2 > tol2 * a * b)) continue;
                // t = sign(z) / (|z| + sqrt(1 + z^2)), z = (b - a) / (2|c|), from
                // hardware reciprocal square roots and one fast reciprocal: an
                // inexact t only changes the angle, and (cs, sn) below stay a
                // rotation to FP32 rounding whatever t is.  |z| is clamped so
                // 1 + z^2 stays finite.
                const float rac = rsqrtf(ac2);  // 1 / |c|
                const float ac = ac2 * rac;
                const float z = fminf(fmaxf(0.5f * (b - a) * rac, -1e18f), 1e18f);
                const float w = fmaf(z, z, 1.f);
                const float tn = copysignf(__fdividef(1.f, fabsf(z) + w * rsqrtf(w)), z);
                kvj::Rot<float> rot;
                rot.cs = rsqrtf(fmaf(tn, tn, 1.f));
                const float sn = tn * rot.cs;
                rot.s_re = sn * cr * rac;
                rot.s_im = sn * ci * rac;
                if (gjl == 0) {
                    *rotated = 1;
                    cn[c0] = a - tn * ac;
                    cn[c1] = b + tn * ac;
                }
                if constexpr (E > 0) {
                    const float2 cs2 = make_float2(rot.cs, rot.cs), sr2 = make_float2(rot.s_re, rot.s_re);
                    const float2 msr2 = make_float2(-rot.s_re, -rot.s_re), pm = make_float2(-rot.s_im, rot.s_im);
#pragma unroll
                    for (int kk = 0; kk < E; ++kk) {
                        const int i = gjl + kk * GJ;
                        const float2 xo = xv[kk], yo = yv[kk];
                        float2 nx = __fmul2_rn(cs2, xo);
                        nx = __ffma2_rn(msr2, yo, nx);
                        nx = __ffma2_rn(pm, make_float2(yo.y, yo.x), nx);
                        float2 ny = __fmul2_rn(cs2, yo);
                        ny = __ffma2_rn(sr2, xo, ny);
                        ny = __ffma2_rn(pm, make_float2(xo.y, xo.x), ny);
                        if (i < p) {
                            sw[i * ldw + c0] = nx;
                            sw[i * ldw + c1] = ny;
                        }
                    }
                } else {
                    for (int i = gjl; i < p; i += GJ) {
                        float2 xi = sw[i * ldw + c0], yi = sw[i * ldw + c1];
                        kvj::rotate_pair(rot, xi.x, xi.y, yi.x, yi.y);
                        sw[i * ldw + c0] = xi;
                        sw[i * ldw + c1] = yi;
                    }
                }
            }
            __syncthreads();
        }
        converged = (*rotated == 0);
        __syncthreads();
    }
    return converged ? sweep : -sweep;
}

// Exchange columns of qrj_jacobi_reg: r/2 + 1 columns of the GJ * E packed
// elements a group holds (rows padded past p), the column stride 8 (mod 16)
// float2 so that the four 8-lane pieces one warp moves at a time fall in two
// shared-memory wavefronts, and their norms.  rows: the launch's 8 * EPL.
__host__ __device__ constexpr int qrj_xch_stride(int rows) { return ((rows + 15) / 16) * 16 + 8; }
__host__ __device__ constexpr size_t qrj_xch_bytes(int rows, int kmax) {
    return (size_t)(kmax / 2 + 2) * ((size_t)qrj_xch_stride(rows) * sizeof(float2) + sizeof(float));
}

// The same Jacobi with the columns held in registers for a whole sweep.
// Ordering: odd-even transposition with every pair swapped after its
// rotation, on the N = r + (r & 1) positions (column r is a zero column when r
// is odd): even rounds pair positions (2g, 2g+1), odd rounds (2g+1, 2g+2);
// such a network reverses the order in N rounds, so every pair of columns
// meets exactly once per sweep.  Group g holds (X, Y) = positions (2g, 2g+1)
// in even rounds and (2g+1, 2g+2) in odd ones (group n-1 idles in odd rounds
// holding positions (2n-1, 0)); after each round one column per group moves
// to a neighbouring group: even -> odd Y_g <- Y_{g+1 mod n}; odd -> even
// X_g <- X_{g-1}, X_0 <- Y_{n-1}, Y_{n-1} <- X_{n-1}.  The moving columns go
// through shared memory, one store and one load per element for every lane
// (a warp moves four 8-row pieces at a time, two wavefronts).  The streamed
// form reads and writes both columns of every pair each round; this moves
// one.  On return column 2g holds X and 2g+1 holds Y of group g (positions of
// the even layout): the caller sorts all N columns.  xch: qrj_xch_bytes(GJ E,
// r) of shared memory.
template <int GJ, int E>
__device__ __forceinline__ int qrj_jacobi_reg(float2 *sw, int ldw, int p, int r, unsigned char *xch, int *rotated,
                                              int max_sweeps, float tol2, float zt) {
    constexpr int H = E / 2;
    static_assert(GJ * E <= 128 && GJ <= 32 && E % 2 == 0, "row cover");
    // Each lane holds rows gjl + k GJ (k < E) of its two columns as H pairs of
    // rows (2h, 2h+1), real and imaginary parts apart (XR[h] = (re, re), XI[h]
    // = (im, im)), so the complex dot products and rotations are packed FP32
    // pairs with no swapping of halves.
    constexpr int ps = qrj_xch_stride(GJ * E);
    float2 *xd = reinterpret_cast<float2 *>(xch);  // [n + 1] exchange columns of stride ps
    const int qe = r + (r & 1), n = qe / 2;
    float *xn = reinterpret_cast<float *>(xd + (n + 1) * ps);  // [n + 1] their norms
    const int tid = threadIdx.x, lane = tid & 31;
    const int g = tid / GJ, gjl = tid % GJ;  // group, lane in the group
    const unsigned jmask = GJ == 32 ? 0xFFFFFFFFu : (((1u << GJ) - 1u) << (lane & ~(GJ - 1)));
    const bool act = g < n;
    float2 XR[H], XI[H], YR[H], YI[H];
#pragma unroll
    for (int h = 0; h < H; ++h) {
        const int i0 = gjl + 2 * h * GJ, i1 = i0 + GJ;
        const float2 z = make_float2(0.f, 0.f);
        const float2 x0 = (act && i0 < p && 2 * g < r) ? sw[i0 * ldw + 2 * g] : z;
        const float2 x1 = (act && i1 < p && 2 * g < r) ? sw[i1 * ldw + 2 * g] : z;
        const float2 y0 = (act && i0 < p && 2 * g + 1 < r) ? sw[i0 * ldw + 2 * g + 1] : z;
        const float2 y1 = (act && i1 < p && 2 * g + 1 < r) ? sw[i1 * ldw + 2 * g + 1] : z;
        XR[h] = make_float2(x0.x, x1.x);
        XI[h] = make_float2(x0.y, x1.y);
        YR[h] = make_float2(y0.x, y1.x);
        YI[h] = make_float2(y0.y, y1.y);
    }
    auto gsum = [&](float v) {
#pragma unroll
        for (int o = GJ / 2; o > 0; o >>= 1) v += __shfl_xor_sync(jmask, v, o, GJ);
        return v;
    };
    float nx = 0.f, ny = 0.f;
    int sweep = 0;
    bool converged = r < 2;
    for (; sweep < max_sweeps && !converged; ++sweep) {
        {
            float2 a = make_float2(0.f, 0.f), b = a;
#pragma unroll
            for (int h = 0; h < H; ++h) {
                a = __ffma2_rn(XR[h], XR[h], a);
                a = __ffma2_rn(XI[h], XI[h], a);
                b = __ffma2_rn(YR[h], YR[h], b);
                b = __ffma2_rn(YI[h], YI[h], b);
            }
            nx = gsum(a.x + a.y);
            ny = gsum(b.x + b.y);
        }
        if (tid == 0) *rotated = 0;
        __syncthreads();
        for (int t = 0; t < qe; ++t) {
            const bool odd = t & 1;
            // ---- rotate this group's pair: c = <X, Y> = sum conj(x) y
            if (act && !(odd && g == n - 1) && nx > zt && ny > zt) {
                float2 ar = make_float2(0.f, 0.f), ai = ar, bi = ar;
#pragma unroll
                for (int h = 0; h < H; ++h) {
                    ar = __ffma2_rn(XR[h], YR[h], ar);
                    ar = __ffma2_rn(XI[h], YI[h], ar);
                    ai = __ffma2_rn(XR[h], YI[h], ai);
                    bi = __ffma2_rn(XI[h], YR[h], bi);
                }
                const float cr = gsum(ar.x + ar.y);
                const float ci = gsum((ai.x + ai.y) - (bi.x + bi.y));
                const float ac2 = cr * cr + ci * ci;
                if (ac2 > tol2 * nx * ny) {  // group-uniform
                    const float rac = rsqrtf(ac2);
                    const float ac = ac2 * rac;
                    const float z = fminf(fmaxf(0.5f * (ny - nx) * rac, -1e18f), 1e18f);
                    const float w = fmaf(z, z, 1.f);
                    const float tn = copysignf(__fdividef(1.f, fabsf(z) + w * rsqrtf(w)), z);
                    const float cs = rsqrtf(fmaf(tn, tn, 1.f));
                    const float sn = tn * cs;
                    const float s_re = sn * cr * rac, s_im = sn * ci * rac;
                    if (gjl == 0) *rotated = 1;
                    nx = nx - tn * ac;
                    ny = ny + tn * ac;
                    // x' = cs x - conj(s) y, y' = cs y + s x, s = s_re + i s_im
                    const float2 cs2 = make_float2(cs, cs), sr2 = make_float2(s_re, s_re), si2 = make_float2(s_im, s_im);
                    const float2 msr2 = make_float2(-s_re, -s_re), msi2 = make_float2(-s_im, -s_im);
#pragma unroll
                    for (int h = 0; h < H; ++h) {
                        const float2 xr = XR[h], xi = XI[h], yr = YR[h], yi = YI[h];
                        XR[h] = __ffma2_rn(msi2, yi, __ffma2_rn(msr2, yr, __fmul2_rn(cs2, xr)));
                        XI[h] = __ffma2_rn(si2, yr, __ffma2_rn(msr2, yi, __fmul2_rn(cs2, xi)));
                        YR[h] = __ffma2_rn(msi2, xi, __ffma2_rn(sr2, xr, __fmul2_rn(cs2, yr)));
                        YI[h] = __ffma2_rn(si2, xr, __ffma2_rn(sr2, xi, __fmul2_rn(cs2, yi)));
                    }
                }
            }
            // ---- move one column per group through the exchange columns
            // (column c at xd + c * ps, the lanes' packed pairs as they are held;
            // norms at xn[c]): store, barrier, load, barrier (the next round's
            // stores wait for every load)
            float2 *mine = xd + g * ps + gjl;
            if (!odd) {
                // Y_g <- Y_{(g+1) mod n}
                if (act) {
#pragma unroll
                    for (int h = 0; h < H; ++h) {
                        mine[2 * h * GJ] = YR[h];
                        mine[(2 * h + 1) * GJ] = YI[h];
                    }
                    if (gjl == 0) xn[g] = ny;
                }
                __syncthreads();
                if (act) {
                    const int src = g + 1 < n ? g + 1 : 0;
                    const float2 *from = xd + src * ps + gjl;
#pragma unroll
                    for (int h = 0; h < H; ++h) {
                        YR[h] = from[2 * h * GJ];
                        YI[h] = from[(2 * h + 1) * GJ];
                    }
                    ny = xn[src];
                }
            } else {
                // X_g <- X_{g-1}, X_0 <- Y_{n-1} (column n), Y_{n-1} <- X_{n-1}
                if (act) {
#pragma unroll
                    for (int h = 0; h < H; ++h) {
                        mine[2 * h * GJ] = XR[h];
                        mine[(2 * h + 1) * GJ] = XI[h];
                    }
                    if (g == n - 1) {
                        float2 *tail = xd + n * ps + gjl;
#pragma unroll
                        for (int h = 0; h < H; ++h) {
                            tail[2 * h * GJ] = YR[h];
                            tail[(2 * h + 1) * GJ] = YI[h];
                        }
                    }
                    if (gjl == 0) {
                        xn[g] = nx;
                        if (g == n - 1) xn[n] = ny;
                    }
                }
                __syncthreads();
                if (act) {
                    if (g == n - 1) {
#pragma unroll
                        for (int h = 0; h < H; ++h) {
                            YR[h] = XR[h];
                            YI[h] = XI[h];
                        }
                        ny = nx;
                    }
                    const int src = g == 0 ? n : g - 1;
                    const float2 *from = xd + src * ps + gjl;
#pragma unroll
                    for (int h = 0; h < H; ++h) {
                        XR[h] = from[2 * h * GJ];
                        XI[h] = from[(2 * h + 1) * GJ];
                    }
                    nx = xn[src];
                }
            }
            __syncthreads();
        }
        converged = (*rotated == 0);
        __syncthreads();
    }
    if (act) {
#pragma unroll
        for (int h = 0; h < H; ++h) {
            const int i0 = gjl + 2 * h * GJ, i1 = i0 + GJ;
            if (i0 < p) {
                sw[i0 * ldw + 2 * g] = make_float2(XR[h].x, XI[h].x);
                sw[i0 * ldw + 2 * g + 1] = make_float2(YR[h].x, YI[h].x);
            }
            if (i1 < p) {
                sw[i1 * ldw + 2 * g] = make_float2(XR[h].y, XI[h].y);
                sw[i1 * ldw + 2 * g + 1] = make_float2(YR[h].y, YI[h].y);
            }
        }
    }
    __syncthreads();
    return converged ? sweep : -sweep;
}

// QR-preconditioned one-sided Jacobi (mixed mode).  One CTA of 512 threads
// per charge sector; the sector is held in shared memory in FP32 as p rows of
// length q (row stride q + 1, so reads of one column by consecutive rows fall
// in distinct banks), scaled by a power of two so that its largest element
// lies in [0.5, 1).  The wanted singular vectors are T's left ones (its
// column space).
//
//  1. Pivoted Householder from the right on T's rows: at step k the row with
//     the largest trailing norm (positions k..q-1) is the pivot; the unitary
//     reflector H_k with x H_k = (beta, 0, ..., 0) for that row's trailing part
//     x is applied to every row not yet pivoted.  After r steps
//     T H_1 ... H_r = [M | E]: M = T Q (p x r, Q the first r columns of the
//     product) and E has rows of norm below qr_floor * ||T||_F, where the loop
//     stops.  T = M Q^H + E Q'^H, so T's left singular vectors above the FP32
//     noise level are M's.  One barrier per step: every warp finds the next
//     pivot itself from the per-warp maxima of the previous step (double
//     buffered), and each row's exact trailing norm is accumulated while the
//     row is updated.  A group of 16 lanes updates two rows at once, so each
//     pivot-row element it loads serves both.
//  2. One-sided Jacobi on M's r columns (qrj_jacobi: round-robin pairs, 32,
//     16 or 8 lanes a pair for r <= 32, <= 64 or more, so that a round's r/2
//     pairs occupy most warps; each lane holds its elements of both columns in
//     registers between the dot product and the rotation, 8 EPL rows per pair
//     in all; tolerance `tol` on the cosine).  M is row-pivoted triangular, so
//     it converges in fewer sweeps than T, and only r columns are rotated.
//  3. Columns sorted by norm: S = norms (descending), Us = normalised columns
//     (column-major p x r at the sector's t_off), S = 0 in the sector's
//     remaining slots up to q.
// status[sector] = Jacobi sweeps used (negative: no convergence), ranks[sector] = r.
// Load one sector into sw (p rows of stride ldw, in shared or global memory)
// in FP32 scaled by a power of two (*up is the inverse factor), then the
// pivoted Householder reduction of its rows to the numerical rank r (rows
// below qr_floor ||T||_F dropped); on return M = sw's first r columns with
// conj(alpha_k) at (piv[k], k) and zeros beyond.  Returns r, or -1 for a
// sector holding Inf or NaN.  alph, piv: [min(p, q)]; done: [p].  512 threads.
__device__ __forceinline__ int qrj_reduce(const SvdSector &s, const double2 *__restrict__ T64, float2 *sw, int ldw,
                                          float2 *alph, int *piv, int *done, float qr_floor, double *up,
                                          float *fro2_out) {
    constexpr int NT = 512, NW = NT / 32;
    constexpr int GQ = 16;  // lanes per row (two rows at a time)
    __shared__ float wbest[2][NW];
    __shared__ int wbesti[2][NW];
    __shared__ float red[NW];
    __shared__ double dred[NW];
    const int p = s.p, q = s.q, kmax = min(p, q);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // ---- load (FP64 column-major p x q -> FP32 rows) scaled by a power of two
    // that brings the largest element to [0.5, 1): sectors whose entries are
    // far below 1 would otherwise underflow FP32 in the squared norms
    const double2 *src = T64 + s.t_off;
    const int pq = p * q;
    double amax = 0.0;  // largest |re|, |im|; +inf if any element is Inf or NaN
    for (int e = tid; e < pq; e += NT) {
        const double2 v = src[e];
        const double m = fmax(fabs(v.x), fabs(v.y));
        amax = (isfinite(v.x) && isfinite(v.y)) ? fmax(amax, m) : INFINITY;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xFFFFFFFFu, amax, o));
    if (lane == 0) dred[warp] = amax;
    __syncthreads();
    amax = 0.0;
    for (int w = 0; w < NW; ++w) amax = fmax(amax, dred[w]);
    if (!isfinite(amax)) return -1;  // a non-finite sector (uniform over the CTA)
    int ex = 0;
    if (amax > 0.0) frexp(amax, &ex);
    const double down = ldexp(1.0, -ex);  // exact powers of two
    *up = ldexp(1.0, ex);
    for (int e = tid; e < pq; e += NT) {
        const int i = e % p, c = e / p;
        const double2 v = src[e];
        sw[i * ldw + c] = make_float2((float)(v.x * down), (float)(v.y * down));
    }
    __syncthreads();

    // ---- row norms, the first pivot candidates per warp, Frobenius norm
    const int gq = tid / GQ, gql = tid % GQ, ngq = NT / GQ;
    const unsigned qmask = 0xFFFFu << (lane & ~(GQ - 1));
    float bv = -1.f;
    int bi = 0x7FFFFFFF;
    float fro = 0.f;
    for (int i0 = 0; i0 < p; i0 += ngq) {
        const int i = i0 + gq;
        float a = 0.f;
        if (i < p)
            for (int c = gql; c < q; c += GQ) {
                const float2 w = sw[i * ldw + c];
                a += w.x * w.x + w.y * w.y;
            }
#pragma unroll
        for (int o = GQ / 2; o > 0; o >>= 1) a += __shfl_xor_sync(qmask, a, o, GQ);
        if (i < p) {
            if (gql == 0) { done[i] = 0; fro += a; }
            if (a > bv || (a == bv && i < bi)) { bv = a; bi = i; }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xFFFFFFFFu, bv, o);
        const int oi = __shfl_xor_sync(0xFFFFFFFFu, bi, o);
        if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
        fro += __shfl_xor_sync(0xFFFFFFFFu, fro, o);
    }
    if (lane == 0) { wbest[0][warp] = bv; wbesti[0][warp] = bi; red[warp] = fro; }
    __syncthreads();
    float fro2 = 0.f;
    for (int w = 0; w < NW; ++w) fro2 += red[w];
    const float thr2 = qr_floor * qr_floor * fro2;
    *fro2_out = fro2;

    // ---- pivoted Householder on the rows
    int r = 0;
    for (int k = 0; k < kmax; ++k) {
        const int cur = k & 1;
        float mv = lane < NW ? wbest[cur][lane] : -1.f;
        int mi = lane < NW ? wbesti[cur][lane] : 0x7FFFFFFF;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(0xFFFFFFFFu, mv, o);
            const int oi = __shfl_xor_sync(0xFFFFFFFFu, mi, o);
            if (ov > mv || (ov == mv && oi < mi)) { mv = ov; mi = oi; }
        }
        if (!(mv > thr2) || mi >= p) break;  // uniform: every warp computed the same maximum
        r = k + 1;
        const int ip = mi;
        const float2 *xr = sw + ip * ldw;
        // u = conj(x), alpha = -e^{i phi} |u| (phi = arg u_0), v = u - alpha e_0,
        // beta = 2 / |v|^2 = 1 / (|u| (|u| + |u_0|));  x H = conj(alpha) e_0^T
        const float nu = sqrtf(mv);
        const float2 x0 = xr[k];
        const float a0 = sqrtf(x0.x * x0.x + x0.y * x0.y);
        const float ph_r = a0 > 0.f ? x0.x / a0 : 1.f, ph_i = a0 > 0.f ? -x0.y / a0 : 0.f;  // e^{i phi}
        const float2 v0 = make_float2(ph_r * (a0 + nu), ph_i * (a0 + nu));              // u_0 - alpha
        const float beta = 1.f / (nu * (nu + a0));
        if (tid == 0) {
            alph[k] = make_float2(-ph_r * nu, ph_i * nu);  // conj(alpha)
            piv[k] = ip;
            done[ip] = 1;
        }
        float gbv = -1.f;
        int gbi = 0x7FFFFFFF;
        for (int i0 = gq; i0 < p; i0 += 2 * ngq) {
            const int iA = i0, iB = i0 + ngq;
            // group-uniform: every lane of the group has the same rows
            const bool lA = iA != ip && !done[iA];
            const bool lB = iB < p && iB != ip && !done[iB];
            if (!lA && !lB) continue;
            float2 *wa = sw + iA * ldw, *wb = sw + (lB ? iB : iA) * ldw;
            // s = sum_c w_c v_c, v_c = conj(x_c) for c > k, v_k = v0
            float sar = 0.f, sai = 0.f, sbr = 0.f, sbi = 0.f;
#pragma unroll 4
            for (int c = k + gql; c < q; c += GQ) {
                const float2 xc = xr[c];
                const float2 vc = c == k ? v0 : make_float2(xc.x, -xc.y);
                const float2 a = wa[c], b = wb[c];
                sar += a.x * vc.x - a.y * vc.y;
                sai += a.x * vc.y + a.y * vc.x;
                sbr += b.x * vc.x - b.y * vc.y;
                sbi += b.x * vc.y + b.y * vc.x;
            }
#pragma unroll
            for (int o = GQ / 2; o > 0; o >>= 1) {
                sar += __shfl_xor_sync(qmask, sar, o, GQ);
                sai += __shfl_xor_sync(qmask, sai, o, GQ);
                sbr += __shfl_xor_sync(qmask, sbr, o, GQ);
                sbi += __shfl_xor_sync(qmask, sbi, o, GQ);
            }
            const float far = lA ? beta * sar : 0.f, fai = lA ? beta * sai : 0.f;
            const float fbr = lB ? beta * sbr : 0.f, fbi = lB ? beta * sbi : 0.f;
            float ta = 0.f, tb = 0.f;
#pragma unroll 4
            for (int c = k + gql; c < q; c += GQ) {
                const float2 xc = xr[c];
                const float2 cv = c == k ? make_float2(v0.x, -v0.y) : xc;  // conj(v_c)
                float2 a = wa[c], b = wb[c];
                a.x -= far * cv.x - fai * cv.y;
                a.y -= far * cv.y + fai * cv.x;
                b.x -= fbr * cv.x - fbi * cv.y;
                b.y -= fbr * cv.y + fbi * cv.x;
                if (lA) wa[c] = a;
                if (lB) wb[c] = b;
                if (c > k) {
                    ta += a.x * a.x + a.y * a.y;
                    tb += b.x * b.x + b.y * b.y;
                }
            }
#pragma unroll
            for (int o = GQ / 2; o > 0; o >>= 1) {
                ta += __shfl_xor_sync(qmask, ta, o, GQ);
                tb += __shfl_xor_sync(qmask, tb, o, GQ);
            }
            if (lA && (ta > gbv || (ta == gbv && iA < gbi))) { gbv = ta; gbi = iA; }
            if (lB && (tb > gbv || (tb == gbv && iB < gbi))) { gbv = tb; gbi = iB; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(0xFFFFFFFFu, gbv, o);
            const int oi = __shfl_xor_sync(0xFFFFFFFFu, gbi, o);
            if (ov > gbv || (ov == gbv && oi < gbi)) { gbv = ov; gbi = oi; }
        }
        if (lane == 0) { wbest[cur ^ 1][warp] = gbv; wbesti[cur ^ 1][warp] = gbi; }
        __syncthreads();
    }
    // pivot rows: conj(alpha_k) at position k, zeros after it (within the r columns kept)
    for (int e = tid; e < r * r; e += NT) {
        const int kk = e / r, c = e % r;
        if (c >= kk) sw[piv[kk] * ldw + c] = c == kk ? alph[kk] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    return r;
}

template <int EPL>
__global__ void __launch_bounds__(512, 1) k_svd_qrj(const SvdSector *__restrict__ secs,
                                                    const double2 *__restrict__ T64, float2 *__restrict__ Us,
                                                    double *__restrict__ S, int *status, int *ranks, int max_sweeps,
                                                    float tol, float qr_floor, int use_reg) {
    constexpr int NT = 512, NW = NT / 32;
    extern __shared__ float2 sw[];
    __shared__ int rotated;
    const SvdSector s = secs[blockIdx.x];
    const int p = s.p, q = s.q, ldw = q + 1, kmax = min(p, q);
    float2 *alph = sw + p * ldw;                          // [kmax] conj(alpha_k)
    float *cn = reinterpret_cast<float *>(alph + kmax);   // [kmax + 1] column norms^2 (Jacobi), then norms
    int *piv = reinterpret_cast<int *>(cn + kmax + 1);    // [kmax] pivot rows
    int *done = piv + kmax;                               // [p] row already pivoted
    // [qrj_xch_bytes(8 EPL, kmax)] exchange columns of the register-resident Jacobi (use_reg)
    unsigned char *xch = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(done + p) + 15) & ~static_cast<uintptr_t>(15));
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    double up = 1.0;
    float fro2 = 0.f;
    const int r = qrj_reduce(s, T64, sw, ldw, alph, piv, done, qr_floor, &up, &fro2);
    if (r < 0) {  // a non-finite sector: its singular values are NaN (reported by the host)
        for (int j = tid; j < q; j += NT) S[s.s_off + j] = nan("");
        if (tid == 0) {
            status[blockIdx.x] = 0;
            ranks[blockIdx.x] = 0;
        }
        return;
    }

    // ---- one-sided Jacobi on the r columns of M; the group width follows r
    // (r/2 pairs a round), the register capacity per lane follows EPL
    const float zt = 1e-14f * fro2;  // (1e-7 ||T||_F)^2: numerically zero columns
    const float tol2 = tol * tol;
    int sweeps;
    int ncol = r;  // columns holding the result (r + 1 when the register form ran on odd r)
    if constexpr (EPL > 0) {
        constexpr int E32 = EPL >= 4 ? EPL / 4 : 1;
        if (use_reg && r <= 128 && (r > 32 || E32 >= 2)) {
            ncol = r + (r & 1);
            if (r <= 32) sweeps = qrj_jacobi_reg<32, (E32 >= 2 ? E32 : 2)>(sw, ldw, p, r, xch, &rotated, max_sweeps, tol2, zt);
            else if (r <= 64) sweeps = qrj_jacobi_reg<16, EPL / 2>(sw, ldw, p, r, xch, &rotated, max_sweeps, tol2, zt);
            else sweeps = qrj_jacobi_reg<8, EPL>(sw, ldw, p, r, xch, &rotated, max_sweeps, tol2, zt);
        } else if (r <= 32) {
            sweeps = qrj_jacobi<32, E32>(sw, ldw, p, r, cn, &rotated, max_sweeps, tol2, zt);
        } else if (r <= 64) {
            sweeps = qrj_jacobi<16, EPL / 2>(sw, ldw, p, r, cn, &rotated, max_sweeps, tol2, zt);
        } else {
            sweeps = qrj_jacobi<8, EPL>(sw, ldw, p, r, cn, &rotated, max_sweeps, tol2, zt);
        }
    } else {
        sweeps = qrj_jacobi<8, 0>(sw, ldw, p, r, cn, &rotated, max_sweeps, tol2, zt);
    }

    // ---- sorted singular values and normalised columns (of ncol columns the
    // r largest: a zero column beyond r sorts last)
    for (int j = warp; j < ncol; j += NW) {
        float a = 0.f;
        for (int i = lane; i < p; i += 32) {
            const float2 x = sw[i * ldw + j];
            a += x.x * x.x + x.y * x.y;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xFFFFFFFFu, a, o);
        if (lane == 0) cn[j] = sqrtf(a);
    }
    __syncthreads();
    for (int j = warp; j < ncol; j += NW) {
        const float sj = cn[j];
        int rank = 0;
        for (int i = 0; i < ncol; ++i) rank += (cn[i] > sj) || (cn[i] == sj && i < j);
        if (rank >= r) continue;  // warp-uniform
        const float inv = sj > 0.f ? 1.f / sj : 0.f;
        for (int i = lane; i < p; i += 32) {
            const float2 x = sw[i * ldw + j];
            Us[s.t_off + (int64_t)rank * p + i] = make_float2(x.x * inv, x.y * inv);
        }
        if (lane == 0) S[s.s_off + rank] = (double)sj * up;
    }
    for (int j = r + tid; j < q; j += NT) S[s.s_off + j] = 0.0;  // every one of the sector's q slots
    if (tid == 0) {
        status[blockIdx.x] = sweeps;
        ranks[blockIdx.x] = r;
    }
}

// Sectors too large for shared memory (mixed mode): the same load and
// pivoted Householder reduction (qrj_reduce) on a global, L2-resident
// workspace W (p rows of stride q + 1 at w_off[sector]), then M written
// column-major into T32 (p x q at the sector's t_off, unscaled, columns r..q-1
// zero) for the global-memory Jacobi, ranks[sector] = r.  A sector holding Inf
// or NaN gets NaN in T32 and rank 0, so its singular values come out NaN.
// Dynamic shared memory: alph [kmax] float2, piv [kmax] int, done [p] int.
__global__ void __launch_bounds__(512, 1) k_svd_qr_g(const SvdSector *__restrict__ secs,
                                                     const double2 *__restrict__ T64, float2 *__restrict__ W,
                                                     const int64_t *__restrict__ w_off, float2 *__restrict__ T32,
                                                     int *ranks, float qr_floor) {
    extern __shared__ float2 sm_qr[];
    const SvdSector s = secs[blockIdx.x];
    const int p = s.p, q = s.q, ldw = q + 1, kmax = min(p, q);
    float2 *sw = W + w_off[blockIdx.x];
    float2 *alph = sm_qr;
    int *piv = reinterpret_cast<int *>(alph + kmax);
    int *done = piv + kmax;
    double up = 1.0;
    float fro2 = 0.f;
    const int r = qrj_reduce(s, T64, sw, ldw, alph, piv, done, qr_floor, &up, &fro2);
    float2 *out = T32 + s.t_off;
    const int64_t pq = (int64_t)p * q;
    if (r < 0) {
        const float nanf_ = __int_as_float(0x7FC00000);
        for (int64_t e = threadIdx.x; e < pq; e += blockDim.x) out[e] = make_float2(nanf_, nanf_);
        if (threadIdx.x == 0) ranks[blockIdx.x] = 0;
        return;
    }
    for (int64_t e = threadIdx.x; e < pq; e += blockDim.x) {
        const int i = (int)(e % p), j = (int)(e / p);
        const float2 v = j < r ? sw[(int64_t)i * ldw + j] : make_float2(0.f, 0.f);
        out[e] = make_float2((float)((double)v.x * up), (float)((double)v.y * up));
    }
    if (threadIdx.x == 0) ranks[blockIdx.x] = r;
}

// singular values (as double), descending order, normalised U columns
template <class R>
__global__ void __launch_bounds__(256) k_svd_finalize(const SvdSector *__restrict__ secs,
                                                      const typename Cx<R>::T *__restrict__ T,
                                                      const typename Cx<R>::T *__restrict__ V,
                                                      typename Cx<R>::T *__restrict__ Us,
                                                      typename Cx<R>::T *__restrict__ Vs, double *__restrict__ S) {
    using C = typename Cx<R>::T;
    const SvdSector s = secs[blockIdx.x];
    const int p = s.p, q = s.q;
    extern __shared__ unsigned char sv_raw[];  // q norms, in the Jacobi's precision
    R *sv = reinterpret_cast<R *>(sv_raw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = 256 / 32;
    for (int j = warp; j < q; j += nw) {
        R a = 0;
        for (int i = lane; i < p; i += 32) {
            C x = T[s.t_off + (int64_t)j * p + i];
            a += x.x * x.x + x.y * x.y;
        }
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) sv[j] = sqrt(a);
    }
    __syncthreads();
    for (int j = warp; j < q; j += nw) {
        const R sj = sv[j];
        int rank = 0;
        for (int i = 0; i < q; ++i) rank += (sv[i] > sj) || (sv[i] == sj && i < j);
        const R inv = sj > R(0) ? R(1) / sj : R(0);
        for (int i = lane; i < p; i += 32) {
            C x = T[s.t_off + (int64_t)j * p + i];
            x.x *= inv;
            x.y *= inv;
            Us[s.t_off + (int64_t)rank * p + i] = x;
        }
        if (V)
            for (int i = lane; i < q; i += 32) Vs[s.v_off + (int64_t)rank * q + i] = V[s.v_off + (int64_t)j * q + i];
        if (lane == 0) S[s.s_off + rank] = sj;
    }
}

__global__ void k_to_f32(const double2 *__restrict__ in, float2 *__restrict__ out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = make_float2((float)in[i].x, (float)in[i].y);
}

// ------------------------------------------------------- FP64 polish
// The first k sorted Jacobi columns (the kept singular vectors of the side
// T's columns live in), each divided by its singular value, as a row-major
// FP64 matrix W (p x k): A W then has columns of norm ~1 (a well-conditioned
// start for Cholesky-QR).
__global__ void k_svd_extract(const SvdPolish *__restrict__ pol, const SvdSector *__restrict__ secs,
                              const float2 *__restrict__ Us, const double *__restrict__ S, double2 *__restrict__ W) {
    const SvdPolish d = pol[blockIdx.x];
    const SvdSector s = secs[d.sector];
    const int k = d.k;
    for (int64_t e = threadIdx.x; e < (int64_t)s.p * k; e += blockDim.x) {
        const int i = (int)(e / k), j = (int)(e % k);
        const float2 v = Us[s.t_off + (int64_t)j * s.p + i];
        const double sj = S[s.s_off + j];
        const double inv = sj > 0.0 ? 1.0 / sj : 1.0;
        W[d.w_off + e] = make_double2(v.x * inv, v.y * inv);
    }
}

// Squared norms of the columns of each polish factor X (rows x k, row stride
// ldx), written as G[g_off + j].x: one CTA per factor, one warp per column.
__global__ void k_col_norm2(const SvdPolish *__restrict__ pol, const double2 *__restrict__ X, double2 *__restrict__ G) {
    const SvdPolish d = pol[blockIdx.x];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = warp; j < d.k; j += nw) {
        double a = 0.0;
        for (int i = lane; i < d.rows; i += 32) {
            const double2 v = X[d.x_off + (int64_t)i * d.ldx + j];
            a += v.x * v.x + v.y * v.y;
        }
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xFFFFFFFFu, a, o);
        if (lane == 0) G[d.g_off + j] = make_double2(a, 0.0);
    }
}

// In place: G (k x k, row-major, Hermitian positive definite) -> upper R with
// G = R^H R (lower triangle left as is).  One CTA per sector, column-wise.
__global__ void k_chol(const SvdPolish *__restrict__ pol, double2 *__restrict__ G, int *status, double *diagv,
                       double shift) {
    const SvdPolish d = pol[blockIdx.x];
    const int k = d.k;
    double2 *g = G + d.g_off;
    __shared__ double diag;
    if (shift > 0.0 && threadIdx.x == 0) {
        // shifted Cholesky-QR: G + shift * max diag * I is safely positive definite
        double mx = 0.0;
        for (int j = 0; j < k; ++j) mx = fmax(mx, g[(int64_t)j * k + j].x);
        for (int j = 0; j < k; ++j) g[(int64_t)j * k + j].x += shift * mx;
    }
    __syncthreads();
    for (int j = 0; j < k; ++j) {
        if (threadIdx.x == 0) {
            double r = g[(int64_t)j * k + j].x;
            if ((!(r > 0.0) || !isfinite(r)) && status[blockIdx.x] == 0) {
                status[blockIdx.x] = j + 1;  // first failing pivot (1-based) for the error report
                diagv[blockIdx.x] = r;
            }
            if (!(r > 0.0) || !isfinite(r)) r = 1e-300;
            diag = sqrt(r);
            g[(int64_t)j * k + j] = make_double2(diag, 0.0);
        }
        __syncthreads();
        const double inv = 1.0 / diag;
        for (int c = j + 1 + threadIdx.x; c < k; c += blockDim.x) {  // row j of R
            double2 v = g[(int64_t)j * k + c];
            g[(int64_t)j * k + c] = make_double2(v.x * inv, v.y * inv);
        }
        __syncthreads();
        // trailing update G[a, b] -= conj(R[j, a]) R[j, b] for j < a <= b
        for (int64_t e = threadIdx.x; e < (int64_t)(k - j - 1) * (k - j - 1); e += blockDim.x) {
            const int a = j + 1 + (int)(e / (k - j - 1)), b = j + 1 + (int)(e % (k - j - 1));
            if (b < a) continue;
            const double2 ra = g[(int64_t)j * k + a], rb = g[(int64_t)j * k + b];
            double2 v = g[(int64_t)a * k + b];
            v.x -= ra.x * rb.x + ra.y * rb.y;
            v.y -= ra.x * rb.y - ra.y * rb.x;
            g[(int64_t)a * k + b] = v;
        }
        __syncthreads();
    }
}

// X <- X R^{-1} row by row (R upper, from k_chol): y_c = (x_c - sum_{a<c} y_a R[a,c]) / R[c,c].
// One warp per row (kTrsmRows rows per CTA): the solved y live in shared
// memory, lanes split each inner sum, a shuffle tree reduces it.
__global__ void __launch_bounds__(32 * kTrsmRows) k_trsm_rows(const SvdPolish *__restrict__ pol,
                                                              const int *__restrict__ item_pol,
                                                              const int *__restrict__ item_row0,
                                                              const double2 *__restrict__ G, double2 *__restrict__ X) {
    extern __shared__ double2 ys[];  // [kTrsmRows][kmax]
    const SvdPolish d = pol[item_pol[blockIdx.x]];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = item_row0[blockIdx.x] + warp;
    if (row >= d.rows) return;  // warp-uniform
    const int k = d.k;
    const double2 *r = G + d.g_off;
    double2 *x = X + d.x_off + (int64_t)row * d.ldx;
    double2 *y = ys + (int64_t)warp * k;
    for (int c = 0; c < k; ++c) {
        double sr = 0.0, si = 0.0;
        for (int a = lane; a < c; a += 32) {
            const double2 ya = y[a], rac = r[(int64_t)a * k + c];
            sr += ya.x * rac.x - ya.y * rac.y;
            si += ya.x * rac.y + ya.y * rac.x;
        }
        for (int o = 16; o > 0; o >>= 1) {
            sr += __shfl_xor_sync(0xFFFFFFFFu, sr, o);
            si += __shfl_xor_sync(0xFFFFFFFFu, si, o);
        }
        if (lane == 0) {
            const double2 v = x[c];
            const double inv = 1.0 / r[(int64_t)c * k + c].x;
            y[c] = make_double2((v.x - sr) * inv, (v.y - si) * inv);
        }
        __syncwarp();
    }
    for (int a = lane; a < k; a += 32) x[a] = y[a];
}

// output blocks from dense row-major factors: side 0 block[i, j] = M[(pos+i)*ld + j]
// (conj-transposed source: M[j*ld + pos+i] conjugated); side 1 block[j, c] = M[j*ld + pos+c]
// (conj-transposed source: conj(M[(pos+c)*ld + j]))
__global__ void k_scatter_dense(const SvdDense *__restrict__ d_, const double2 *__restrict__ M, double2 *__restrict__ out) {
    const SvdDense d = d_[blockIdx.x];
    const int64_t n = (int64_t)d.len * d.kept;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
        double2 v;
        if (d.side == 0) {
            const int i = (int)(e / d.kept), j = (int)(e % d.kept);
            v = d.ctrans ? M[d.m_off + (int64_t)j * d.ld + d.pos + i] : M[d.m_off + (int64_t)(d.pos + i) * d.ld + j];
        } else {
            const int j = (int)(e / d.len), c = (int)(e % d.len);
            v = d.ctrans ? M[d.m_off + (int64_t)(d.pos + c) * d.ld + j] : M[d.m_off + (int64_t)j * d.ld + d.pos + c];
        }
        if (d.ctrans) v.y = -v.y;
        out[d.out_off + e] = v;
    }
}

__global__ void __launch_bounds__(256) k_svd_scatter(const SvdScatter *__restrict__ d_,
                                                     const SvdSector *__restrict__ secs,
                                                     const double2 *__restrict__ Us, const double2 *__restrict__ Vs,
                                                     const double *__restrict__ S, double2 *__restrict__ out) {
    const SvdScatter d = d_[blockIdx.x];
    const SvdSector s = secs[d.sector];
    const int64_t n = (int64_t)d.len * d.kept;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
        int i, j;  // i: position inside the micro block (row or column), j: kept state
        int64_t dst;
        if (d.side == 0) { i = (int)(e / d.kept); j = (int)(e % d.kept); dst = (int64_t)i * d.ld + j; }
        else { j = (int)(e / d.len); i = (int)(e % d.len); dst = e; }
        const int r = d.pos + i;
        double2 val;
        if (d.side == 0) {  // U_A[r, j]
            val = s.transposed ? Vs[s.v_off + (int64_t)j * s.q + r] : Us[s.t_off + (int64_t)j * s.p + r];
        } else {  // Vt_A[j, r] = conj(V_A[r, j])
            val = s.transposed ? Us[s.t_off + (int64_t)j * s.p + r] : Vs[s.v_off + (int64_t)j * s.q + r];
            val.y = -val.y;
        }
        if (d.scale_s) {
            const double sj = S[s.s_off + j];
            val.x *= sj;
            val.y *= sj;
        }
        out[d.out_off + dst] = val;
    }
}

// SA-1TDVP: B[r, j] = U_A[r, j] (side 0) or conj(V_A[r, j]) (side 1), the
// sources k_svd_scatter reads
__global__ void __launch_bounds__(256) k_sa_basis(const SaSector *__restrict__ sa, const SvdSector *__restrict__ secs,
                                                  const double2 *__restrict__ Us, const double2 *__restrict__ Vs,
                                                  double2 *__restrict__ B) {
    const SaSector d = sa[blockIdx.x];
    const SvdSector s = secs[d.sector];
    for (int64_t e = threadIdx.x; e < (int64_t)d.n * d.kept; e += blockDim.x) {
        const int r = (int)(e / d.kept), j = (int)(e % d.kept);
        double2 v;
        if (d.side == 0) {
            v = s.transposed ? Vs[s.v_off + (int64_t)j * s.q + r] : Us[s.t_off + (int64_t)j * s.p + r];
        } else {
            v = s.transposed ? Us[s.t_off + (int64_t)j * s.p + r] : Vs[s.v_off + (int64_t)j * s.q + r];
            v.y = -v.y;
        }
        B[d.b_off + e] = v;
    }
}

__global__ void __launch_bounds__(256) k_sa_subtract(double2 *__restrict__ x, const double2 *__restrict__ y,
                                                     int64_t n) {
    for (int64_t i = blockIdx.x * 256ll + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256) {
        x[i].x -= y[i].x;
        x[i].y -= y[i].y;
    }
}

__global__ void __launch_bounds__(256) k_sa_scatter(const SaOut *__restrict__ v, const double2 *__restrict__ X,
                                                    double2 *__restrict__ out) {
    const SaOut d = v[blockIdx.x];
    const int ld = d.kept + d.ext;
    for (int64_t e = threadIdx.x; e < (int64_t)d.len * d.ext; e += blockDim.x) {
        const int i = (int)(e / d.ext), c = (int)(e % d.ext);
        const double2 x = X[d.x_off + (int64_t)(d.pos + i) * d.ext + c];
        if (d.side == 0) out[d.out_off + (int64_t)i * ld + d.kept + c] = x;
        else out[d.out_off + (int64_t)(d.kept + c) * d.len + i] = x;
    }
}

constexpr int kMaxDevices = 64;
std::mutex g_attr_mu;
int g_jacobi_smem[kMaxDevices];
bool g_jacobi_set[kMaxDevices], g_trsm_set[kMaxDevices];

// per device: raise the Jacobi kernels' dynamic shared-memory limit once and
// return it (function attributes belong to the device they were set on)
int jacobi_smem_limit(int dev) {
    KV_REQUIRE(dev >= 0 && dev < kMaxDevices, KV_EINVAL, "device index out of range");
    std::lock_guard<std::mutex> lk(g_attr_mu);
    if (!g_jacobi_set[dev]) {
        int optin = 0;
        KV_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        const int bytes = std::max(0, optin - 4096 - (int)sizeof(float) * kJacobiMaxQ);
        KV_CUDA(cudaFuncSetAttribute(k_svd_jacobi_w<1024, 16, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        KV_CUDA(cudaFuncSetAttribute(k_svd_jacobi_w<1024, 16, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        KV_CUDA(cudaFuncSetAttribute(k_svd_jacobi_w<1024, 16, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        KV_CUDA(cudaFuncSetAttribute(k_svd_jacobi_w<1024, 16, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        g_jacobi_smem[dev] = bytes;
        g_jacobi_set[dev] = true;
    }
    return g_jacobi_smem[dev];
}

bool g_qrj_set[kMaxDevices];
int g_qrj_smem[kMaxDevices];

// per device: the QR-Jacobi kernels may use the whole opt-in shared memory
int qrj_smem_limit(int dev) {
    KV_REQUIRE(dev >= 0 && dev < kMaxDevices, KV_EINVAL, "device index out of range");
    std::lock_guard<std::mutex> lk(g_attr_mu);
    if (!g_qrj_set[dev]) {
        int optin = 0;
        KV_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        const int bytes = std::max(0, optin - 1024);  // less the kernel's static arrays
        KV_CUDA(cudaFuncSetAttribute(k_svd_qrj<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        KV_CUDA(cudaFuncSetAttribute(k_svd_qrj<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        KV_CUDA(cudaFuncSetAttribute(k_svd_qrj<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        KV_CUDA(cudaFuncSetAttribute(k_svd_qrj<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        KV_CUDA(cudaFuncSetAttribute(k_svd_qr_g, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        g_qrj_smem[dev] = bytes;
        g_qrj_set[dev] = true;
    }
    return g_qrj_smem[dev];
}

void trsm_smem_raise(int dev, int bytes) {
    KV_REQUIRE(dev >= 0 && dev < kMaxDevices, KV_EINVAL, "device index out of range");
    std::lock_guard<std::mutex> lk(g_attr_mu);
    if (!g_trsm_set[dev]) {
        KV_CUDA(cudaFuncSetAttribute(k_trsm_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        g_trsm_set[dev] = true;
    }
}

}  // namespace

void svd_gather(const SvdPlan &p, const double2 *A, double2 *T) {
    launch_zero(T, p.t_elems);
    if (!p.gathers.empty()) {
        k_svd_gather<<<(unsigned)p.gathers.size(), 256, 0, ctx().stream>>>(p.d_gathers.as<SvdGather>(),
                                                                           p.d_secs.as<SvdSector>(), A, T);
        counted();
    }
    KV_CUDA(cudaGetLastError());
}

void svd_jacobi(const SvdPlan &p, double2 *T, double2 *V, int *status, int max_sweeps, double tol) {
    if (p.secs.empty()) return;
    k_svd_jacobi<double, ST><<<(unsigned)p.secs.size(), ST, 0, ctx().stream>>>(p.d_secs.as<SvdSector>(), T, V,
                                                                                status, max_sweeps, tol);
    counted();
    KV_CUDA(cudaGetLastError());
}

void svd_finalize(const SvdPlan &p, const double2 *T, const double2 *V, double2 *Us, double2 *Vs, double *S) {
    if (p.secs.empty()) return;
    k_svd_finalize<double><<<(unsigned)p.secs.size(), 256, sizeof(double) * p.max_q, ctx().stream>>>(
        p.d_secs.as<SvdSector>(), T, V, Us, Vs, S);
    counted();
    KV_CUDA(cudaGetLastError());
}

void svd_scatter(const std::vector<SvdScatter> &sc, const SvdPlan &p, const double2 *Us, const double2 *Vs,
                 const double *S, double2 *out) {
    if (sc.empty()) return;
    DevBuf d = upload_vec(sc);
    k_svd_scatter<<<(unsigned)sc.size(), 256, 0, ctx().stream>>>(d.as<SvdScatter>(), p.d_secs.as<SvdSector>(), Us,
                                                                  Vs, S, out);
    counted();
    KV_CUDA(cudaGetLastError());
}

void sa_basis(const std::vector<SaSector> &v, const SvdPlan &p, const double2 *Us, const double2 *Vs, double2 *B) {
    if (v.empty()) return;
    DevBuf d = upload_vec(v);
    k_sa_basis<<<(unsigned)v.size(), 256, 0, ctx().stream>>>(d.as<SaSector>(), p.d_secs.as<SvdSector>(), Us, Vs, B);
    counted();
    KV_CUDA(cudaGetLastError());
}

void sa_subtract(double2 *x, const double2 *y, int64_t n) {
    if (n <= 0) return;
    const unsigned grid = (unsigned)std::min<int64_t>((n + 255) / 256, 4 * ctx().num_sms);
    k_sa_subtract<<<grid, 256, 0, ctx().stream>>>(x, y, n);
    counted();
    KV_CUDA(cudaGetLastError());
}

void sa_scatter(const std::vector<SaOut> &v, const double2 *X, double2 *out) {
    if (v.empty()) return;
    DevBuf d = upload_vec(v);
    k_sa_scatter<<<(unsigned)v.size(), 256, 0, ctx().stream>>>(d.as<SaOut>(), X, out);
    counted();
    KV_CUDA(cudaGetLastError());
}

void svd_qr_global(const SvdPlan &p, const double2 *T64, float2 *T32, int *ranks, float qr_floor) {
    if (p.secs.empty()) return;
    std::vector<int64_t> w_off(p.secs.size());
    int64_t w_elems = 0;
    size_t smem = 0;
    for (size_t i = 0; i < p.secs.size(); ++i) {
        const SvdSector &sc = p.secs[i];
        w_off[i] = w_elems;
        w_elems += (int64_t)sc.p * (sc.q + 1);
        const size_t kmax = (size_t)std::min(sc.p, sc.q);
        smem = std::max(smem, kmax * (sizeof(float2) + sizeof(int)) + (size_t)sc.p * sizeof(int));
    }
    KV_REQUIRE(smem <= (size_t)qrj_smem_limit(ctx().device), KV_EINVAL,
               "mixed-precision SVD: a sector has too many rows for the QR reduction");
    DevBuf W(std::max<int64_t>(1, w_elems) * sizeof(float2));
    DevBuf dw = upload_vec(w_off);
    k_svd_qr_g<<<(unsigned)p.secs.size(), 512, smem, ctx().stream>>>(p.d_secs.as<SvdSector>(), T64, W.as<float2>(),
                                                                      dw.as<int64_t>(), T32, ranks, qr_floor);
    counted();
    KV_CUDA(cudaGetLastError());
}

void svd_jacobi_f32(const SvdPlan &p, const double2 *T64, float2 *T, int *status, int max_sweeps, float tol) {
    if (p.secs.empty()) return;
    // dynamic shared memory: opt-in maximum less the static arrays and 4 KB,
    // raised once per device (kv_sweep_batched runs this from several threads)
    const int smem_bytes = jacobi_smem_limit(ctx().device);
    int64_t max_pq = 0;
    int max_p = 0;
    for (auto &s : p.secs) {
        KV_REQUIRE(s.q <= kJacobiMaxQ, KV_EINVAL, "mixed-precision SVD: a sector has more than 2048 columns");
        max_pq = std::max<int64_t>(max_pq, (int64_t)s.p * s.q);
        max_p = std::max(max_p, s.p);
    }
    const int cap = smem_bytes / (int)sizeof(float2);
    const int elems = (int)std::min<int64_t>(max_pq, cap);
    if (T64) {
        k_to_f32<<<std::max(1, ctx().num_sms * 4), 256, 0, ctx().stream>>>(T64, T, p.t_elems);
        counted();
    }
    // elements per lane from the longest column of the launch (16 lanes a pair)
    auto launch = [&](auto kernel) {
        kernel<<<(unsigned)p.secs.size(), 1024, (size_t)elems * sizeof(float2), ctx().stream>>>(
            p.d_secs.as<SvdSector>(), T, status, max_sweeps, tol, elems);
    };
    if (max_p <= 32) launch(k_svd_jacobi_w<1024, 16, 2>);
    else if (max_p <= 64) launch(k_svd_jacobi_w<1024, 16, 4>);
    else if (max_p <= 128) launch(k_svd_jacobi_w<1024, 16, 8>);
    else launch(k_svd_jacobi_w<1024, 16, 0>);
    counted();
    KV_CUDA(cudaGetLastError());
}

// shared-memory bytes of k_svd_qrj for a p x q sector
static size_t qrj_smem(int p, int q) {
    const size_t kmax = (size_t)std::min(p, q);
    return sizeof(float2) * ((size_t)p * (q + 1) + kmax) + sizeof(float) * ((size_t)p + 2 * kmax + 1);
}

bool svd_qrjacobi_f32(const SvdPlan &p, const double2 *T64, float2 *Us, double *S, int *status, int *ranks,
                      int max_sweeps, float tol, float qr_floor) {
    if (p.secs.empty()) return true;
    const int limit = qrj_smem_limit(ctx().device);
    size_t smem = 0;
    int max_p = 0;
    for (auto &sc : p.secs) {
        smem = std::max(smem, qrj_smem(sc.p, sc.q));
        max_p = std::max(max_p, sc.p);
    }
    if (smem > (size_t)limit) return false;
    // the register-resident Jacobi where its exchange columns also fit
    const int rows = max_p <= 32 ? 32 : max_p <= 64 ? 64 : 128;  // 8 EPL of the kernel launched below
    size_t xch = 0;
    for (auto &sc : p.secs) xch = std::max(xch, qrj_smem(sc.p, sc.q) + 16 + qrj_xch_bytes(rows, std::min(sc.p, sc.q)));
    const int use_reg = max_p <= 128 && xch <= (size_t)limit ? 1 : 0;
    if (use_reg) smem = xch;
    auto launch = [&](auto kernel) {
        kernel<<<(unsigned)p.secs.size(), 512, smem, ctx().stream>>>(p.d_secs.as<SvdSector>(), T64, Us, S, status,
                                                                     ranks, max_sweeps, tol, qr_floor, use_reg);
    };
    // elements per lane from the longest column of the launch (8 lanes a pair)
    if (max_p <= 32) launch(k_svd_qrj<4>);
    else if (max_p <= 64) launch(k_svd_qrj<8>);
    else if (max_p <= 128) launch(k_svd_qrj<16>);
    else launch(k_svd_qrj<0>);
    counted();
    KV_CUDA(cudaGetLastError());
    return true;
}

void svd_finalize_f32(const SvdPlan &p, const float2 *T, float2 *Us, double *S) {
    if (p.secs.empty()) return;
    k_svd_finalize<float><<<(unsigned)p.secs.size(), 256, sizeof(double) * p.max_q, ctx().stream>>>(
        p.d_secs.as<SvdSector>(), T, nullptr, Us, nullptr, S);
    counted();
    KV_CUDA(cudaGetLastError());
}

void svd_extract(const DevBuf &pol, int npol, const SvdPlan &p, const float2 *Us, const double *S, double2 *W) {
    if (npol == 0) return;
    k_svd_extract<<<npol, 256, 0, ctx().stream>>>(pol.as<SvdPolish>(), p.d_secs.as<SvdSector>(), Us, S, W);
    counted();
    KV_CUDA(cudaGetLastError());
}

void svd_col_norm2(const DevBuf &pol, int npol, const double2 *X, double2 *G) {
    if (npol == 0) return;
    k_col_norm2<<<npol, 256, 0, ctx().stream>>>(pol.as<SvdPolish>(), X, G);
    counted();
    KV_CUDA(cudaGetLastError());
}

void svd_chol(const DevBuf &pol, int npol, double2 *G, int *status, double *diagv, double shift) {
    if (npol == 0) return;
    k_chol<<<npol, 256, 0, ctx().stream>>>(pol.as<SvdPolish>(), G, status, diagv, shift);
    counted();
    KV_CUDA(cudaGetLastError());
}

void svd_trsm(const DevBuf &pol, const std::vector<int> &item_pol, const std::vector<int> &item_row0,
              const double2 *G, double2 *X, int kmax) {
    if (item_pol.empty()) return;
    const size_t smem = (size_t)kTrsmRows * std::max(1, kmax) * sizeof(double2);
    constexpr int kTrsmSmemMax = 200 * 1024;
    KV_REQUIRE(smem <= kTrsmSmemMax, KV_EINVAL, "SVD polish: kept dimension of one sector too large");
    trsm_smem_raise(ctx().device, kTrsmSmemMax);  // once per device, to the largest size allowed here
    DevBuf ip = upload_vec(item_pol), ir = upload_vec(item_row0);
    k_trsm_rows<<<(unsigned)item_pol.size(), 32 * kTrsmRows, smem, ctx().stream>>>(pol.as<SvdPolish>(), ip.as<int>(),
                                                                                  ir.as<int>(), G, X);
    counted();
    KV_CUDA(cudaGetLastError());
}

void svd_scatter_dense(const std::vector<SvdDense> &d, const double2 *M, double2 *out) {
    if (d.empty()) return;
    DevBuf dd = upload_vec(d);
    k_scatter_dense<<<(unsigned)d.size(), 256, 0, ctx().stream>>>(dd.as<SvdDense>(), M, out);
    counted();
    KV_CUDA(cudaGetLastError());
}

}  // namespace kv
