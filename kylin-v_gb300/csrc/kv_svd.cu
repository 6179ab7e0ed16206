// Device block SVD for svd_impl (holstein/svd.h:296-440).
//
// Each charge sector's dense matrix is gathered in tall orientation T (p x q,
// p >= q, column-major; T = A or T = A^H), orthogonalised by one-sided
// (Hestenes) Jacobi with round-robin ordering (one CTA per sector, each warp
// rotates disjoint column pairs, rows split across lanes), and sorted by
// descending singular value.  The host applies the reference's global
// truncation and the scatter kernel writes the kept columns into the U and
// S.V^H block tensors.
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
        if (d.side == 0) { i = (int)(e / d.kept); j = (int)(e % d.kept); dst = e; }
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

void svd_jacobi_f32(const SvdPlan &p, const double2 *T64, float2 *T, int *status, int max_sweeps, float tol) {
    if (p.secs.empty()) return;
    // dynamic shared memory: opt-in maximum less the static arrays and 4 KB
    // (set once; kv_sweep_batched runs this from several threads)
    static int smem_bytes = 0;
    static std::once_flag once;
    std::call_once(once, [] {
        int optin = 0;
        KV_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx().device));
        const int bytes = std::max(0, optin - 4096 - (int)sizeof(float) * kJacobiMaxQ);
        KV_CUDA(cudaFuncSetAttribute(k_svd_jacobi_w<1024, 16, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        KV_CUDA(cudaFuncSetAttribute(k_svd_jacobi_w<1024, 16, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        KV_CUDA(cudaFuncSetAttribute(k_svd_jacobi_w<1024, 16, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        KV_CUDA(cudaFuncSetAttribute(k_svd_jacobi_w<1024, 16, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        smem_bytes = bytes;
    });
    int64_t max_pq = 0;
    int max_p = 0;
    for (auto &s : p.secs) {
        KV_REQUIRE(s.q <= kJacobiMaxQ, KV_EINVAL, "mixed-precision SVD: a sector has more than 2048 columns");
        max_pq = std::max<int64_t>(max_pq, (int64_t)s.p * s.q);
        max_p = std::max(max_p, s.p);
    }
    const int cap = smem_bytes / (int)sizeof(float2);
    const int elems = (int)std::min<int64_t>(max_pq, cap);
    k_to_f32<<<std::max(1, ctx().num_sms * 4), 256, 0, ctx().stream>>>(T64, T, p.t_elems);
    counted();
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
    static std::once_flag once;  // the limit is raised once, to the largest size allowed here
    std::call_once(once, [] {
        KV_CUDA(cudaFuncSetAttribute(k_trsm_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrsmSmemMax));
    });
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
