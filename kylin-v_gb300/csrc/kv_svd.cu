// Device block SVD for svd_impl (holstein/svd.h:296-440).
//
// Each charge sector's dense matrix is gathered in tall orientation T (p x q,
// p >= q, column-major; T = A or T = A^H), orthogonalised by one-sided
// (Hestenes) Jacobi with round-robin ordering (one CTA per sector, each warp
// rotates disjoint column pairs, rows split across lanes), and sorted by
// descending singular value.  The host applies the reference's global
// truncation and the scatter kernel writes the kept columns into the U and
// S.V^H block tensors.
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

__device__ __forceinline__ void warp_sum3(double &a, double &b, double &cr, double &ci) {
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        cr += __shfl_xor_sync(0xffffffffu, cr, o);
        ci += __shfl_xor_sync(0xffffffffu, ci, o);
    }
}

// One CTA per sector.  status[sector] = sweeps used (negative: no convergence).
__global__ void __launch_bounds__(ST) k_svd_jacobi(const SvdSector *__restrict__ secs, double2 *__restrict__ T,
                                                   double2 *__restrict__ V, int *status, int max_sweeps,
                                                   double tol) {
    const SvdSector s = secs[blockIdx.x];
    const int p = s.p, q = s.q;
    double2 *t = T + s.t_off;
    double2 *v = V + s.v_off;
    for (int64_t e = threadIdx.x; e < (int64_t)q * q; e += ST)
        v[e] = make_double2((e % q) == (e / q) ? 1.0 : 0.0, 0.0);
    __syncthreads();
    const int qe = q + (q & 1);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = ST / 32;
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
                double2 *x = t + (int64_t)c0 * p, *y = t + (int64_t)c1 * p;
                double a = 0.0, b = 0.0, cr = 0.0, ci = 0.0;
                for (int i = lane; i < p; i += 32) {
                    double2 xi = x[i], yi = y[i];
                    a += xi.x * xi.x + xi.y * xi.y;
                    b += yi.x * yi.x + yi.y * yi.y;
                    cr += xi.x * yi.x + xi.y * yi.y;
                    ci += xi.x * yi.y - xi.y * yi.x;
                }
                warp_sum3(a, b, cr, ci);
                kvj::Rot<double> R;
                if (!kvj::make_rotation<double>(a, b, cr, ci, tol, R)) continue;
                if (lane == 0) rotated = 1;
                for (int i = lane; i < p; i += 32) {
                    double2 xi = x[i], yi = y[i];
                    kvj::rotate_pair(R, xi.x, xi.y, yi.x, yi.y);
                    x[i] = xi;
                    y[i] = yi;
                }
                double2 *vx = v + (int64_t)c0 * q, *vy = v + (int64_t)c1 * q;
                for (int i = lane; i < q; i += 32) {
                    double2 xi = vx[i], yi = vy[i];
                    kvj::rotate_pair(R, xi.x, xi.y, yi.x, yi.y);
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

// singular values, descending order, normalised U columns
__global__ void __launch_bounds__(ST) k_svd_finalize(const SvdSector *__restrict__ secs, const double2 *__restrict__ T,
                                                     const double2 *__restrict__ V, double2 *__restrict__ Us,
                                                     double2 *__restrict__ Vs, double *__restrict__ S) {
    const SvdSector s = secs[blockIdx.x];
    const int p = s.p, q = s.q;
    extern __shared__ double sv[];  // q norms
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = ST / 32;
    for (int j = warp; j < q; j += nw) {
        double a = 0.0;
        for (int i = lane; i < p; i += 32) {
            double2 x = T[s.t_off + (int64_t)j * p + i];
            a += x.x * x.x + x.y * x.y;
        }
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) sv[j] = sqrt(a);
    }
    __syncthreads();
    for (int j = warp; j < q; j += nw) {
        const double sj = sv[j];
        int rank = 0;
        for (int i = 0; i < q; ++i) rank += (sv[i] > sj) || (sv[i] == sj && i < j);
        const double inv = sj > 0.0 ? 1.0 / sj : 0.0;
        for (int i = lane; i < p; i += 32) {
            double2 x = T[s.t_off + (int64_t)j * p + i];
            Us[s.t_off + (int64_t)rank * p + i] = make_double2(x.x * inv, x.y * inv);
        }
        for (int i = lane; i < q; i += 32) Vs[s.v_off + (int64_t)rank * q + i] = V[s.v_off + (int64_t)j * q + i];
        if (lane == 0) S[s.s_off + rank] = sj;
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
    k_svd_jacobi<<<(unsigned)p.secs.size(), ST, 0, ctx().stream>>>(p.d_secs.as<SvdSector>(), T, V, status,
                                                                    max_sweeps, tol);
    counted();
    KV_CUDA(cudaGetLastError());
}

void svd_finalize(const SvdPlan &p, const double2 *T, const double2 *V, double2 *Us, double2 *Vs, double *S) {
    if (p.secs.empty()) return;
    k_svd_finalize<<<(unsigned)p.secs.size(), ST, sizeof(double) * p.max_q, ctx().stream>>>(
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

}  // namespace kv
