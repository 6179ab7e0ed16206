// FP64 device kernels of the contraction engine: grouped block-sparse complex
// GEMM, MPO mixing, block permutation, fills.
#include "kv_internal.h"

namespace kv {

namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ void cfma(double2 &acc, double2 a, double2 b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}

// ------------------------------------------------------------------ GEMM
// One CTA per output tile (T x T complex, T = 32 or 16), 256 threads,
// (T/16) x (T/16) outputs per thread.  Each tile sums all block pairs
// (segments) that accumulate into it, so no atomics are needed and the
// summation order is fixed.  GB300 runs FP64 at a few multiply-adds per clock
// per SM, so a tile's K loop is long in time: the 16 x 16 tiles put four
// times as many CTAs (SMs) on the same product, for the small products of the
// SVD's FP64 rebuild.
constexpr int TK = 16;

template <int T>
__global__ void __launch_bounds__(256) k_gemm_fp64(const GemmTile *__restrict__ tiles,
                                                   const GemmSeg *__restrict__ segs,
                                                   const double2 *__restrict__ A,
                                                   const double2 *__restrict__ B, double2 *__restrict__ C,
                                                   double alpha, const int *skip, int step, int write_inactive) {
    if (skip && *skip) return;
    constexpr int TM = T, TN = T, R = T / 16;  // R x R outputs per thread
    constexpr int LOADS = (TM * TK + 255) / 256;
    __shared__ double2 As[TK][TM + 1];
    __shared__ double2 Bs[TK][TN + 1];
    const GemmTile t = tiles[blockIdx.x];
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    double2 acc[R][R] = {};
    bool any = false;
    for (int s = t.seg_begin; s < t.seg_end; ++s) {
        const GemmSeg g = segs[s];
        if (g.entry > step) continue;  // uniform over the CTA
        any = true;
        const double2 *a = A + g.a_off;
        const double2 *b = B + g.b_off;
        for (int k0 = 0; k0 < g.K; k0 += TK) {
#pragma unroll
            for (int r = 0; r < LOADS; ++r) {
                int idx = tid + r * 256;
                int m, k;
                const bool a_kc = (g.opa == 0 || g.opa == 3);  // contiguous along k
                if (a_kc) { m = idx / TK; k = idx % TK; }
                else { m = idx % TM; k = idx / TM; }
                int gm = t.m0 + m, gk = k0 + k;
                double2 v = make_double2(0.0, 0.0);
                if (gm < t.M && gk < g.K) {
                    v = a_kc ? a[(int64_t)gm * g.lda + gk] : a[(int64_t)gk * g.lda + gm];
                    if (g.opa == 1 || g.opa == 3) v.y = -v.y;
                }
                As[k][m] = v;
                int n;
                const bool b_nc = (g.opb == 0 || g.opb == 3);  // contiguous along n
                if (b_nc) { n = idx % TN; k = idx / TN; }
                else { k = idx % TK; n = idx / TK; }
                int gn = t.n0 + n;
                gk = k0 + k;
                double2 w = make_double2(0.0, 0.0);
                if (gn < t.N && gk < g.K) {
                    w = b_nc ? b[(int64_t)gk * g.ldb + gn] : b[(int64_t)gn * g.ldb + gk];
                    if (g.opb == 2 || g.opb == 3) w.y = -w.y;
                }
                Bs[k][n] = w;
            }
            __syncthreads();
#pragma unroll
            for (int kk = 0; kk < TK; ++kk) {
                double2 a[R], b[R];
#pragma unroll
                for (int i = 0; i < R; ++i) {
                    a[i] = As[kk][ty * R + i];
                    b[i] = Bs[kk][tx * R + i];
                }
#pragma unroll
                for (int i = 0; i < R; ++i)
#pragma unroll
                    for (int j = 0; j < R; ++j) cfma(acc[i][j], a[i], b[j]);
            }
            __syncthreads();
        }
    }
    if (!any && !write_inactive) return;
#pragma unroll
    for (int i = 0; i < R; ++i)
#pragma unroll
        for (int j = 0; j < R; ++j) {
            int gm = t.m0 + ty * R + i, gn = t.n0 + tx * R + j;
            if (gm < t.M && gn < t.N)
                C[t.c_off + (int64_t)gm * t.ldc + gn] = make_double2(alpha * acc[i][j].x, alpha * acc[i][j].y);
        }
}

// ------------------------------------------------------------------ mix
// out[k, k2, r, n] = sum_terms sum_kk W[k2, kk, r] in[k, kk, n]; one CTA per
// (job, chunk of kMixChunk elements).  The FP64 unit (two thread-operations
// per clock per SM on GB300) bounds this kernel, and an MPO's local operators
// are mostly zeros and real: a zero W entry adds nothing and is skipped, a
// real one takes two fused multiply-adds instead of four.  Consecutive
// threads share (k2, r), so the branch is uniform across a warp where n spans
// it; for finite inputs the sums equal the four-FMA product's (up to the
// sign of a zero sum).

__global__ void __launch_bounds__(256) k_mix(const MixItem *__restrict__ items, const MixJob *__restrict__ jobs,
                                             const MixTerm *__restrict__ terms, const double2 *__restrict__ in,
                                             const double2 *__restrict__ W, double2 *__restrict__ out,
                                             const int *skip, int step, int write_inactive) {
    if (skip && *skip) return;
    const MixItem it = items[blockIdx.x];
    const MixJob jb = jobs[it.job];
    if (!write_inactive) {
        bool any = false;
        for (int ti = jb.term_begin; ti < jb.term_end; ++ti) any = any || terms[ti].entry <= step;
        if (!any) return;
    }
    for (int j = threadIdx.x; j < kMixChunk; j += blockDim.x) {
        int64_t e = it.start + j;
        if (e >= jb.count) break;
        int64_t n = e % jb.rest;
        int64_t r = (e / jb.rest) % jb.wr;
        int64_t k2 = (e / (jb.rest * jb.wr)) % jb.so;
        int64_t k = e / (jb.rest * jb.wr * jb.so);
        double2 acc = make_double2(0.0, 0.0);
        for (int ti = jb.term_begin; ti < jb.term_end; ++ti) {
            const MixTerm tm = terms[ti];
            if (tm.entry > step) continue;
            const double2 *w = W + tm.w_off + (k2 * tm.K) * jb.wr + r;
            const double2 *x = in + tm.in_off + (k * tm.K) * jb.rest + n;
            for (int kk = 0; kk < tm.K; ++kk) {
                const double2 wv = w[(int64_t)kk * jb.wr];
                if (wv.y == 0.0) {
                    if (wv.x == 0.0) continue;
                    const double2 xv = x[(int64_t)kk * jb.rest];
                    acc.x = fma(wv.x, xv.x, acc.x);
                    acc.y = fma(wv.x, xv.y, acc.y);
                } else {
                    cfma(acc, wv, x[(int64_t)kk * jb.rest]);
                }
            }
        }
        out[jb.out_off + e] = acc;
    }
}

// ------------------------------------------------------------ permute
// desc per block (16 int64): in_off, out_off, size, rank, shape[6], perm[6]
__global__ void k_permute(const int64_t *__restrict__ desc, const double2 *__restrict__ in,
                          double2 *__restrict__ out) {
    const int64_t *d = desc + 16 * blockIdx.x;
    const int64_t in_off = d[0], out_off = d[1], size = d[2];
    const int rank = (int)d[3];
    int64_t sd[kMaxRank], od[kMaxRank], osh[kMaxRank];
    sd[rank - 1] = 1;
    for (int i = rank - 2; i >= 0; --i) sd[i] = sd[i + 1] * d[4 + i + 1];
    for (int i = 0; i < rank; ++i) osh[i] = d[4 + d[10 + i]];
    od[rank - 1] = 1;
    for (int i = rank - 2; i >= 0; --i) od[i] = od[i + 1] * osh[i + 1];
    for (int64_t e = threadIdx.x; e < size; e += blockDim.x) {
        int64_t dst = 0;
        for (int j = 0; j < rank; ++j) {
            int ax = (int)d[10 + j];
            dst += ((e / sd[ax]) % d[4 + ax]) * od[j];
        }
        out[out_off + dst] = in[in_off + e];
    }
}

__global__ void k_zero(double2 *p, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = make_double2(0.0, 0.0);
}
__global__ void k_copy(double2 *dst, const double2 *src, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

int grid_for(int64_t n, int threads) {
    int64_t g = (n + threads - 1) / threads;
    int cap = std::max(1, ctx().num_sms * 8);
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, cap));
}

}  // namespace

void launch_gemm_fp64(const GemmPlan &p, const double2 *A, const double2 *B, double2 *C, double alpha,
                      const int *skip, int step) {
    if (p.tiles.empty()) return;
    KV_REQUIRE(p.tile_m == p.tile_n && (p.tile_m == 32 || p.tile_m == 16 || p.tile_m == 0), KV_EINVAL,
               "internal: FP64 GEMM tiles are 32 x 32 or 16 x 16");
    if (p.tile_m == 16)
        k_gemm_fp64<16><<<(unsigned)p.tiles.size(), 256, 0, ctx().stream>>>(
            p.d_tiles.as<GemmTile>(), p.d_segs.as<GemmSeg>(), A, B, C, alpha, skip, step, p.write_inactive ? 1 : 0);
    else
        k_gemm_fp64<32><<<(unsigned)p.tiles.size(), 256, 0, ctx().stream>>>(
            p.d_tiles.as<GemmTile>(), p.d_segs.as<GemmSeg>(), A, B, C, alpha, skip, step, p.write_inactive ? 1 : 0);
    counted();
    KV_CUDA(cudaGetLastError());
}

void launch_mix(const MixPlan &p, const double2 *in, const double2 *W, double2 *out, const int *skip, int step) {
    if (p.items.empty()) return;
    k_mix<<<(unsigned)p.items.size(), 256, 0, ctx().stream>>>(p.d_items.as<MixItem>(), p.d_jobs.as<MixJob>(),
                                                               p.d_terms.as<MixTerm>(), in, W, out, skip, step,
                                                               p.write_inactive ? 1 : 0);
    counted();
    KV_CUDA(cudaGetLastError());
}

void launch_permute(const double2 *in, double2 *out, const std::vector<int64_t> &desc, int nblocks) {
    if (nblocks == 0) return;
    DevBuf d = upload_vec(desc);
    k_permute<<<nblocks, 256, 0, ctx().stream>>>(d.as<int64_t>(), in, out);
    counted();
    KV_CUDA(cudaGetLastError());
    // d is freed stream-ordered after the kernel
}

void launch_zero(double2 *p, int64_t n) {
    if (n <= 0) return;
    k_zero<<<grid_for(n, 256), 256, 0, ctx().stream>>>(p, n);
    counted();
    KV_CUDA(cudaGetLastError());
}

void launch_copy(double2 *dst, const double2 *src, int64_t n) {
    if (n <= 0) return;
    k_copy<<<grid_for(n, 256), 256, 0, ctx().stream>>>(dst, src, n);
    counted();
    KV_CUDA(cudaGetLastError());
}

}  // namespace kv
