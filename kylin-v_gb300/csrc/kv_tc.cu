// Mixed-precision grouped complex GEMM on the 5th-generation tensor cores.
//
// Same task format as the FP64 kernel (one CTA per 128 x 64 output tile,
// summing every block pair that accumulates into it).  Complex products use
// the 3M (Gauss) form
//     T1 = Ar Br,  T2 = Ai Bi,  T3 = (Ar + Ai)(Br + Bi)
//     Cr = T1 - T2,  Ci = T3 - T1 - T2
// with every real operand split into three TF32 parts x = hi + mid + lo
// (each the round-to-nearest TF32 of the remaining residual, ~33 bits in all)
// and each real product formed as the six terms of order <= 2^-22:
// hi*hi + hi*mid + mid*hi + hi*lo + mid*mid + lo*hi.
// The 18 MMAs per K-step run as tcgen05.mma.kind::tf32 (M=128, N=64, K=8)
// issued by one thread into three FP32 accumulators in tensor memory;
// operands are staged by all threads from the FP64 tensors into shared memory
// in the canonical K-major no-swizzle layout (8-row x 16-byte core matrices,
// K-adjacent core matrices 128 B apart, 8-row groups 1024 B apart).  The
// epilogue reads the accumulators with tcgen05.ld, forms Cr/Ci and writes
// FP64.  All mbarrier waits are bounded; on timeout the CTA records an error,
// drains (bounded) and frees its tensor memory.
#include <cstdint>

#include "kv_internal.h"

namespace kv {

namespace {

constexpr int BM = 128, BN = 64, BK = 32;
constexpr int A_PLANE = BM * BK * 4;  // bytes per TF32 plane of A
constexpr int B_PLANE = BN * BK * 4;
constexpr int NSPLIT = 3;           // TF32 parts per real operand
constexpr int NPLANE = 3 * NSPLIT;  // (re, im, re+im) x parts
constexpr int SMEM_BYTES = NPLANE * A_PLANE + NPLANE * B_PLANE + 1024 + 64;
constexpr uint32_t TMEM_COLS = 256;  // 3 accumulators x 64 columns, rounded to a power of two
constexpr long long WAIT_LIMIT = 1ll << 22;

// plane order: (re, im, re+im) x (hi, mid, lo): plane = 3 * component + part
__device__ __forceinline__ uint32_t kmaj_off(int r, int k) {
    return (uint32_t)(((r >> 3) * (BK / 4) + (k >> 2)) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ void split3(double x, float &hi, float &mid, float &lo) {
    hi = tf32_rna((float)x);
    const double r = x - (double)hi;
    mid = tf32_rna((float)r);
    lo = tf32_rna((float)(r - (double)mid));
}

// UMMA shared-memory descriptor: start >> 4 (bits 0-13), leading byte offset
// >> 4 (16-29), stride byte offset >> 4 (32-45), descriptor version 1 (46-47),
// base offset 0, layout type 0 = no swizzle (61-63).
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// instruction descriptor, kind::tf32: D = F32 (bits 4-5 = 1), A = B = TF32
// (bits 7-9, 10-12 = 2), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(IDESC), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (long long i = 0; i < WAIT_LIMIT; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__global__ void __launch_bounds__(128, 1) k_gemm_tc(const GemmTile *__restrict__ tiles, const GemmSeg *__restrict__ segs,
                                                    const double2 *__restrict__ A, const double2 *__restrict__ B,
                                                    double2 *__restrict__ C, double alpha, const int *skip,
                                                    int *err) {
    if (skip && *skip) return;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    float *Ap = (float *)smem;
    float *Bp = (float *)(smem + NPLANE * A_PLANE);
    uint64_t *mbar = (uint64_t *)(smem + NPLANE * A_PLANE + NPLANE * B_PLANE);
    uint32_t *tslot = (uint32_t *)(mbar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const GemmTile t = tiles[blockIdx.x];

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;
    const uint32_t mb = smem_u32(mbar);

    uint32_t parity = 0;
    bool pending = false, first = true, ok = true;
    for (int s = t.seg_begin; s < t.seg_end && ok; ++s) {
        const GemmSeg g = segs[s];
        const double2 *a = A + g.a_off;
        const double2 *b = B + g.b_off;
        for (int k0 = 0; k0 < g.K && ok; k0 += BK) {
            if (pending) {  // the previous MMAs still read shared memory
                if (!__syncthreads_and(mbar_wait(mb, parity))) { ok = false; break; }
                parity ^= 1u;
                pending = false;
            }
            for (int idx = tid; idx < BM * BK; idx += 128) {
                int m, k;
                if (g.opa == 0) { m = idx / BK; k = idx % BK; }
                else { m = idx % BM; k = idx / BM; }
                const int gm = t.m0 + m, gk = k0 + k;
                double re = 0.0, im = 0.0;
                if (gm < t.M && gk < g.K) {
                    double2 v = (g.opa == 0) ? a[(int64_t)gm * g.lda + gk] : a[(int64_t)gk * g.lda + gm];
                    re = v.x;
                    im = (g.opa == 0) ? v.y : -v.y;
                }
                const uint32_t o = kmaj_off(m, k) >> 2;
                float h, md, l;
                split3(re, h, md, l);
                Ap[0 * (A_PLANE / 4) + o] = h;
                Ap[1 * (A_PLANE / 4) + o] = md;
                Ap[2 * (A_PLANE / 4) + o] = l;
                split3(im, h, md, l);
                Ap[3 * (A_PLANE / 4) + o] = h;
                Ap[4 * (A_PLANE / 4) + o] = md;
                Ap[5 * (A_PLANE / 4) + o] = l;
                split3(re + im, h, md, l);
                Ap[6 * (A_PLANE / 4) + o] = h;
                Ap[7 * (A_PLANE / 4) + o] = md;
                Ap[8 * (A_PLANE / 4) + o] = l;
            }
            for (int idx = tid; idx < BN * BK; idx += 128) {
                int n, k;
                if (g.opb == 0) { n = idx % BN; k = idx / BN; }
                else { k = idx % BK; n = idx / BK; }
                const int gn = t.n0 + n, gk = k0 + k;
                double re = 0.0, im = 0.0;
                if (gn < t.N && gk < g.K) {
                    double2 v = (g.opb == 0) ? b[(int64_t)gk * g.ldb + gn] : b[(int64_t)gn * g.ldb + gk];
                    re = v.x;
                    im = v.y;
                }
                const uint32_t o = kmaj_off(n, k) >> 2;
                float h, md, l;
                split3(re, h, md, l);
                Bp[0 * (B_PLANE / 4) + o] = h;
                Bp[1 * (B_PLANE / 4) + o] = md;
                Bp[2 * (B_PLANE / 4) + o] = l;
                split3(im, h, md, l);
                Bp[3 * (B_PLANE / 4) + o] = h;
                Bp[4 * (B_PLANE / 4) + o] = md;
                Bp[5 * (B_PLANE / 4) + o] = l;
                split3(re + im, h, md, l);
                Bp[6 * (B_PLANE / 4) + o] = h;
                Bp[7 * (B_PLANE / 4) + o] = md;
                Bp[8 * (B_PLANE / 4) + o] = l;
            }
            // make the generic-proxy smem writes visible to the tensor core
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
            if (tid == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t a0 = smem_u32(Ap), b0 = smem_u32(Bp);
#pragma unroll
                for (int kk = 0; kk < BK / 8; ++kk) {
#pragma unroll
                    for (int p = 0; p < 3; ++p) {  // T1 = Ar Br, T2 = Ai Bi, T3 = As Bs
                        const uint32_t d = tmem + (uint32_t)(p * BN);
                        // (a part, b part) pairs with part-order sum <= 2, smallest terms first
                        const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
                        for (int t = 0; t < 6; ++t) {
                            const uint32_t aa = a0 + (3 * p + pa[t]) * A_PLANE + kk * 256;
                            const uint32_t bb = b0 + (3 * p + pb[t]) * B_PLANE + kk * 256;
                            const uint32_t acc = (first && kk == 0 && t == 0) ? 0u : 1u;
                            mma_tf32(d, make_desc(aa, 128, 1024), make_desc(bb, 128, 1024), acc);
                        }
                    }
                }
                mma_commit(mb);
            }
            first = false;
            pending = true;
        }
    }
    if (pending && ok) {
        if (__syncthreads_and(mbar_wait(mb, parity))) pending = false;
        else ok = false;
    }
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
        // drain what may still be in flight (bounded) before releasing tensor memory
        if (pending) mbar_wait(mb, parity);
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int m = warp * 32 + lane;
    const int gm = t.m0 + m;
    if (ok) {
        for (int c0 = 0; c0 < BN; c0 += 32) {
            float t1[32], t2[32], t3[32];
            if (!first) {  // at least one MMA ran: read the accumulators (all warps, aligned)
                const uint32_t row = (uint32_t)(warp * 32) << 16;
                tmem_ld32(tmem + row + 0 * BN + c0, t1);
                tmem_ld32(tmem + row + 1 * BN + c0, t2);
                tmem_ld32(tmem + row + 2 * BN + c0, t3);
            } else {
#pragma unroll
                for (int j = 0; j < 32; ++j) t1[j] = t2[j] = t3[j] = 0.f;
            }
            if (gm < t.M) {
                double2 *crow = C + t.c_off + (int64_t)gm * t.ldc;
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const int gn = t.n0 + c0 + j;
                    if (gn < t.N) {
                        const double cr = (double)t1[j] - (double)t2[j];
                        const double ci = (double)t3[j] - (double)t1[j] - (double)t2[j];
                        crow[gn] = make_double2(alpha * cr, alpha * ci);
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS)
                     : "memory");
}

int *g_err = nullptr;
bool g_attr = false;

}  // namespace

void launch_gemm_mixed(const GemmPlan &p, const double2 *A, const double2 *B, double2 *C, double alpha,
                       const int *skip) {
    if (p.tiles.empty()) return;
    if (!g_attr) {
        KV_CUDA(cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
        KV_CUDA(cudaMalloc(&g_err, sizeof(int)));
        KV_CUDA(cudaMemset(g_err, 0, sizeof(int)));
        g_attr = true;
    }
    k_gemm_tc<<<(unsigned)p.tiles.size(), 128, SMEM_BYTES, ctx().stream>>>(
        p.d_tiles.as<GemmTile>(), p.d_segs.as<GemmSeg>(), A, B, C, alpha, skip, g_err);
    counted();
    KV_CUDA(cudaGetLastError());
}

// 0 if no tensor-core wait has timed out since the last call (then cleared)
int mixed_gemm_status() {
    if (!g_err) return KV_OK;
    int h = 0;
    KV_CUDA(cudaMemcpy(&h, g_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) KV_CUDA(cudaMemset(g_err, 0, sizeof(int)));
    return h ? KV_ETIMEOUT : KV_OK;
}

}  // namespace kv
