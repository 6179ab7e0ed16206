// Mixed-precision grouped complex GEMM on the 5th-generation tensor cores
// with exact accumulation.
//
// GB300 runs FP64 arithmetic at a small fraction of its FP32 and tensor
// rates, so no FP64 instruction is issued per element of a tile.  Instead:
//
//  1. Slicing (slice_item; one launch per call for both operands).  Every GEMM row of an A
//     block (and every GEMM column of a B block) gets a binary exponent e
//     with max_k |x| < 2^e over that row; each real value becomes the
//     fixed-point integer X = round(x 2^(37-e)), |X| <= 2^37, written as five
//     balanced base-256 digits X = d0 2^32 + d1 2^24 + d2 2^16 + d3 2^8 + d4
//     (|d0| <= 33, |d1..d4| <= 128) in FP16 (exact).  For the 3M complex form
//     three values are sliced per element: re, im and re + im (the last as
//     the exact integer sum X_re + X_im).  Integer arithmetic only.  Where
//     the contracted index runs over parts of very different magnitude (MPO
//     channels, Schmidt values), it is first balanced by exact powers of two
//     (kmax_item, GemmPlan::balance_k; on the main stream the maxima and the
//     slicing are one cooperative launch, k_slice_coop, with grid barriers
//     between zeroing, maxima and slicing).  The digits are written directly in the
//     tensor cores' shared-memory panel layout (K-major, no swizzle: 8-row x
//     16-byte core matrices, K-adjacent core matrices 128 B apart, 8-row
//     groups 256 B apart), one 16-deep K panel after another, all 15 digit
//     planes of a panel contiguous, so a pipeline stage is one bulk copy per
//     operand.
//  2. Products (k_gemm_tc).  T1 = Ar Br, T2 = Ai Bi, T3 = As Bs are formed as
//     digit-pair products of orders o = i + j <= 4 (15 per real product, 45
//     tcgen05.mma.kind::f16 of M=128, N=32, K=16 per K panel) into 15 FP32
//     accumulators in tensor memory.  Every digit product is an integer of
//     at most 2^14 in magnitude, an order sums at most 2^16 of them per K
//     step, and at most 240 K-steps are accumulated between drains, so every
//     accumulator is an integer below 2^24 and the FP32 accumulation is
//     exact.
//  3. Drains (epilogue warps).  At the end of each segment (one block pair)
//     or every 240 K, the accumulators are read with tcgen05.ld, converted to
//     int64 (sum_o P_o 2^(8(4-o)) = X Y / 2^32), combined into Cr = T1 - T2
//     and Ci = T3 - T1 - T2, aligned to the tile's largest row/column
//     exponents and added to int64 running sums; the final sums are converted
//     to FP64 by integer operations (exponent and mantissa assembled
//     directly).
//
// Result: each output element is exact up to the rounding of X (2^-38 of
// the row/column maximum) and the dropped digit orders 5 to 8 (below
// 2^-33 of the same scale), i.e. ~1e-10 relative to max|A_row| max|B_col| K
// (the 30-bit form this replaced left ~1e-8 per product, too much for 20
// time steps of a 160-site chain), with no FP64 arithmetic in the GEMM.
//
// Pipeline: warp 0 (one thread) issues the bulk copies of 3 stages
// (cp.async.bulk completing on mbarriers), warp 1 allocates tensor memory and
// one thread issues the MMAs (tcgen05.commit frees a stage and signals a
// drain), warps 2-17 drain (four per 32-lane quarter of tensor memory, each
// taking a quarter of the tile's columns: the drain is a long chain of
// dependent integer operations per column, so it is spread thin and four
// warps per scheduler hide its latency).
// Every mbarrier wait is bounded; on timeout the CTA records an error, waits
// (bounded) for its copies and MMAs in flight, frees tensor memory and exits.
#include <mutex>
#include <cooperative_groups.h>
#include <cuda_fp16.h>

#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <utility>

#include "kv_internal.h"

namespace kv {

namespace {

constexpr int BM = kMixedTileM, BN = kMixedTileN, BKC = 16;
constexpr int NDIG = 5, NORD = 5, NCOMP = 3;
constexpr int NPL = NCOMP * NDIG;              // digit planes per operand
constexpr int A_PANEL = NPL * BM * BKC;        // FP16 elements per A panel (all planes)
constexpr int B_PANEL = NPL * BN * BKC;
constexpr int A_BYTES = A_PANEL * 2, B_BYTES = B_PANEL * 2;
constexpr int PLANE_A = BM * BKC * 2, PLANE_B = BN * BKC * 2;  // bytes per plane within a panel
constexpr int STAGES = 3;
constexpr int NACC = NCOMP * NORD;             // accumulators of BN columns
constexpr uint32_t TMEM_COLS = 512;            // NACC * BN = 480, rounded to a power of two
constexpr int KDRAIN = 240;                    // K-steps accumulated exactly between drains
constexpr int GKC = KDRAIN / BKC;              // K panels per drain group
constexpr int FRAC = 37;                       // fixed point: X = round(x 2^(FRAC - e)), |X| <= 2^37
// a drained combination sum_o P_o 2^(8(NORD-1-o)) is X Y / 2^COMB_SHIFT
constexpr int COMB_SHIFT = 8 * (2 * (NDIG - 1) - (NORD - 1));
constexpr int kZeroExp = -4000;                // exponent of an all-zero row
constexpr int kErrTimeout = 1, kErrNonFinite = 2;  // bits of the per-device error word
constexpr int kMaxFiniteExp = 1024;            // row / column exponents of finite operands are <= 1024
constexpr long long WAIT_LIMIT = 1ll << 22;   // try_wait polls before a wait gives up
constexpr int EPI_WARPS = 16;                  // four per tensor-memory lane quarter, 8 columns each
constexpr int EPI_COLS = BN / (EPI_WARPS / 4);
constexpr int NTHREADS = 32 * (2 + EPI_WARPS);
constexpr int SMEM_ALIGN = 128;                // stage base alignment (no-swizzle layout, bulk copies)
constexpr int SMEM_BYTES = STAGES * (A_BYTES + B_BYTES) + SMEM_ALIGN + 1024;
static_assert(SMEM_BYTES <= 227 * 1024, "pipeline stages exceed the shared memory of one CTA");

static_assert(NACC * BN <= (int)TMEM_COLS, "accumulators exceed tensor memory");
static_assert(EPI_COLS % 4 == 0, "the drain loads 4 columns per accumulator at once");
static_assert(A_BYTES + B_BYTES < (1 << 20), "transaction count per stage");

// ----------------------------------------------------------- slicing
// round(x 2^(FRAC-e)) for |x| < 2^e, from the bits of x (integer operations only)
__device__ __forceinline__ long long fixq(double x, int e) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const int E = (int)((u >> 52) & 0x7FF);
    // X = m >> s with m the 53-bit significand; s >= 53 - FRAC when |x| < 2^e
    const int s = 1075 - FRAC + e - E;
    if (E == 0 || s >= 64) return 0;
    long long X;
    if (s < 53 - FRAC) X = 1ll << FRAC;  // only for non-finite input (the exponent came from an inf/NaN row)
    else X = (long long)((((u & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull) + (1ull << (s - 1))) >> s);
    return (u >> 63) ? -X : X;
}

__device__ __forceinline__ void digits(long long X, int d[NDIG]) {
#pragma unroll
    for (int i = NDIG - 1; i > 0; --i) {
        d[i] = (int)(((X + 128) & 255) - 128);
        X = (X - d[i]) >> 8;  // exact
    }
    d[0] = (int)X;
}

// element offset of (row r, k) inside one plane of a TR x 16 panel
template <int TR>
__device__ __forceinline__ int panel_off(int r, int k) {
    return (r >> 3) * 128 + (k >> 3) * 64 + (r & 7) * 8 + (k & 7);
}

// two digits (|d| <= 512) as FP16: 1536 + d in the binade [1024, 2048) has
// unit spacing, so its bits are 0x6600 + d; subtracting 1536 is exact
__device__ __forceinline__ __half2 digits2(int d0, int d1) {
    const uint32_t u = (uint32_t)(0x6600 + d0) | ((uint32_t)(0x6600 + d1) << 16);
    __half2 h;
    memcpy(&h, &u, sizeof(h));
    return __hsub2(h, __float2half2_rn(1536.f));
}

// One CTA per (job, 8 consecutive rows); one warp per row: pass 1 finds the
// row exponent, pass 2 writes the digits of two adjacent K positions per lane.
// Balancing of the contracted index k: kmax[k] holds the largest |re|, |im|
// of A's column k over the A views of a segment component, kmax[kscales + k]
// that of B's row k.  A's column is scaled by 2^s, B's row by 2^-s, with
// s = floor((E_B - E_A) / 2) from their binary exponents, so both reach about
// sqrt(max_A max_B) and every digit product is resolved at the same scale.
__device__ __forceinline__ int balance_shift(const unsigned long long *kmax, int64_t kscales, int64_t k, int b_side) {
    const int ea = (int)(kmax[k] >> 52), eb = (int)(kmax[kscales + k] >> 52);
    if (ea == 0 || eb == 0) return 0;
    const int sh = (eb - ea) >> 1;
    return b_side ? -sh : sh;
}

// x * 2^sh by the exponent field alone (no FP64 arithmetic): exact for
// normal results; results below the normal range become +-0 and results
// beyond it +-inf (as the product would round; a subnormal input stays as it
// is, and fixq reads subnormals as 0 either way)
__device__ __forceinline__ double scale_exp(double x, int sh) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const int E = (int)((u >> 52) & 0x7FF);
    if (sh == 0 || E == 0 || E == 0x7FF) return x;
    const int En = E + sh;
    const unsigned long long sign = u & 0x8000000000000000ull;
    if (En <= 0) return __longlong_as_double((long long)sign);
    if (En >= 0x7FF) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull));
    return __longlong_as_double((long long)((u & ~(0x7FFull << 52)) | ((unsigned long long)En << 52)));
}

// Per-k maxima for balancing: one CTA per (view, 8 rows), one warp per row;
// the 8 rows' values are reduced in shared memory, then one atomicMax per k
// (non-negative doubles order like their bit patterns).
// item bid of the A items followed by the B items (CTA-uniform)
__device__ __forceinline__ void kmax_item(const SliceJob *__restrict__ ajobs, const int2 *__restrict__ aitems, int na,
                                          const SliceJob *__restrict__ bjobs, const int2 *__restrict__ bitems,
                                          const double2 *__restrict__ A, const double2 *__restrict__ B,
                                          unsigned long long *kmax, int64_t kscales, int step, int bid) {
    __shared__ unsigned long long red[8][33];
    const bool is_b = bid >= na;
    const int2 it = is_b ? bitems[bid - na] : aitems[bid];
    const SliceJob j = is_b ? bjobs[it.x] : ajobs[it.x];
    if (j.entry > step || j.ks_off < 0) return;  // uniform over the CTA
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = it.y + warp;
    const double2 *s = (is_b ? B : A) + j.src_off;
    unsigned long long *dst = kmax + (is_b ? kscales : 0) + j.ks_off;
    for (int k0 = 0; k0 < j.K; k0 += 32) {
        const int k = k0 + lane;
        unsigned long long m = 0;
        if (r < j.rows && k < j.K) {
            const double2 v = s[j.trans ? (int64_t)k * j.ld + r : (int64_t)r * j.ld + k];
            const unsigned long long br = (unsigned long long)__double_as_longlong(v.x) & 0x7FFFFFFFFFFFFFFFull;
            const unsigned long long bi = (unsigned long long)__double_as_longlong(v.y) & 0x7FFFFFFFFFFFFFFFull;
            m = max(br, bi);
        }
        red[warp][lane] = m;
        __syncthreads();
        if (warp == 0) {
            unsigned long long x = 0;
#pragma unroll
            for (int w = 0; w < 8; ++w) x = max(x, red[w][lane]);
            if (x && k < j.K) atomicMax(dst + k, x);
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_kmax(const SliceJob *__restrict__ ajobs, const int2 *__restrict__ aitems,
                                              int na, const SliceJob *__restrict__ bjobs,
                                              const int2 *__restrict__ bitems, const double2 *__restrict__ A,
                                              const double2 *__restrict__ B, unsigned long long *kmax,
                                              int64_t kscales, const int *skip, int step) {
    if (skip && *skip) return;
    kmax_item(ajobs, aitems, na, bjobs, bitems, A, B, kmax, kscales, step, (int)blockIdx.x);
}

// One slicing item (a job's 8 rows from it.y, one per warp).  A row holding
// an Inf or NaN sets bit kErrNonFinite of *err: fixed point has no code for
// it, and the digits written for that row are meaningless.  Warps return on
// their own; there is no barrier here.
template <int TR>
__device__ __forceinline__ void slice_item(const SliceJob *__restrict__ jobs, int2 it, const double2 *__restrict__ src,
                                           __half *__restrict__ dst, int *__restrict__ exps, double alpha, int step,
                                           int *err, const unsigned long long *kmax, int64_t kscales, int b_side) {
    const SliceJob j = jobs[it.x];
    if (j.entry > step) return;  // no active segment reads this block
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = it.y + warp;
    // rows past the block (up to the panel's TR) are not written: they only
    // reach output rows / columns the GEMM epilogue never stores
    if (r >= j.rows) return;
    const int kpad = j.nkc * BKC;
    const double2 *s = src + j.src_off;
    const bool scale = alpha != 1.0;
    const bool bal = kmax != nullptr && j.ks_off >= 0;
    auto load = [&](int k) {
        double2 v = s[j.trans ? (int64_t)k * j.ld + r : (int64_t)r * j.ld + k];
        if (scale) { v.x *= alpha; v.y *= alpha; }
        if (j.conj) v.y = -v.y;
        if (bal) {  // exact power-of-two balancing of the contracted index
            const int sh = balance_shift(kmax, kscales, j.ks_off + k, b_side);
            v.x = scale_exp(v.x, sh);
            v.y = scale_exp(v.y, sh);
        }
        return v;
    };
    unsigned long long mx = 0;
    for (int k = lane; k < j.K; k += 32) {
        const double2 v = load(k);
        const unsigned long long br = (unsigned long long)__double_as_longlong(v.x) & 0x7FFFFFFFFFFFFFFFull;
        const unsigned long long bi = (unsigned long long)__double_as_longlong(v.y) & 0x7FFFFFFFFFFFFFFFull;
        mx = max(mx, max(br, bi));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) mx = max(mx, (unsigned long long)__shfl_xor_sync(0xFFFFFFFFu, mx, o));
    const int e = mx ? (int)(mx >> 52) - 1022 : kZeroExp;
    if (lane == 0) {
        exps[j.exp_off + r] = e;
        if (mx >= 0x7FF0000000000000ull) atomicOr(err, kErrNonFinite);
    }
    __half *pan = dst + j.dst_off + (int64_t)(r / TR) * j.nkc * (NPL * TR * BKC);
    const int rr = r % TR;
    for (int k = 2 * lane; k < kpad; k += 64) {  // k even: k and k + 1 are adjacent in the panel
        long long x[2][NCOMP];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            long long xr = 0, xi = 0;
            if (k + h < j.K) {
                const double2 v = load(k + h);
                xr = fixq(v.x, e);
                xi = fixq(v.y, e);
            }
            x[h][0] = xr;
            x[h][1] = xi;
            x[h][2] = xr + xi;
        }
        __half *p = pan + (int64_t)(k / BKC) * (NPL * TR * BKC) + panel_off<TR>(rr, k & (BKC - 1));
#pragma unroll
        for (int c = 0; c < NCOMP; ++c) {
            int d0[NDIG], d1[NDIG];
            digits(x[0][c], d0);
            digits(x[1][c], d1);
#pragma unroll
            for (int i = 0; i < NDIG; ++i)
                *reinterpret_cast<__half2 *>(p + (c * NDIG + i) * (TR * BKC)) = digits2(d0[i], d1[i]);
        }
    }
}

// Both operands' slicing in one launch: CTAs [0, na) take the A items, the
// rest the B items.
__global__ void __launch_bounds__(256) k_slice_ab(const SliceJob *__restrict__ ajobs, const int2 *__restrict__ aitems,
                                                  int na, const SliceJob *__restrict__ bjobs,
                                                  const int2 *__restrict__ bitems, const double2 *__restrict__ A,
                                                  const double2 *__restrict__ B, __half *__restrict__ ap,
                                                  __half *__restrict__ bp, int *__restrict__ ae,
                                                  int *__restrict__ be, double alpha, const int *skip, int step,
                                                  int *err, const unsigned long long *kmax, int64_t kscales) {
    if (skip && *skip) return;
    const int bid = (int)blockIdx.x;
    if (bid < na) slice_item<BM>(ajobs, aitems[bid], A, ap, ae, 1.0, step, err, kmax, kscales, 0);
    else slice_item<BN>(bjobs, bitems[bid - na], B, bp, be, alpha, step, err, kmax, kscales, 1);
}

// The balanced slicing as one cooperative launch: zero the per-index maxima,
// grid barrier, the maxima of every contracted index (k_kmax's work), grid
// barrier, both operands' slicing (k_slice_ab's work); each CTA walks the
// items with a stride of the grid.  kmax == nullptr: no balancing, no barrier.
__global__ void __launch_bounds__(256) k_slice_coop(const SliceJob *__restrict__ ajobs,
                                                    const int2 *__restrict__ aitems, int na,
                                                    const SliceJob *__restrict__ bjobs,
                                                    const int2 *__restrict__ bitems, int nb,
                                                    const double2 *__restrict__ A, const double2 *__restrict__ B,
                                                    __half *__restrict__ ap, __half *__restrict__ bp,
                                                    int *__restrict__ ae, int *__restrict__ be, double alpha,
                                                    const int *skip, int step, int *err, unsigned long long *kmax,
                                                    int64_t kscales) {
    namespace cg = cooperative_groups;
    if (skip && *skip) return;  // uniform over the grid: nothing in this launch writes it
    const int nitems = na + nb;
    if (kmax) {
        cg::grid_group grid = cg::this_grid();
        for (int64_t e = blockIdx.x * 256ll + threadIdx.x; e < 2 * kscales; e += (int64_t)gridDim.x * 256)
            kmax[e] = 0;
        grid.sync();
        for (int bid = blockIdx.x; bid < nitems; bid += gridDim.x)
            kmax_item(ajobs, aitems, na, bjobs, bitems, A, B, kmax, kscales, step, bid);
        grid.sync();
    }
    for (int bid = blockIdx.x; bid < nitems; bid += gridDim.x) {
        if (bid < na) slice_item<BM>(ajobs, aitems[bid], A, ap, ae, 1.0, step, err, kmax, kscales, 0);
        else slice_item<BN>(bjobs, bitems[bid - na], B, bp, be, alpha, step, err, kmax, kscales, 1);
    }
}

// -------------------------------------------------------- tensor-core GEMM
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

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

// instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = F16
// (bits 7-9, 10-12 = 0), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
constexpr uint32_t IDESC = (1u << 4) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

// D (+)= A B with the accumulate flag fixed at compile time (no per-MMA predicate set-up)
template <bool ACC>
__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc) {
    if constexpr (ACC)
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.eq.u32 p, 1, 1;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
            "l"(adesc), "l"(bdesc), "n"(IDESC));
    else
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, 1, 1;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
            "l"(adesc), "l"(bdesc), "n"(IDESC));
}

// The 45 MMAs of one K panel.  Shared-memory descriptors are the stage's
// plane-0 descriptors plus compile-time plane offsets (a plane offset is a
// multiple of 16 bytes, and no address leaves the 14-bit field, so adding
// offset / 16 to the descriptor is adding it to the address).  FIRST: the
// panel opens a drain group, so each order's first digit pair overwrites its
// accumulator.
template <bool FIRST>
__device__ __forceinline__ void mma_panel(uint32_t tmem, uint64_t da, uint64_t db) {
#pragma unroll
    for (int c = 0; c < NCOMP; ++c)
#pragma unroll
        for (int o = 0; o < NORD; ++o) {
            const uint32_t d = tmem + (uint32_t)((c * NORD + o) * BN);
#pragma unroll
            for (int i = (o > NDIG - 1 ? o - (NDIG - 1) : 0); i <= (o < NDIG - 1 ? o : NDIG - 1); ++i) {
                const int jj = o - i;
                const uint64_t ad = da + (uint64_t)(((c * NDIG + i) * PLANE_A) >> 4);
                const uint64_t bd = db + (uint64_t)(((c * NDIG + jj) * PLANE_B) >> 4);
                if (FIRST && i == (o > NDIG - 1 ? o - (NDIG - 1) : 0)) mma_f16<false>(d, ad, bd);
                else mma_f16<true>(d, ad, bd);
            }
        }
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, long long limit = WAIT_LIMIT) {
    for (long long i = 0; i < limit; ++i) {
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

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(mbar)
        : "memory");
}

__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float *v) {
    uint32_t r0, r1, r2, r3;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(taddr));
    v[0] = __uint_as_float(r0);
    v[1] = __uint_as_float(r1);
    v[2] = __uint_as_float(r2);
    v[3] = __uint_as_float(r3);
}

__device__ __forceinline__ void epi_bar() { asm volatile("bar.sync 1, %0;" ::"n"(32 * EPI_WARPS) : "memory"); }

// v / 2^sh rounded to nearest, sh >= 0
__device__ __forceinline__ long long sra_round(long long v, int sh) {
    if (sh <= 0) return v;
    if (sh >= 62) return 0;
    return (v + (1ll << (sh - 1))) >> sh;
}

// v 2^sc as FP64, rounded to nearest even, from integer operations
__device__ __forceinline__ double i64_ldexp(long long v, int sc) {
    if (v == 0) return 0.0;
    const unsigned long long neg = v < 0 ? 1ull : 0ull;
    unsigned long long a = neg ? (unsigned long long)(-v) : (unsigned long long)v;
    const int lz = __clzll((long long)a);
    a <<= lz;  // leading one at bit 63
    int ex = 63 - lz + sc;
    unsigned long long mant = a >> 11;
    const unsigned long long rem = a & 0x7FFull;
    if (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) {
        ++mant;
        if (mant >> 53) { mant >>= 1; ++ex; }
    }
    const int E = ex + 1023;
    if (E <= 0) return 0.0;
    if (E >= 2047) return __longlong_as_double((long long)((neg << 63) | 0x7FF0000000000000ull));
    return __longlong_as_double((long long)((neg << 63) | ((unsigned long long)E << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

// sum_o P_o 2^(8(4-o)) from the five order accumulators (exact integers < 2^24)
__device__ __forceinline__ long long combine(const float *p) {
    long long u = __float2int_rn(p[0]);
    u = (u << 8) + __float2int_rn(p[1]);
    u = (u << 8) + __float2int_rn(p[2]);
    u = (u << 8) + __float2int_rn(p[3]);
    return (u << 8) + __float2int_rn(p[4]);
}

// Persistent: CTA b takes tiles b, b + gridDim.x, ...; each role walks the
// same tile sequence and keeps its mbarrier phase counters across tiles, so
// the producer streams the next tile's panels while the current tile drains.
__device__ __forceinline__ bool tile_active(const GemmTile &t, const SegX *segs, int step) {
    for (int s = t.seg_begin; s < t.seg_end; ++s)
        if (segs[s].entry <= step) return true;
    return false;
}

__global__ void __launch_bounds__(NTHREADS, 1) k_gemm_tc(const GemmTile *__restrict__ tiles, int ntiles,
                                                    const SegX *__restrict__ segs,
                                                    const __half *__restrict__ Apl, const __half *__restrict__ Bpl,
                                                    const int *__restrict__ Aexp, const int *__restrict__ Bexp,
                                                    double2 *__restrict__ C, const int *skip, int *err, int step,
                                                    int write_inactive, long long wait_limit, int no_copies) {
    if (skip && *skip) return;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + SMEM_ALIGN - 1) & ~(uintptr_t)(SMEM_ALIGN - 1));
    uint8_t *sA = smem;
    uint8_t *sB = smem + STAGES * A_BYTES;
    uint64_t *bars = (uint64_t *)(smem + STAGES * (A_BYTES + B_BYTES));
    uint64_t *full = bars, *empty = bars + STAGES, *accf = bars + 2 * STAGES, *acce = accf + 1, *mdone = acce + 1;
    uint32_t *tslot = (uint32_t *)(mdone + 1);
    int *s_ecol = (int *)(tslot + 4);  // [BN] largest column exponent over the tile's segments
    int *s_fcol = s_ecol + BN;         // [EPI_WARPS][EPI_COLS] each epilogue warp's copy of a segment's
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(smem_u32(full + s), 1);
            mbar_init(smem_u32(empty + s), 1);
        }
        mbar_init(smem_u32(accf), 1);
        mbar_init(smem_u32(acce), 32 * EPI_WARPS);
        mbar_init(smem_u32(mdone), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;

    if (warp == 0) {
        // ------------------------------------------------ producer
        if (lane == 0) {
            int it = 0;
            int uses[STAGES] = {0, 0, 0};
            bool ok = true;
            for (int ti = blockIdx.x; ti < ntiles && ok; ti += gridDim.x) {
                const GemmTile t = tiles[ti];
                const int rt = t.m0 / BM, nt = t.n0 / BN;
                for (int s = t.seg_begin; s < t.seg_end && ok; ++s) {
                    const SegX g = segs[s];
                    if (g.entry > step) continue;
                    const __half *ap = Apl + g.a_pan + (int64_t)rt * g.nkc * A_PANEL;
                    const __half *bp = Bpl + g.b_pan + (int64_t)nt * g.nkc * B_PANEL;
                    for (int kc = 0; kc < g.nkc && !no_copies; ++kc, ++it) {
                        const int st = it % STAGES;
                        const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
                        if (!mbar_wait(smem_u32(empty + st), ph ^ 1u, wait_limit)) { ok = false; break; }
                        mbar_expect_tx(smem_u32(full + st), (uint32_t)(A_BYTES + B_BYTES));
                        bulk_g2s(smem_u32(sA + st * A_BYTES), ap + (int64_t)kc * A_PANEL, A_BYTES,
                                 smem_u32(full + st));
                        bulk_g2s(smem_u32(sB + st * B_BYTES), bp + (int64_t)kc * B_PANEL, B_BYTES,
                                 smem_u32(full + st));
                        ++uses[st];
                    }
                }
            }
            if (!ok) atomicOr(err, kErrTimeout);
            // no copy may land after the CTA exits: wait (bounded) for the last one into each stage
            for (int st = 0; st < STAGES; ++st)
                if (uses[st]) mbar_wait(smem_u32(full + st), (uint32_t)(uses[st] - 1) & 1u, wait_limit);
        }
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issue
        if (lane == 0) {
            // plane-0 descriptors of stage 0; stage st adds st * bytes / 16 to the address field
            const uint64_t desc_a0 = make_desc(smem_u32(sA), 128, 256), desc_b0 = make_desc(smem_u32(sB), 128, 256);
            int it = 0, grp = 0;
            bool ok = true;
            for (int ti = blockIdx.x; ti < ntiles && ok; ti += gridDim.x) {
                const GemmTile t = tiles[ti];
                for (int s = t.seg_begin; s < t.seg_end && ok; ++s) {
                    if (segs[s].entry > step) continue;
                    const int nkc = segs[s].nkc;
                    for (int kc0 = 0; kc0 < nkc && ok; kc0 += GKC, ++grp) {
                        // the epilogue has read the previous group's accumulators
                        if (!mbar_wait(smem_u32(acce), ((uint32_t)grp & 1u) ^ 1u, wait_limit)) { ok = false; break; }
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        const int kc1 = min(nkc, kc0 + GKC);
                        for (int kc = kc0; kc < kc1; ++kc, ++it) {
                            const int st = it % STAGES;
                            const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
                            if (!mbar_wait(smem_u32(full + st), ph, wait_limit)) { ok = false; break; }
                            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                            const uint64_t da = desc_a0 + (uint64_t)(st * (A_BYTES >> 4));
                            const uint64_t db = desc_b0 + (uint64_t)(st * (B_BYTES >> 4));
                            if (kc == kc0) mma_panel<true>(tmem, da, db);
                            else mma_panel<false>(tmem, da, db);
                            mma_commit(smem_u32(empty + st));  // stage free once these MMAs are done
                        }
                        if (!ok) break;
                        mma_commit(smem_u32(accf));  // accumulators ready for the drain
                    }
                }
            }
            if (!ok) atomicOr(err, kErrTimeout);
            // every MMA issued by this thread has completed before tensor memory is freed
            mma_commit(smem_u32(mdone));
            mbar_wait(smem_u32(mdone), 0u, wait_limit);
        }
    } else {
        // ------------------------------------------------ drains and epilogue
        // warp w reads lane quarter w % 4 (the rows it may access in tensor
        // memory) and columns [c_lo, c_lo + EPI_COLS)
        const int q = warp & 3;
        const int c_lo = ((warp - 2) / 4) * EPI_COLS;
        const int m = q * 32 + lane;
        const uint32_t trow = tmem + ((uint32_t)(q * 32) << 16);
        int *fw = s_fcol + (warp - 2) * EPI_COLS;  // this warp's copy of the segment's column exponents
        bool ok = true;  // warp-uniform; after a timed-out wait the warp stops waiting but keeps the barriers
        int grp = 0;
        for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x) {
            const GemmTile t = tiles[ti];
            const bool act = tile_active(t, segs, step);
            if (!act && !write_inactive) continue;  // the same for every epilogue warp
            const int nseg = t.seg_end - t.seg_begin;
            int erow = kZeroExp;
            for (int s = t.seg_begin; s < t.seg_end; ++s)
                if (segs[s].entry <= step) erow = max(erow, Aexp[segs[s].a_exp + t.m0 + m]);
            if (warp == 2) {
                int ec = kZeroExp;
                for (int s = t.seg_begin; s < t.seg_end; ++s)
                    if (segs[s].entry <= step) ec = max(ec, Bexp[segs[s].b_exp + t.n0 + lane]);
                s_ecol[lane] = ec;
            }
            epi_bar();  // s_ecol written; reached by every epilogue warp for every tile
            long long cr[EPI_COLS], ci[EPI_COLS];
#pragma unroll
            for (int c = 0; c < EPI_COLS; ++c) cr[c] = ci[c] = 0;
            for (int sl = 0; sl < nseg; ++sl) {
                const SegX g = segs[t.seg_begin + sl];
                if (g.entry > step) continue;
                // column shifts of this segment, into the warp's own shared-memory slots
                if (lane < EPI_COLS) fw[lane] = s_ecol[c_lo + lane] - Bexp[g.b_exp + t.n0 + c_lo + lane];
                __syncwarp();
                const int shr = erow - Aexp[g.a_exp + t.m0 + m];
                for (int kc0 = 0; kc0 < g.nkc; kc0 += GKC, ++grp) {
                    // warp-uniform decision: tcgen05.ld below is a warp-wide instruction
                    if (ok && !__all_sync(0xFFFFFFFFu, mbar_wait(smem_u32(accf), (uint32_t)grp & 1u, wait_limit)))
                        ok = false;
                    if (!ok) continue;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
                    for (int c0 = 0; c0 < EPI_COLS; c0 += 4) {
                        long long I[NCOMP][4];
#pragma unroll
                        for (int c = 0; c < NCOMP; ++c) {
                            float a[NORD][4];
#pragma unroll
                            for (int o = 0; o < NORD; ++o)
                                tmem_ld4(trow + (uint32_t)((c * NORD + o) * BN + c_lo + c0), a[o]);
                            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                            for (int jx = 0; jx < 4; ++jx) {
                                float p[NORD];
#pragma unroll
                                for (int o = 0; o < NORD; ++o) p[o] = a[o][jx];
                                I[c][jx] = combine(p);
                            }
                        }
#pragma unroll
                        for (int jx = 0; jx < 4; ++jx) {
                            const int col = c0 + jx;
                            const int sh = shr + fw[col];
                            cr[col] += sra_round(I[0][jx] - I[1][jx], sh);
                            ci[col] += sra_round(I[2][jx] - I[0][jx] - I[1][jx], sh);
                        }
                    }
                    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                    mbar_arrive(smem_u32(acce));
                }
                __syncwarp();  // fw is rewritten for the next segment
            }
            const int gm = t.m0 + m;
            if (ok && gm < t.M) {
                double2 *crow = C + t.c_off + (int64_t)gm * t.ldc;
#pragma unroll
                for (int c = 0; c < EPI_COLS; ++c) {
                    const int gn = t.n0 + c_lo + c;
                    if (gn < t.N) {
                        const int ec = s_ecol[c_lo + c];
                        const int sc = erow + ec - 2 * FRAC + COMB_SHIFT;
                        // a row or column holding Inf or NaN (slicer exponent above the
                        // FP64 range) gives NaN, as the FP64 product would
                        crow[gn] = (erow > kMaxFiniteExp || ec > kMaxFiniteExp)
                                       ? make_double2(__longlong_as_double(0x7FF8000000000000ll),
                                                      __longlong_as_double(0x7FF8000000000000ll))
                                       : make_double2(i64_ldexp(cr[c], sc), i64_ldexp(ci[c], sc));
                    }
                }
            }
            epi_bar();  // every warp has used s_ecol before the next tile rewrites it
        }
        if (!ok && lane == 0) atomicOr(err, kErrTimeout);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS)
                     : "memory");
    }
}

// Per device: the kernel's shared-memory limit is raised and its error word
// (kErrTimeout | kErrNonFinite bits, cleared when read) allocated once.
constexpr int kMaxDevices = 64;
std::mutex g_dev_mu;
int *g_err[kMaxDevices] = {};
// test hook (kv_debug_gemm_stall): copies withheld and a short wait limit
int g_stall_test = 0;

int *device_err_word(int dev) {
    KV_REQUIRE(dev >= 0 && dev < kMaxDevices, KV_EINVAL, "device index out of range");
    std::lock_guard<std::mutex> lk(g_dev_mu);
    if (!g_err[dev]) {
        KV_CUDA(cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
        int *e = nullptr;
        KV_CUDA(cudaMalloc(&e, sizeof(int)));
        KV_CUDA(cudaMemset(e, 0, sizeof(int)));
        g_err[dev] = e;
    }
    return g_err[dev];
}

}  // namespace

// Slicing jobs and per-segment panel addresses of a mixed-precision plan:
// one job per distinct (block, operation) view of A and of B.
void plan_mixed(GemmPlan &g) {
    g.ajobs.clear();
    g.bjobs.clear();
    g.xsegs.assign(g.segs.size(), SegX{});
    g.a_planes = g.b_planes = 0;
    g.a_exps = g.b_exps = 0;
    std::vector<std::pair<int, int>> seg_mn(g.segs.size(), {0, 0});
    std::vector<std::pair<int, int>> seg_job(g.segs.size(), {0, 0});  // (A view, B view) of each segment
    for (auto &t : g.tiles)
        for (int s = t.seg_begin; s < t.seg_end; ++s) seg_mn[s] = {t.M, t.N};
    // one job per distinct (block offset, operation) of each operand
    std::unordered_map<int64_t, int> amap, bmap;
    amap.reserve(2 * g.segs.size());
    bmap.reserve(2 * g.segs.size());
    for (size_t s = 0; s < g.segs.size(); ++s) {
        const GemmSeg &sg = g.segs[s];
        const int M = seg_mn[s].first, N = seg_mn[s].second;
        if (M == 0) continue;  // segment of no tile
        const int nkc = (sg.K + BKC - 1) / BKC;
        auto ia = amap.find(sg.a_off * 4 + sg.opa);
        if (ia == amap.end()) {
            SliceJob j{};
            j.src_off = sg.a_off;
            j.dst_off = g.a_planes;
            j.rows = M;
            j.K = sg.K;
            j.ld = sg.lda;
            j.trans = (sg.opa == 1 || sg.opa == 2) ? 1 : 0;
            j.conj = (sg.opa == 1 || sg.opa == 3) ? 1 : 0;
            j.exp_off = (int)g.a_exps;
            j.nkc = nkc;
            j.entry = kAllSteps;
            j.ks_off = -1;
            const int nrt = (M + BM - 1) / BM;
            g.a_planes += (int64_t)nrt * nkc * A_PANEL;
            g.a_exps += (int64_t)nrt * BM;
            ia = amap.emplace(sg.a_off * 4 + sg.opa, (int)g.ajobs.size()).first;
            g.ajobs.push_back(j);
        }
        auto ib = bmap.find(sg.b_off * 4 + sg.opb);
        if (ib == bmap.end()) {
            SliceJob j{};
            j.src_off = sg.b_off;
            j.dst_off = g.b_planes;
            j.rows = N;
            j.K = sg.K;
            j.ld = sg.ldb;
            j.trans = (sg.opb == 0 || sg.opb == 3) ? 1 : 0;  // B element (n, k) at b[k*ldb + n]
            j.conj = (sg.opb == 2 || sg.opb == 3) ? 1 : 0;
            j.exp_off = (int)g.b_exps;
            j.nkc = nkc;
            j.entry = kAllSteps;
            j.ks_off = -1;
            const int nnt = (N + BN - 1) / BN;
            g.b_planes += (int64_t)nnt * nkc * B_PANEL;
            g.b_exps += (int64_t)nnt * BN;
            ib = bmap.emplace(sg.b_off * 4 + sg.opb, (int)g.bjobs.size()).first;
            g.bjobs.push_back(j);
        }
        seg_job[s] = {ia->second, ib->second};
        const SliceJob &ja = g.ajobs[ia->second], &jb = g.bjobs[ib->second];
        KV_REQUIRE(ja.rows == M && jb.rows == N && ja.K == sg.K && jb.K == sg.K, KV_EINVAL,
                   "internal: inconsistent block views in a mixed-precision plan");
        g.xsegs[s] = SegX{ja.dst_off, jb.dst_off, nkc, ja.exp_off, jb.exp_off, sg.entry};
        g.ajobs[ia->second].entry = std::min(g.ajobs[ia->second].entry, sg.entry);
        g.bjobs[ib->second].entry = std::min(g.bjobs[ib->second].entry, sg.entry);
    }
    // balancing: A and B views joined by a segment share one vector of
    // per-k scales, so the views of each connected component get one range
    g.k_scales = 0;
    if (g.balance_k) {
        const int na = (int)g.ajobs.size(), nb = (int)g.bjobs.size();
        std::vector<int> parent(na + nb);
        for (int i = 0; i < na + nb; ++i) parent[i] = i;
        auto root = [&](int x) {
            while (parent[x] != x) x = parent[x] = parent[parent[x]];
            return x;
        };
        for (size_t s = 0; s < g.segs.size(); ++s) {
            if (seg_mn[s].first == 0) continue;
            const int a = root(seg_job[s].first), b = root(na + seg_job[s].second);
            if (a != b) parent[a] = b;
        }
        std::vector<int64_t> comp_off(na + nb, -1);
        std::vector<int> comp_k(na + nb, -1);
        auto assign = [&](SliceJob &j, int id) {
            const int c = root(id);
            if (comp_off[c] < 0) {
                comp_off[c] = g.k_scales;
                comp_k[c] = j.K;
                g.k_scales += j.K;
            }
            KV_REQUIRE(comp_k[c] == j.K, KV_EINVAL, "internal: views of one segment component differ in K");
            j.ks_off = (int)comp_off[c];
        };
        for (int i = 0; i < na; ++i) assign(g.ajobs[i], i);
        for (int i = 0; i < nb; ++i) assign(g.bjobs[i], na + i);
        KV_REQUIRE(g.k_scales < (1ll << 31), KV_EINVAL, "mixed-precision plan too large");
    }
    g.aitems.clear();
    g.bitems.clear();
    for (size_t i = 0; i < g.ajobs.size(); ++i)
        for (int r0 = 0; r0 < g.ajobs[i].rows; r0 += 8) g.aitems.push_back({(int)i, r0});
    for (size_t i = 0; i < g.bjobs.size(); ++i)
        for (int r0 = 0; r0 < g.bjobs[i].rows; r0 += 8) g.bitems.push_back({(int)i, r0});
    KV_REQUIRE(g.a_exps < (1ll << 31) && g.b_exps < (1ll << 31), KV_EINVAL, "mixed-precision plan too large");
    g.d_ajobs = upload_vec(g.ajobs);
    g.d_bjobs = upload_vec(g.bjobs);
    g.d_xsegs = upload_vec(g.xsegs);
    g.d_aitems = upload_vec(g.aitems);
    g.d_bitems = upload_vec(g.bitems);
}

// Grid of the cooperative slicing launch on a device: every CTA resident at
// once (0: cooperative launches unavailable).  Checked once per device.
static int slice_coop_grid(int device) {
    static std::mutex mu;
    static int grid[kMaxDevices] = {};  // 0 unknown, > 0 the grid, -1 unavailable
    if (device < 0 || device >= kMaxDevices) return 0;
    std::lock_guard<std::mutex> lk(mu);
    if (grid[device] == 0) {
        int coop = 0, per_sm = 0, sms = 0;
        KV_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device));
        KV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        KV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_slice_coop, 256, 0));
        grid[device] = (coop && per_sm > 0) ? per_sm * sms : -1;
    }
    return std::max(0, grid[device]);
}

void launch_gemm_mixed(const GemmPlan &p, const double2 *A, const double2 *B, double2 *C, double alpha,
                       const int *skip, int step) {
    if (p.tiles.empty()) return;
    KV_REQUIRE(p.tile_m == BM && p.tile_n == BN && p.xsegs.size() == p.segs.size(), KV_EINVAL,
               "internal: GEMM plan not prepared for the tensor-core path");
    auto &c = ctx();
    int *err = device_err_word(c.device);
    DevBuf ap(std::max<int64_t>(1, p.a_planes) * sizeof(__half)), bp(std::max<int64_t>(1, p.b_planes) * sizeof(__half));
    DevBuf ae(std::max<int64_t>(1, p.a_exps) * sizeof(int)), be(std::max<int64_t>(1, p.b_exps) * sizeof(int));
    int n = 0;
    const bool bal = p.balance_k && p.k_scales > 0 && !p.aitems.empty() && !p.bitems.empty();
    DevBuf kmax(bal ? 2 * (size_t)p.k_scales * sizeof(unsigned long long) : 8);
    unsigned long long *km = bal ? kmax.as<unsigned long long>() : nullptr;
    int na = (int)p.aitems.size(), nb = (int)p.bitems.size();
    const int grid = slice_coop_grid(c.device);
    if (na + nb > 0 && &c == &main_ctx() && grid > 0) {
        // one cooperative launch (zero, maxima, slicing); only on the main
        // context's stream, whose kernels never overlap, so its grid barrier
        // waits on no other launch of this library
        const SliceJob *aj = p.d_ajobs.as<SliceJob>(), *bj = p.d_bjobs.as<SliceJob>();
        const int2 *ai = p.d_aitems.as<int2>(), *bi = p.d_bitems.as<int2>();
        __half *aph = ap.as<__half>(), *bph = bp.as<__half>();
        int *aex = ae.as<int>(), *bex = be.as<int>();
        int64_t ks = p.k_scales;
        void *args[] = {&aj, &ai, &na, &bj, &bi, &nb, &A, &B, &aph, &bph, &aex, &bex, &alpha, &skip, &step, &err, &km,
                        &ks};
        KV_CUDA(cudaLaunchCooperativeKernel((const void *)k_slice_coop, dim3((unsigned)std::min(na + nb, grid)),
                                            dim3(256), args, 0, c.stream));
        ++n;
    } else if (na + nb > 0) {
        if (bal) {
            KV_CUDA(cudaMemsetAsync(kmax.p, 0, 2 * (size_t)p.k_scales * sizeof(unsigned long long), c.stream));
            k_kmax<<<(unsigned)(na + nb), 256, 0, c.stream>>>(p.d_ajobs.as<SliceJob>(), p.d_aitems.as<int2>(), na,
                                                              p.d_bjobs.as<SliceJob>(), p.d_bitems.as<int2>(), A, B,
                                                              km, p.k_scales, skip, step);
            KV_CUDA(cudaGetLastError());
            ++n;
        }
        k_slice_ab<<<(unsigned)(na + nb), 256, 0, c.stream>>>(
            p.d_ajobs.as<SliceJob>(), p.d_aitems.as<int2>(), na, p.d_bjobs.as<SliceJob>(), p.d_bitems.as<int2>(), A, B,
            ap.as<__half>(), bp.as<__half>(), ae.as<int>(), be.as<int>(), alpha, skip, step, err, km, p.k_scales);
        KV_CUDA(cudaGetLastError());
        ++n;
    }
    // persistent: one CTA per SM at most (the kernel holds all of an SM's tensor memory)
    const int ntiles = (int)p.tiles.size();
    k_gemm_tc<<<(unsigned)std::min(ntiles, c.num_sms), NTHREADS, SMEM_BYTES, c.stream>>>(
        p.d_tiles.as<GemmTile>(), ntiles, p.d_xsegs.as<SegX>(), ap.as<__half>(), bp.as<__half>(), ae.as<int>(),
        be.as<int>(), C, skip, err, step, p.write_inactive ? 1 : 0, g_stall_test ? (1ll << 10) : WAIT_LIMIT,
        g_stall_test);
    KV_CUDA(cudaGetLastError());
    counted(n + 1);
    // the slices are freed stream-ordered after the GEMM
}

// KV_ETIMEOUT if a tensor-core wait gave up, else KV_ENONFINITE if an operand
// held an Inf or NaN, since the last call on this device (then cleared)
int mixed_gemm_status() {
    const int dev = ctx().device;
    int *e = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_dev_mu);
        if (dev >= 0 && dev < kMaxDevices) e = g_err[dev];
    }
    if (!e) return KV_OK;
    int h = 0;
    KV_CUDA(cudaMemcpy(&h, e, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) KV_CUDA(cudaMemset(e, 0, sizeof(int)));
    return (h & kErrTimeout) ? KV_ETIMEOUT : (h & kErrNonFinite) ? KV_ENONFINITE : KV_OK;
}

void set_gemm_stall_test(int on) { g_stall_test = on ? 1 : 0; }

}  // namespace kv
