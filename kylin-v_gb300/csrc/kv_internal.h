// Internal runtime of libkvgpu: device block tensors, contraction plans,
// kernel launch wrappers.  Not part of the public ABI (include/kvgpu.h).
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <complex>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/kvgpu.h"

namespace kv {

constexpr int kMaxRank = 6;
constexpr int kMaxKrylov = 32;  // largest Krylov dimension of local_krylov
using cplx = std::complex<double>;

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define KV_CUDA(expr)                                                                           \
    do {                                                                                        \
        cudaError_t e_ = (expr);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            throw ::kv::Error(e_ == cudaErrorMemoryAllocation ? KV_ENOMEM : KV_ECUDA,            \
                              std::string(#expr) + ": " + cudaGetErrorString(e_));              \
    } while (0)

#define KV_REQUIRE(cond, code, msg)                          \
    do {                                                     \
        if (!(cond)) throw ::kv::Error((code), (msg));       \
    } while (0)

// ------------------------------------------------------------------ context
struct KrylovState;

// One profiled launch: its events, the reference flops of the block pairs a
// grouped GEMM multiplies (or the algorithmic bytes of a Lanczos step or an
// MPO mixing), and (for Lanczos iterations) the Krylov state and iteration
// whose stop flag may have skipped it.
enum ProfKind { kProfGemm = 0, kProfLanczos = 1, kProfMix = 2 };
struct ProfRec {
    cudaEvent_t a, b;
    double flops;
    const KrylovState *st;
    int k;
    int kind = kProfGemm;  // kProfLanczos / kProfMix: flops holds bytes
};

struct PlanCache;  // H_eff plans keyed by block structure (kv_engine.cu)

// Device, stream and host staging of one host thread's work.  The calling
// thread uses the library's main context; kv_sweep_batched binds a worker
// context (its own stream, staging ring and plan cache) to each of its
// threads, so chains advance on concurrent streams.
struct Context {
    int device = -1;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    long long launches = 0;  // kernels launched by this library since kv_init
    bool prof = false;       // bracket grouped-GEMM launches with events
    std::vector<ProfRec> prof_pending;
    std::vector<cudaEvent_t> ev_free;
    double prof_ms = 0.0, prof_flops = 0.0;
    long long prof_launches = 0;
    // profiled Lanczos steps and MPO mixings that ran, per ProfKind: device
    // ms, algorithmic bytes, launches
    double bw_ms[3] = {}, bw_bytes[3] = {};
    long long bw_launches[3] = {};
    // pinned staging ring for plan uploads: kRingChunks chunks of kRingChunk bytes
    static constexpr int kRingChunks = 16;
    static constexpr size_t kRingChunk = 4u << 20;
    char *ring = nullptr;
    int ring_cur = 0;
    size_t ring_used = 0;
    cudaEvent_t ring_ev[kRingChunks] = {};
    bool ring_live[kRingChunks] = {};
    PlanCache *plans = nullptr;
    // charge sectors through the mixed/FP64 SVD: count, columns, rank
    // reached by the QR reduction (else min(rows, columns)), Jacobi sweeps
    struct SvdStats {
        long long sectors = 0, columns = 0, rank = 0, sweeps = 0;
        int max_sweeps = 0;
    } svd;
    long long plans_built = 0;  // plan-cache misses
    double plan_ms = 0.0;       // host ms spent building those plans
    // Lanczos early stop: a pinned, device-mapped int that the Krylov
    // kernels set to 1 when the recurrence stops (stop_dev is its device
    // address), and one event per issued iteration
    int *stop_host = nullptr, *stop_dev = nullptr;
    cudaEvent_t iter_ev[kMaxKrylov] = {};
    // local_krylov calls, iterations issued, Krylov dimensions reached
    long long krylov_calls = 0, krylov_issued = 0, krylov_used = 0;
};
// the calling thread's context: its bound worker context, else the main one
Context &ctx();
Context &main_ctx();
void bind_thread_context(Context *c);
// create / destroy a context's stream, staging ring and plan cache
void context_open(Context &c, int device);
void context_close(Context &c);
void require_init();
inline void counted(int n = 1) { ctx().launches += n; }
cudaEvent_t prof_event();
// resolve pending profiled launches; iters_of(st) gives the Krylov dimension
// reached by a state (launches at iteration k >= that were skipped)
void prof_resolve(int (*iters_of)(const KrylovState *, void *), void *arg);

// Stream-ordered device buffer (cudaMallocAsync on the library stream).
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    explicit DevBuf(size_t b) { alloc(b); }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
    DevBuf &operator=(DevBuf &&o) noexcept {
        if (this != &o) { release(); p = o.p; bytes = o.bytes; o.p = nullptr; o.bytes = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t b);
    void release();
    template <class T> T *as() const { return static_cast<T *>(p); }
};

// Host-to-device copy of a small host array through a pinned staging ring,
// so the copy is asynchronous and the source may be freed on return.
void upload_bytes(void *dst, const void *src, size_t n);

template <class T>
DevBuf upload_vec(const std::vector<T> &v) {
    DevBuf b(std::max<size_t>(1, v.size()) * sizeof(T));
    if (!v.empty()) upload_bytes(b.p, v.data(), v.size() * sizeof(T));
    return b;
}

// ------------------------------------------------------------ block tensors
struct BlockMeta {
    std::array<int, kMaxRank> shape{}, qn{};
    int64_t off = 0;   // complex elements from the start of the tensor buffer
    int64_t size = 0;  // complex elements
};

// (shape, charge) of legs [lo, hi) of a block: hash and equality.
inline uint64_t legs_hash(const BlockMeta &b, int lo, int hi) {
    uint64_t h = 0x9E3779B97F4A7C15ull ^ (uint64_t)(hi - lo);
    for (int i = lo; i < hi; ++i) {
        h ^= ((uint64_t)(uint32_t)b.shape[i] << 32) | (uint64_t)(uint32_t)b.qn[i];
        h *= 0xBF58476D1CE4E5B9ull;
        h ^= h >> 31;
    }
    return h;
}
inline bool legs_equal(const BlockMeta &a, int alo, const BlockMeta &b, int blo, int n) {
    for (int i = 0; i < n; ++i)
        if (a.shape[alo + i] != b.shape[blo + i] || a.qn[alo + i] != b.qn[blo + i]) return false;
    return true;
}

// Blocks grouped by the (shape, charge) of legs [lo, hi), each group in block
// order (open addressing over the groups, CSR lists of members).
struct LegIndex {
    const std::vector<BlockMeta> *blk = nullptr;
    int lo = 0, n = 0;
    std::vector<int> slot;   // group id or -1
    std::vector<int> rep;    // first member of each group
    std::vector<int> start;  // members of group g: items[start[g] .. start[g+1])
    std::vector<int> items;
    void build(const std::vector<BlockMeta> &blocks, int lo_, int hi_) {
        blk = &blocks;
        lo = lo_;
        n = hi_ - lo_;
        size_t cap = 16;
        while (cap < 2 * blocks.size()) cap <<= 1;
        slot.assign(cap, -1);
        rep.clear();
        std::vector<int> gid(blocks.size());
        for (size_t j = 0; j < blocks.size(); ++j) {
            size_t h = (size_t)legs_hash(blocks[j], lo, lo + n) & (cap - 1);
            while (slot[h] >= 0 && !legs_equal(blocks[rep[slot[h]]], lo, blocks[j], lo, n)) h = (h + 1) & (cap - 1);
            if (slot[h] < 0) {
                slot[h] = (int)rep.size();
                rep.push_back((int)j);
            }
            gid[j] = slot[h];
        }
        start.assign(rep.size() + 1, 0);
        for (int g : gid) ++start[g + 1];
        for (size_t g = 0; g < rep.size(); ++g) start[g + 1] += start[g];
        items.resize(blocks.size());
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (size_t j = 0; j < blocks.size(); ++j) items[fill[gid[j]]++] = (int)j;
    }
    // group whose key equals legs [xlo, xlo + n) of x, or -1
    int find(const BlockMeta &x, int xlo) const {
        const size_t cap = slot.size();
        size_t h = (size_t)legs_hash(x, xlo, xlo + n) & (cap - 1);
        while (slot[h] >= 0) {
            if (legs_equal((*blk)[rep[slot[h]]], lo, x, xlo, n)) return slot[h];
            h = (h + 1) & (cap - 1);
        }
        return -1;
    }
};

struct Meta {
    int rank = 0;
    std::array<int, kMaxRank> dirs{};
    std::vector<BlockMeta> blocks;
    int64_t nelem = 0;
    // open-addressing index of the full (shape, charge) key; valid while
    // nindexed == blocks.size()
    std::vector<int> slots;
    size_t nindexed = 0;
    void layout();  // contiguous offsets in block order, rebuilds the index
    void rebuild_index() {
        size_t cap = 16;
        while (cap < 2 * blocks.size()) cap <<= 1;
        slots.assign(cap, -1);
        for (size_t j = 0; j < blocks.size(); ++j) {
            size_t h = (size_t)legs_hash(blocks[j], 0, rank) & (cap - 1);
            while (slots[h] >= 0) h = (h + 1) & (cap - 1);
            slots[h] = (int)j;
        }
        nindexed = blocks.size();
    }
    bool same_key(const BlockMeta &a, const BlockMeta &b) const { return legs_equal(a, 0, b, 0, rank); }
    int find(const BlockMeta &b) const {
        if (nindexed == blocks.size() && !slots.empty()) {
            const size_t cap = slots.size();
            size_t h = (size_t)legs_hash(b, 0, rank) & (cap - 1);
            while (slots[h] >= 0) {
                if (same_key(blocks[slots[h]], b)) return slots[h];
                h = (h + 1) & (cap - 1);
            }
            return -1;
        }
        for (size_t i = 0; i < blocks.size(); ++i)
            if (same_key(blocks[i], b)) return (int)i;
        return -1;
    }
    // append b if its key is new; returns its index
    int add(const BlockMeta &b) {
        if (nindexed != blocks.size() || slots.empty()) rebuild_index();
        size_t cap = slots.size();
        size_t h = (size_t)legs_hash(b, 0, rank) & (cap - 1);
        while (slots[h] >= 0) {
            if (same_key(blocks[slots[h]], b)) return slots[h];
            h = (h + 1) & (cap - 1);
        }
        blocks.push_back(b);
        if (2 * blocks.size() > cap) rebuild_index();
        else {
            slots[h] = (int)blocks.size() - 1;
            nindexed = blocks.size();
        }
        return (int)blocks.size() - 1;
    }
};

// A device tensor: host metadata + one contiguous complex128 device buffer.
struct DTensor {
    Meta meta;
    DevBuf buf;
    double2 *data() const { return buf.as<double2>(); }
    static std::shared_ptr<DTensor> make(const Meta &m, bool zero);
};
using TensorP = std::shared_ptr<DTensor>;

TensorP upload_tensor(int rank, const int *dirs, int nb, const int *shapes, const int *qns, const double *data);
TensorP clone(const DTensor &t);
void download_tensor(const DTensor &t, int *dirs, int *shapes, int *qns, double *data);

// ------------------------------------------------------------ GEMM plans
// One output tile of a grouped complex GEMM and the contributions summed into
// it.  C[m, n] = alpha * sum_seg opA(A_seg)[m, k] opB(B_seg)[k, n].
struct GemmSeg {
    int64_t a_off, b_off;  // complex elements into the A / B buffers
    int K, lda, ldb;
    int opa;  // 0: A[m*lda + k]; 1: conj(A[k*lda + m]); 2: A[k*lda + m]; 3: conj(A[m*lda + k])
    int opb;  // 0: B[k*ldb + n]; 1: B[n*ldb + k]; 2: conj(B[n*ldb + k]); 3: conj(B[k*ldb + n])
    int entry = 0;  // Lanczos step from which this block pair is nonzero (launches skip it before)
};
struct GemmTile {
    int64_t c_off;
    int ldc, M, N, m0, n0;
    int seg_begin, seg_end;
};
// Tile shape of the tensor-core path (kv_tc.cu).
constexpr int kMixedTileM = 128, kMixedTileN = 32;

// Tensor-core path: one operand block viewed as GEMM rows x K, sliced into
// fixed-point digit panels (dst_off: FP16 elements into the panel buffer,
// exp_off: first of its per-row exponents).
struct SliceJob {
    int64_t src_off, dst_off;
    int rows, K, ld;
    int trans;  // 0: (row, k) at src[row*ld + k]; 1: at src[k*ld + row]
    int conj;   // negate the imaginary part
    int exp_off, nkc;
    int entry;  // first step at which a segment reading this block is active
    int ks_off; // balanced plans: first of this view's K power-of-two scale entries (-1: none)
};
// Tensor-core path: a segment's sliced A and B blocks.
struct SegX {
    int64_t a_pan, b_pan;
    int nkc, a_exp, b_exp, entry;
};

struct GemmPlan;
void plan_mixed(GemmPlan &g);  // slicing jobs of a plan built with the tensor-core tile shape

struct GemmPlan {
    std::vector<GemmTile> tiles;
    std::vector<GemmSeg> segs;
    DevBuf d_tiles, d_segs;
    double ref_flops = 0.0;  // sum of 8*M*N*K over the reference's zgemm pairs
    int max_k = 0;
    int tile_m = 0, tile_n = 0;
    // tiles whose segments are all inactive at the launch's step write zeros
    // (false: they write nothing; for intermediates only read by active consumers)
    bool write_inactive = true;
    // tensor-core path only.  balance_k: the contracted index is balanced
    // before slicing -- column k of every A view scaled by 2^s_k, row k of
    // every B view by 2^-s_k, s_k from the largest |A[., k]| and |B[k, .]|
    // over the views that meet in a segment -- so that digits of operands
    // whose magnitudes vary along k (MPO channels) keep their precision.
    bool balance_k = false;
    int64_t k_scales = 0;  // entries of the per-k maxima arrays
    std::vector<SliceJob> ajobs, bjobs;
    std::vector<SegX> xsegs;
    std::vector<int2> aitems, bitems;  // (job, first of 8 rows) per slicing CTA
    int64_t a_planes = 0, b_planes = 0, a_exps = 0, b_exps = 0;
    DevBuf d_ajobs, d_bjobs, d_xsegs, d_aitems, d_bitems;
    void upload() {
        d_tiles = upload_vec(tiles);
        d_segs = upload_vec(segs);
        if (tile_m == kMixedTileM && tile_n == kMixedTileN) plan_mixed(*this);
    }
};

// MPO mixing (env_mps_mpo family) with merging of equal output blocks.
struct MixTerm {
    int64_t in_off, w_off;
    int K;          // contracted extent (w_l sector dim * sigma dim)
    int entry = 0;  // Lanczos step from which the input block is nonzero
};
struct MixJob {
    int64_t out_off, count;    // output block and its element count
    int nk_unused, so, wr, rest;
    int term_begin, term_end;
};
// elements of one job handled by one CTA of the mixing kernel (256 threads,
// one element each): small jobs still spread over many SMs
constexpr int kMixChunk = 256;
struct MixItem {  // a chunk of one job handled by one CTA
    int job;
    int64_t start;
};
struct MixPlan {
    std::vector<MixTerm> terms;
    std::vector<MixJob> jobs;
    std::vector<MixItem> items;
    DevBuf d_terms, d_jobs, d_items;
    bool write_inactive = true;  // as GemmPlan::write_inactive, per output block
    // profiling: algorithmic bytes of a launch at Lanczos step s (s clamped to
    // the last entry step), filled on first use
    mutable std::vector<double> prof_bytes;
    void upload() { d_terms = upload_vec(terms); d_jobs = upload_vec(jobs); d_items = upload_vec(items); }
};

// Launch step meaning "every segment / term is active".
constexpr int kAllSteps = 1 << 30;

// ------------------------------------------------------- kernel wrappers
// step: block pairs (and mixing terms) with entry > step are skipped
void launch_gemm_fp64(const GemmPlan &p, const double2 *A, const double2 *B, double2 *C, double alpha,
                      const int *skip, int step = kAllSteps);
// dispatch by precision; st/k identify a Lanczos apply for profiling and
// its step (k >= 0: only block pairs with entry <= k are multiplied)
void run_gemm(const GemmPlan &g, const double2 *A, const double2 *B, double2 *C, double alpha, int precision,
              const int *skip, const KrylovState *st = nullptr, int k = -1, double credit_flops = -1.0);
void launch_gemm_mixed(const GemmPlan &p, const double2 *A, const double2 *B, double2 *C, double alpha,
                       const int *skip, int step = kAllSteps);
// KV_ETIMEOUT if a tensor-core kernel's bounded wait gave up, KV_ENONFINITE if
// a sliced operand held an Inf or NaN, since the last call (then cleared)
int mixed_gemm_status();
// test hook: tensor-core GEMMs issue no copies and wait briefly, so their first
// wait runs out with nothing in flight (kv_debug_gemm_stall)
void set_gemm_stall_test(int on);
void launch_mix(const MixPlan &p, const double2 *in, const double2 *W, double2 *out, const int *skip,
                int step = kAllSteps);
void launch_permute(const double2 *in, double2 *out, const std::vector<int64_t> &desc, int nblocks);
void launch_zero(double2 *p, int64_t n);
void launch_copy(double2 *dst, const double2 *src, int64_t n);

// Krylov (FP64) state kept on the device for one local_krylov call.  The
// loop is launched ahead of the device: every kernel of an iteration returns
// immediately once `done` is set, and the host stops issuing iterations once
// it sees the stop flag (Context::stop_host) of an iteration two behind.
struct KrylovState {
    double2 alpha[kMaxKrylov];  // overlap(V_k, hv) as the reference stores it
    double2 beta[kMaxKrylov];   // overlap(V_{k-1}, hv): the upper off-diagonal
    double err[kMaxKrylov + 1]; // running product of Lanczos norms, err[0] = 1
    double2 coef[kMaxKrylov];   // c = Z exp(-+i Lambda) Z^H e0
    double psi_norm;
    int done;
    int iters;                  // number of alphas (Krylov dimension)
    int status;                 // KV_OK or KV_ENONFINITE
};

int reduce_parts();  // number of partial sums used by the vector kernels
// v0 = psi / |psi|; resets the state (err[0] = 1).  stop (device address,
// may be null) is set to 1 if the recurrence stops here (psi zero or not finite).
void krylov_start(KrylovState *st, const double2 *psi, double2 *v0, int64_t n, double2 *parts, int *stop);
// Support of the Krylov vectors: v_j is zero beyond n[j] complex elements
// (its blocks are a prefix of the layout, the blocks reached within j
// applications of H_eff).
struct KrylovLens {
    int64_t n[kMaxKrylov + 1];
};
// after hv = (dt/2) H v_k: Gram-Schmidt against v_{k-1} (k > 0) and v_k,
// norm, stop test, v_{k+1} = hv / |hv|, each on the vectors' supports; one
// cooperative launch.  stop (device address, may be null) is set to 1 when
// the recurrence stops at this iteration.
void krylov_step(KrylovState *st, int k, double2 *hv, const double2 *vprev, const double2 *vk, double2 *vnext,
                 const KrylovLens &nl, double2 *parts, double tol, int max_iter, int *stop);
// coefficients from the tridiagonal exponential, then out = sum_i c_i v_i on
// the support of v_{iters-1}
void krylov_finish(KrylovState *st, double2 *const *dV, double2 *out, const KrylovLens &nl, int reverse);
// st->coef = exp(-+i T) e0 for T = tridiag(Re alpha, beta upper) of dimension st->iters
void tridiag_exp(KrylovState *st, int reverse);
// sum |x|^2 into a device double (deterministic)
void vec_norm2(const double2 *x, int64_t n, double2 *parts, double *result);

}  // namespace kv
