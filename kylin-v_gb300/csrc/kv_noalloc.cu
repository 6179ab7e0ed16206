// kv_expectation_noalloc: <a|W|b> with every piece of device scratch taken
// from one fixed static device array instead of cudaMalloc.
//
// Some callers cannot let a library allocate GPU memory: host applications
// that own all device memory through their own allocator or a fixed budget,
// and latency-critical loops that must not stall on an allocation.  This
// entry point serves them: it computes the same value as kv_expectation but
// its intermediate environments, MPO-mixing buffers and GEMM task lists live
// in g_noalloc_scratch (kNoAllocBytes, reserved on every GPU that loads this
// library until the process exits).  Inputs are device tensors the caller
// already holds; the result is written to caller-provided host doubles.
//
// Set-up: the first call on a device resolves the array's device address with
// cudaGetSymbolAddress (with that device current, under a mutex, so first
// calls from several threads are safe); make that first call before any
// stream capture.  Every call reuses the same array, so calls that overlap on
// the GPU (different threads or streams) race; buffers are written before
// they are read, nothing relies on the array's previous contents.
//
// Limit: the scratch needed is set by one site, not by the number of sites
// (after each site only the new environment is kept): about
// 16 * D^2 * w * (2 d + 2) bytes for bond dimension D, MPO bond dimension w
// and local dimension d, plus the GEMM and mixing task lists.
#include <cstring>
#include <mutex>
#include <string>

#include "kv_engine.h"

namespace kv {

namespace {

constexpr size_t kNoAllocBytes = size_t(64) << 20;  // 64 MiB
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
char *g_scratch_addr[kMaxDevices] = {};  // device -> address of g_noalloc_scratch

char *scratch_base() {
    const int dev = ctx().device;
    KV_REQUIRE(dev >= 0 && dev < kMaxDevices, KV_EINVAL, "device index out of range");
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (g_scratch_addr[dev]) return g_scratch_addr[dev];
    void *p = nullptr;
    KV_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    KV_REQUIRE(p != nullptr, KV_ECUDA, "cudaGetSymbolAddress returned null for the no-alloc scratch");
    g_scratch_addr[dev] = static_cast<char *>(p);
    return g_scratch_addr[dev];
}

// Bump allocator over the static array.
struct Arena {
    char *base;
    size_t top = 0;
    void *take(size_t n) {
        const size_t off = (top + 255) & ~size_t(255);
        KV_REQUIRE(off + n <= kNoAllocBytes, KV_ENOMEM,
                   "kv_expectation_noalloc: scratch needed exceeds the 64 MiB no-alloc maximum");
        top = off + n;
        return base + off;
    }
};

// DevBufs pointing into the arena.  Every view is cleared when the set goes
// out of scope -- on return and when an exception leaves the scope -- so a
// plan's destructor never hands an arena address to cudaFreeAsync.
struct Views {
    std::vector<DevBuf *> held;
    Views() = default;
    Views(const Views &) = delete;
    Views &operator=(const Views &) = delete;
    void view(DevBuf &d, void *p, size_t n) {
        held.push_back(&d);
        d.p = p;
        d.bytes = n;
    }
    ~Views() {
        for (DevBuf *d : held) {
            d->p = nullptr;
            d->bytes = 0;
        }
    }
};

template <class T>
void put(Arena &ar, Views &vw, DevBuf &d, const std::vector<T> &v) {
    const size_t n = std::max<size_t>(1, v.size()) * sizeof(T);
    void *p = ar.take(n);
    vw.view(d, p, n);
    if (!v.empty()) upload_bytes(p, v.data(), v.size() * sizeof(T));
}

// product<> of two arena-resident operands into an arena-resident output
void arena_product(Arena &ar, const Meta &A, const double2 *a, const Meta &B, const double2 *b, int nc, int opA,
                   int opB, Meta &out, double2 *&c) {
    ProductPlan P = plan_product(A, B, nc, opA, opB);
    out = P.out;
    c = static_cast<double2 *>(ar.take(std::max<int64_t>(1, out.nelem) * sizeof(double2)));
    std::vector<int64_t> offs;
    for (auto &blk : out.blocks) offs.push_back(blk.off);
    build_tiles(P, offs, kTileM(KV_FP64), kTileN(KV_FP64));
    Views vw;
    put(ar, vw, P.gemm.d_tiles, P.gemm.tiles);
    put(ar, vw, P.gemm.d_segs, P.gemm.segs);
    launch_gemm_fp64(P.gemm, a, b, c, 1.0, nullptr);
}

}  // namespace

cplx expectation_noalloc(const std::vector<DTensor *> &bra, const std::vector<DTensor *> &w,
                         const std::vector<DTensor *> &ket) {
    Arena ar{scratch_base()};
    cudaStream_t s = ctx().stream;
    // the current environment always sits at the start of the array
    Meta env;
    env.rank = 3;
    env.dirs = {1, -1, -1};
    BlockMeta b0;
    b0.shape = {1, 1, 1};
    b0.qn = {0, 0, 0};
    env.blocks.push_back(b0);
    env.layout();
    double2 *env_d = static_cast<double2 *>(ar.take(sizeof(double2)));
    const double2 one = make_double2(1.0, 0.0);
    KV_CUDA(cudaMemcpyAsync(env_d, &one, sizeof(one), cudaMemcpyHostToDevice, s));
    KV_CUDA(cudaStreamSynchronize(s));
    for (size_t i = 0; i < bra.size(); ++i) {
        // env_sweep(env, a_i, W_i, b_i): holstein/product.h:505-521
        Meta t1;
        double2 *t1_d;
        arena_product(ar, env, env_d, ket[i]->meta, ket[i]->data(), 1, KV_OP_N, KV_OP_N, t1, t1_d);
        MixPlanFull M = plan_mix(t1, w[i]->meta, 1);
        double2 *t2_d = static_cast<double2 *>(ar.take(std::max<int64_t>(1, M.out.nelem) * sizeof(double2)));
        {
            Views vw;
            put(ar, vw, M.mix.d_terms, M.mix.terms);
            put(ar, vw, M.mix.d_jobs, M.mix.jobs);
            put(ar, vw, M.mix.d_items, M.mix.items);
            launch_mix(M.mix, t1_d, w[i]->data(), t2_d, nullptr);
        }
        Meta next;
        double2 *next_d;
        arena_product(ar, bra[i]->meta, bra[i]->data(), M.out, t2_d, 2, KV_OP_C, KV_OP_N, next, next_d);
        // move the new environment to the start and release everything else
        // (through a free region after it if source and destination overlap)
        const size_t nb = std::max<int64_t>(1, next.nelem) * sizeof(double2);
        const char *src = reinterpret_cast<const char *>(next_d);
        if ((size_t)(src - ar.base) < nb) {
            char *tmp = static_cast<char *>(ar.take(nb));
            KV_CUDA(cudaMemcpyAsync(tmp, src, nb, cudaMemcpyDeviceToDevice, s));
            src = tmp;
        }
        KV_CUDA(cudaMemcpyAsync(ar.base, src, nb, cudaMemcpyDeviceToDevice, s));
        env = next;
        env_d = reinterpret_cast<double2 *>(scratch_base());
        ar.top = std::max<int64_t>(1, env.nelem) * sizeof(double2);
        KV_REQUIRE(ar.top <= kNoAllocBytes, KV_ENOMEM, "kv_expectation_noalloc: environment exceeds the scratch");
    }
    if (env.blocks.empty()) return 0.0;
    std::vector<double2> h(env.nelem);
    KV_CUDA(cudaMemcpyAsync(h.data(), env_d, env.nelem * sizeof(double2), cudaMemcpyDeviceToHost, s));
    KV_CUDA(cudaStreamSynchronize(s));
    const int q = env.blocks[0].qn[0];
    cplx r = 0.0;
    for (auto &blk : env.blocks)
        if (blk.size == 1 && blk.qn[0] == q && blk.qn[1] == 0 && blk.qn[2] == q) r += cplx(h[blk.off].x, h[blk.off].y);
    return r;
}

}  // namespace kv
