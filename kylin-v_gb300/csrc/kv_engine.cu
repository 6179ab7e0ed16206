// Host side of libkvgpu: device tensors, contraction planning, the four
// hot-path operations and the TDVP sweep driver.
//
// Planning mirrors the reference's block matching exactly (so every block
// pair the reference multiplies is multiplied here, and output blocks carry
// the same charges and shapes); execution is batched: one grouped-GEMM launch
// per contraction, one mixing launch per MPO application, and the Lanczos
// loop runs without host synchronisation.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <string>

#include <functional>

#include "kv_engine.h"
#include "kv_svd.h"

namespace kv {

// ================================================================ runtime
static Context g_ctx;
thread_local Context *t_ctx = nullptr;
Context &ctx() { return t_ctx ? *t_ctx : g_ctx; }
Context &main_ctx() { return g_ctx; }
void bind_thread_context(Context *c) { t_ctx = c; }
void require_init() { KV_REQUIRE(g_ctx.device >= 0, KV_ENOTINIT, "kv_init has not been called"); }

void DevBuf::alloc(size_t b) {
    release();
    if (b == 0) b = 16;
    KV_CUDA(cudaMallocAsync(&p, b, ctx().stream));
    bytes = b;
}

void DevBuf::release() {
    if (p) {
        if (ctx().stream) cudaFreeAsync(p, ctx().stream);
        else cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
}

void upload_bytes(void *dst, const void *src, size_t n) {
    auto &c = ctx();
    if (!c.ring || n > Context::kRingChunk) {
        KV_CUDA(cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, c.stream));
        KV_CUDA(cudaStreamSynchronize(c.stream));  // pageable source: keep the copy safe
        return;
    }
    if (c.ring_used + n > Context::kRingChunk) {
        // leave the chunk: fence its copies, move on, wait for the next chunk's old copies
        KV_CUDA(cudaEventRecord(c.ring_ev[c.ring_cur], c.stream));
        c.ring_live[c.ring_cur] = true;
        c.ring_cur = (c.ring_cur + 1) % Context::kRingChunks;
        c.ring_used = 0;
        if (c.ring_live[c.ring_cur]) KV_CUDA(cudaEventSynchronize(c.ring_ev[c.ring_cur]));
        c.ring_live[c.ring_cur] = false;
    }
    char *stage = c.ring + (size_t)c.ring_cur * Context::kRingChunk + c.ring_used;
    std::memcpy(stage, src, n);
    c.ring_used += (n + 255) & ~size_t(255);
    KV_CUDA(cudaMemcpyAsync(dst, stage, n, cudaMemcpyHostToDevice, c.stream));
}

void Meta::layout() {
    int64_t off = 0;
    for (auto &b : blocks) {
        int64_t s = 1;
        for (int i = 0; i < rank; ++i) s *= b.shape[i];
        b.size = s;
        b.off = off;
        off += s;
    }
    nelem = off;
    rebuild_index();
}

TensorP DTensor::make(const Meta &m, bool zero) {
    auto t = std::make_shared<DTensor>();
    t->meta = m;
    t->meta.layout();
    t->buf.alloc(std::max<int64_t>(1, t->meta.nelem) * sizeof(double2));
    if (zero) launch_zero(t->data(), t->meta.nelem);
    return t;
}

TensorP upload_tensor(int rank, const int *dirs, int nb, const int *shapes, const int *qns, const double *data) {
    KV_REQUIRE(rank >= 1 && rank <= kMaxRank, KV_EINVAL, "rank must be in [1, 6]");
    KV_REQUIRE(nb >= 0, KV_EINVAL, "negative block count");
    Meta m;
    m.rank = rank;
    for (int i = 0; i < rank; ++i) {
        KV_REQUIRE(dirs[i] == 1 || dirs[i] == -1, KV_EINVAL, "leg directions must be +1 or -1");
        m.dirs[i] = dirs[i];
    }
    for (int b = 0; b < nb; ++b) {
        BlockMeta bm;
        for (int i = 0; i < rank; ++i) {
            bm.shape[i] = shapes[b * rank + i];
            bm.qn[i] = qns[b * rank + i];
            KV_REQUIRE(bm.shape[i] > 0, KV_EINVAL, "block dimensions must be positive");
        }
        m.blocks.push_back(bm);
    }
    auto t = DTensor::make(m, data == nullptr);
    if (data && t->meta.nelem > 0)
        KV_CUDA(cudaMemcpyAsync(t->data(), data, t->meta.nelem * sizeof(double2), cudaMemcpyHostToDevice,
                                ctx().stream));
    return t;
}

TensorP clone(const DTensor &t) {
    auto c = DTensor::make(t.meta, false);
    launch_copy(c->data(), t.data(), t.meta.nelem);
    return c;
}

void download_tensor(const DTensor &t, int *dirs, int *shapes, int *qns, double *data) {
    const Meta &m = t.meta;
    for (int i = 0; i < m.rank; ++i) dirs[i] = m.dirs[i];
    for (size_t b = 0; b < m.blocks.size(); ++b)
        for (int i = 0; i < m.rank; ++i) {
            shapes[b * m.rank + i] = m.blocks[b].shape[i];
            qns[b * m.rank + i] = m.blocks[b].qn[i];
        }
    if (m.nelem > 0)
        KV_CUDA(cudaMemcpyAsync(data, t.data(), m.nelem * sizeof(double2), cudaMemcpyDeviceToHost, ctx().stream));
    KV_CUDA(cudaStreamSynchronize(ctx().stream));
}

// ========================================================== product plans
static int64_t prod_range(const BlockMeta &b, int lo, int hi) {
    int64_t s = 1;
    for (int i = lo; i < hi; ++i) s *= b.shape[i];
    return s;
}

// product<N1,N2,nc> planning, holstein/product.h:61-201: pairs match on equal
// shape and charge of all nc contracted legs; output blocks are numbered by
// first appearance of (shape, charges); every pair is one zgemm.
ProductPlan plan_product(const Meta &A, const Meta &B, int nc, int opA, int opB, bool keys_only) {
    KV_REQUIRE(opA == KV_OP_N || opA == KV_OP_C, KV_EINVAL, "opA must be N or C");
    KV_REQUIRE(opB == KV_OP_N || opB == KV_OP_T, KV_EINVAL, "opB must be N or T");
    const int n1 = A.rank, n2 = B.rank, nr = n1 + n2 - 2 * nc;
    KV_REQUIRE(nc >= 1 && nc <= std::min(n1, n2) && nr >= 1 && nr <= kMaxRank, KV_EINVAL, "bad contraction rank");
    ProductPlan P;
    P.out.rank = nr;
    for (int i = 0; i < n1 - nc; ++i) {
        int src = (opA == KV_OP_N) ? i : nc + i;
        P.out.dirs[i] = A.dirs[src] * (opA == KV_OP_C ? -1 : 1);
    }
    for (int i = 0; i < n2 - nc; ++i) {
        int src = (opB == KV_OP_N) ? nc + i : i;
        P.out.dirs[n1 - nc + i] = B.dirs[src];
    }
    const int iax1 = (opA == KV_OP_N) ? n1 - nc : 0;
    const int iax2 = (opB == KV_OP_N) ? 0 : n2 - nc;
    const int f1 = (opA == KV_OP_C) ? -1 : 1;
    for (int ax = 0; ax < nc; ++ax)
        KV_REQUIRE(A.dirs[iax1 + ax] * f1 == -B.dirs[iax2 + ax], KV_EMISMATCH,
                   "contracted legs' directions mismatch");
    // B blocks grouped by (shape, charge) of their contracted legs, in block order
    LegIndex bidx;
    bidx.build(B.blocks, iax2, iax2 + nc);
    std::vector<GemmSeg> segs;
    std::vector<std::pair<int, int>> pr;
    std::vector<int> seg_out;
    P.out.slots.reserve(4 * A.blocks.size());
    for (size_t i = 0; i < A.blocks.size(); ++i) {
        const BlockMeta &a = A.blocks[i];
        const int grp = bidx.find(a, iax1);
        if (grp < 0) continue;
        for (int gi = bidx.start[grp]; gi < bidx.start[grp + 1]; ++gi) {
            const int j = bidx.items[gi];
            const BlockMeta &b = B.blocks[j];
            BlockMeta o;
            int nrow = 1, ncol = 1;
            for (int u = 0; u < n1 - nc; ++u) {
                int src = (opA == KV_OP_N) ? u : nc + u;
                o.shape[u] = a.shape[src];
                o.qn[u] = a.qn[src];
                nrow *= a.shape[src];
            }
            for (int u = 0; u < n2 - nc; ++u) {
                int src = (opB == KV_OP_N) ? nc + u : u;
                o.shape[n1 - nc + u] = b.shape[src];
                o.qn[n1 - nc + u] = b.qn[src];
                ncol *= b.shape[src];
            }
            const int nk = (int)(prod_range(a, 0, n1) / nrow);
            const int before = (int)P.out.blocks.size();
            const int pos = P.out.add(o);
            if (pos == before) P.mn.push_back({nrow, ncol});
            P.gemm.ref_flops += 8.0 * nrow * (double)ncol * nk;
            P.gemm.max_k = std::max(P.gemm.max_k, nk);
            if (keys_only) continue;
            GemmSeg sg;
            sg.a_off = a.off;
            sg.b_off = b.off;
            sg.K = nk;
            sg.opa = (opA == KV_OP_N) ? 0 : 1;
            sg.opb = (opB == KV_OP_N) ? 0 : 1;
            sg.lda = (opA == KV_OP_N) ? nk : nrow;
            sg.ldb = (opB == KV_OP_N) ? ncol : nk;
            segs.push_back(sg);
            pr.push_back({(int)i, j});
            seg_out.push_back(pos);
        }
    }
    P.out.layout();
    // segments grouped by output block, each group in discovery order
    const size_t nout = P.out.blocks.size();
    P.out_start.assign(nout + 1, 0);
    for (int o : seg_out) ++P.out_start[o + 1];
    for (size_t o = 0; o < nout; ++o) P.out_start[o + 1] += P.out_start[o];
    P.segs.resize(segs.size());
    P.pairs.resize(segs.size());
    std::vector<int> fill(P.out_start.begin(), P.out_start.end() - 1);
    for (size_t x = 0; x < segs.size(); ++x) {
        const int at = fill[seg_out[x]]++;
        P.segs[at] = segs[x];
        P.pairs[at] = pr[x];
    }
    return P;
}

// Tiles of the grouped GEMM: output block b of the plan is written at
// target_off[b] (complex elements) of the destination buffer.
void build_tiles(ProductPlan &P, const std::vector<int64_t> &target_off, int tile_m, int tile_n) {
    GemmPlan &g = P.gemm;
    g.tiles.clear();
    g.segs = P.segs;
    g.tile_m = tile_m;
    g.tile_n = tile_n;
    for (size_t b = 0; b + 1 < P.out_start.size(); ++b) {
        const int M = P.mn[b].first, N = P.mn[b].second;
        const int sb = P.out_start[b], se = P.out_start[b + 1];
        for (int m0 = 0; m0 < M; m0 += tile_m)
            for (int n0 = 0; n0 < N; n0 += tile_n) g.tiles.push_back({target_off[b], N, M, N, m0, n0, sb, se});
    }
}

void add_zero_tiles(GemmPlan &g, int64_t off, int M, int N, int tile_m, int tile_n) {
    for (int m0 = 0; m0 < M; m0 += tile_m)
        for (int n0 = 0; n0 < N; n0 += tile_n) g.tiles.push_back({off, N, M, N, m0, n0, 0, 0});
}

static std::vector<int64_t> own_offsets(const Meta &m) {
    std::vector<int64_t> o;
    for (auto &b : m.blocks) o.push_back(b.off);
    return o;
}

// Reference flop count of a product<> whose A operand block i stands for
// multA[i] identical blocks of the reference (unmerged MPO-mixing output).
double ref_product_flops(const Meta &A, const Meta &B, int nc, int opA, int opB, const std::vector<double> *multA,
                         const std::vector<double> *multB) {
    const int n1 = A.rank, n2 = B.rank;
    const int iax1 = (opA == KV_OP_N) ? n1 - nc : 0;
    const int iax2 = (opB == KV_OP_N) ? 0 : n2 - nc;
    LegIndex bidx;
    bidx.build(B.blocks, iax2, iax2 + nc);
    std::vector<double> bsum(bidx.rep.size(), 0.0);  // sum of uncontracted sizes of B per key
    for (size_t bi = 0; bi < B.blocks.size(); ++bi) {
        const BlockMeta &b = B.blocks[bi];
        int64_t sz = 1;
        for (int i = 0; i < n2; ++i) sz *= b.shape[i];
        bsum[bidx.find(b, iax2)] += (multB ? (*multB)[bi] : 1.0) * (double)(sz / prod_range(b, iax2, iax2 + nc));
    }
    double f = 0.0;
    for (size_t ai = 0; ai < A.blocks.size(); ++ai) {
        const BlockMeta &a = A.blocks[ai];
        const int g = bidx.find(a, iax1);
        if (g < 0) continue;
        int64_t sz = 1;
        for (int i = 0; i < n1; ++i) sz *= a.shape[i];
        f += (multA ? (*multA)[ai] : 1.0) * 8.0 * (double)sz * bsum[g];
    }
    return f;
}

// ============================================================ mix plans
// env_mps_mpo / env_mps2_mpo1 / env_mps2_mpo2 (holstein/product.h:203-477):
// legs lead, lead+1 of lm (w_l, sigma) contract with legs 1, 2 of W; W's legs
// 0, 3 (sigma', w_r) replace them.  Equal output blocks are merged here (the
// reference keeps them apart and the following product<> sums them).
MixPlanFull plan_mix(const Meta &lm, const Meta &W, int lead, const std::vector<double> *mult_in, bool keys_only) {
    MixPlanFull R;
    R.out.rank = lm.rank;
    R.out.dirs = lm.dirs;
    R.out.dirs[lead] = W.dirs[0];
    R.out.dirs[lead + 1] = W.dirs[3];
    struct Flat {
        int pos, in;
        MixTerm term;
        double coef;
    };
    std::vector<Flat> flat;
    std::vector<std::array<int, 3>> geo;  // so, wr, rest
    LegIndex widx;
    widx.build(W.blocks, 1, 3);
    for (size_t ai = 0; ai < lm.blocks.size(); ++ai) {
        const BlockMeta &a = lm.blocks[ai];
        const double mi = mult_in ? (*mult_in)[ai] : 1.0;
        const int grp = widx.find(a, lead);
        if (grp < 0) continue;
        for (int gi = widx.start[grp]; gi < widx.start[grp + 1]; ++gi) {
            const BlockMeta &w = W.blocks[widx.items[gi]];
            BlockMeta o = a;
            o.shape[lead] = w.shape[0];
            o.qn[lead] = w.qn[0];
            o.shape[lead + 1] = w.shape[3];
            o.qn[lead + 1] = w.qn[3];
            const int rest = (int)prod_range(a, lead + 2, lm.rank);
            const int before = (int)R.out.blocks.size();
            const int pos = R.out.add(o);
            if (pos == before) {
                geo.push_back({w.shape[0], w.shape[3], rest});
                R.mult.push_back(0.0);
            }
            R.mult[pos] += mi;  // the reference keeps each matched pair as its own block
            const int K = a.shape[lead] * a.shape[lead + 1];
            const double nk = (double)prod_range(a, 0, lead);
            const double coef = 8.0 * nk * w.shape[0] * (double)w.shape[3] * rest * K;
            R.ref_flops += mi * coef;
            if (!keys_only) flat.push_back({pos, (int)ai, MixTerm{a.off, w.off, K}, coef});
        }
    }
    R.out.layout();
    if (keys_only) return R;
    const size_t nout = R.out.blocks.size();
    std::vector<int> start(nout + 1, 0);
    for (auto &f : flat) ++start[f.pos + 1];
    for (size_t b = 0; b < nout; ++b) start[b + 1] += start[b];
    R.mix.terms.resize(flat.size());
    R.term_in.resize(flat.size());
    R.term_coef.resize(flat.size());
    {
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (auto &f : flat) {
            const int at = fill[f.pos]++;
            R.mix.terms[at] = f.term;
            R.term_in[at] = f.in;
            R.term_coef[at] = f.coef;
        }
    }
    for (size_t b = 0; b < nout; ++b) {
        MixJob j;
        j.out_off = R.out.blocks[b].off;
        j.count = R.out.blocks[b].size;
        j.nk_unused = 0;
        j.so = geo[b][0];
        j.wr = geo[b][1];
        j.rest = geo[b][2];
        j.term_begin = start[b];
        j.term_end = start[b + 1];
        const int job = (int)R.mix.jobs.size();
        R.mix.jobs.push_back(j);
        for (int64_t s = 0; s < j.count; s += kMixChunk) R.mix.items.push_back({job, s});
    }
    return R;
}

// ========================================================== precision
cudaEvent_t prof_event() {
    auto &c = ctx();
    if (!c.ev_free.empty()) {
        cudaEvent_t e = c.ev_free.back();
        c.ev_free.pop_back();
        return e;
    }
    cudaEvent_t e;
    KV_CUDA(cudaEventCreate(&e));
    return e;
}

void prof_resolve(int (*iters_of)(const KrylovState *, void *), void *arg) {
    auto &c = ctx();
    if (c.prof_pending.empty()) return;
    KV_CUDA(cudaStreamSynchronize(c.stream));
    for (auto &r : c.prof_pending) {
        float ms = 0.f;
        KV_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
        const bool ran = !r.st || (iters_of && r.k < iters_of(r.st, arg));
        if (r.kind != kProfGemm) {
            if (ran) {  // a launch past the stop returns at once: neither its time nor bytes count
                c.bw_ms[r.kind] += ms;
                c.bw_bytes[r.kind] += r.flops;
                c.bw_launches[r.kind] += 1;
            }
        } else {
            c.prof_ms += ms;
            c.prof_launches += 1;
            if (ran) c.prof_flops += r.flops;
        }
        c.ev_free.push_back(r.a);
        c.ev_free.push_back(r.b);
    }
    c.prof_pending.clear();
}

void run_gemm(const GemmPlan &g, const double2 *A, const double2 *B, double2 *C, double alpha, int precision,
              const int *skip, const KrylovState *st, int k, double credit_flops) {
    precision = gemm_mixed(precision) ? KV_MIXED_TF32 : KV_FP64;
    if (g.tiles.empty()) return;
    const int step = k >= 0 ? k : kAllSteps;
    auto &c = ctx();
    ProfRec rec{};
    if (c.prof) {
        rec = {prof_event(), prof_event(), credit_flops >= 0.0 ? credit_flops : g.ref_flops, st, k};
        KV_CUDA(cudaEventRecord(rec.a, c.stream));
    }
    if (precision == KV_FP64) launch_gemm_fp64(g, A, B, C, alpha, skip, step);
    else if (precision == KV_MIXED_TF32) launch_gemm_mixed(g, A, B, C, alpha, skip, step);
    else throw Error(KV_EINVAL, "unknown precision mode");
    if (c.prof) {
        KV_CUDA(cudaEventRecord(rec.b, c.stream));
        c.prof_pending.push_back(rec);
    }
}

// Algorithmic bytes of one mixing launch at Lanczos step `step`: each output
// element reads 16 B of input per contracted index of every active term and
// writes 16 B (the MPO blocks, a few KB, are left out).  A block with no
// active term is written as zeros only where the plan writes inactive blocks.
// The figure changes only at the terms' entry steps (Lanczos iterations, so
// small), so it is tabulated once per plan for steps 0 .. the last entry.
static double mix_bytes(const MixPlan &p, int step) {
    if (p.prof_bytes.empty()) {
        constexpr int kMaxTabulated = 63;
        int last = 0;
        for (const MixTerm &t : p.terms) last = std::max(last, std::min(t.entry, kMaxTabulated));
        p.prof_bytes.assign((size_t)last + 1, 0.0);
        for (int s = 0; s <= last; ++s) {
            double b = 0.0;
            for (const MixJob &j : p.jobs) {
                double per = 0.0;
                bool any = false;
                for (int t = j.term_begin; t < j.term_end; ++t)
                    if (p.terms[t].entry <= s) {
                        per += 16.0 * p.terms[t].K;
                        any = true;
                    }
                if (any || p.write_inactive) b += (per + 16.0) * (double)j.count;
            }
            p.prof_bytes[s] = b;
        }
    }
    return p.prof_bytes[(size_t)std::min<int>(std::max(step, 0), (int)p.prof_bytes.size() - 1)];
}

// launch_mix, event-timed with its algorithmic bytes when profiling is on
static void run_mix(const MixPlan &p, const double2 *in, const double2 *W, double2 *out, const int *skip, int step,
             const KrylovState *st, int k) {
    if (p.items.empty()) return;
    auto &c = ctx();
    ProfRec rec{};
    if (c.prof) {
        rec = {prof_event(), prof_event(), mix_bytes(p, step), st, k, kProfMix};
        KV_CUDA(cudaEventRecord(rec.a, c.stream));
    }
    launch_mix(p, in, W, out, skip, step);
    if (c.prof) {
        KV_CUDA(cudaEventRecord(rec.b, c.stream));
        c.prof_pending.push_back(rec);
    }
}

static void check_precision(int precision) {
    KV_REQUIRE(precision >= KV_FP64 && precision <= KV_MIXED_SVD, KV_EINVAL, "unknown precision mode");
}

// =========================================================== operations
TensorP op_product(const DTensor &A, const DTensor &B, int nc, int opA, int opB, int precision, Flops *fl) {
    check_precision(precision);
    ProductPlan P = plan_product(A.meta, B.meta, nc, opA, opB);
    if (fl) fl->gemm += P.gemm.ref_flops;
    auto out = DTensor::make(P.out, false);
    build_tiles(P, own_offsets(out->meta), kTileM(precision), kTileN(precision));
    P.gemm.upload();
    run_gemm(P.gemm, A.data(), B.data(), out->data(), 1.0, precision, nullptr);
    return out;
}

// --------------------------------------------------------- H_eff plans
// Krylov layout.  The reference's Lanczos vector v_k carries the blocks
// reached from psi within k applications of H_eff (hv += V_{k-1} beta,
// V_k alpha merge block sets, holstein/exponential.h:126-137), and iteration
// k multiplies exactly the block pairs of v_k.  Here the layout is psi's
// blocks followed by the blocks first reached at application 1, 2, ..., napply
// = max(1, max_iter - 1) (v_k occupies a prefix of the layout), found by
// applying the planner to the newly reached blocks only.  Every block pair
// and mixing term carries the application from which its input is nonzero
// (its entry): launches at iteration k skip entries > k, the vector kernels
// work on the prefix, and iter_flops[k] credits exactly the pairs with entry
// <= k.
HeffPlan plan_heff(int nsite, const Meta &L, const Meta &psi, const Meta *W1, const Meta *W2, const Meta &R,
                   int precision, int max_iter) {
    HeffPlan H;
    H.nsite = nsite;
    H.napply = std::max(1, max_iter - 1);
    Meta K = psi;
    K.layout();
    std::vector<int> entry(K.blocks.size(), 0);
    H.prefix.push_back(K.nelem);
    Meta fresh = psi;  // blocks whose images under H_eff are not yet in K
    fresh.layout();
    for (int reached = 1; reached <= H.napply && !fresh.blocks.empty(); ++reached) {
        Meta last = plan_product(L, fresh, 1, KV_OP_N, KV_OP_N, true).out;
        if (nsite >= 1) last = plan_mix(last, *W1, 1, nullptr, true).out;
        if (nsite == 2) last = plan_mix(last, *W2, 2, nullptr, true).out;
        const Meta out = plan_product(last, R, 2, KV_OP_N, KV_OP_T, true).out;
        Meta next;
        next.rank = K.rank;
        next.dirs = K.dirs;
        for (auto &b : out.blocks) {
            const size_t before = K.blocks.size();
            if ((size_t)K.add(b) == before) {
                entry.push_back(reached);
                next.blocks.push_back(b);
            }
        }
        K.layout();
        H.prefix.push_back(K.nelem);
        next.layout();
        fresh = std::move(next);
    }
    while ((int)H.prefix.size() <= H.napply) H.prefix.push_back(K.nelem);
    // the inputs: blocks of v_0 .. v_{napply-1} (a prefix of K, same offsets)
    Meta Kin;
    Kin.rank = K.rank;
    Kin.dirs = K.dirs;
    for (size_t b = 0; b < K.blocks.size() && entry[b] < H.napply; ++b) Kin.blocks.push_back(K.blocks[b]);
    Kin.layout();
    H.p1 = plan_product(L, Kin, 1, KV_OP_N, KV_OP_N);
    std::vector<int> e_last(H.p1.out.blocks.size(), kAllSteps);
    for (size_t b = 0; b < H.p1.out.blocks.size(); ++b)
        for (int x = H.p1.out_start[b]; x < H.p1.out_start[b + 1]; ++x) {
            const int e = entry[H.p1.pairs[x].second];
            H.p1.segs[x].entry = e;
            e_last[b] = std::min(e_last[b], e);
        }
    // a mixing term is live from its input block's entry; an output block from its first live term
    auto mix_entries = [](MixPlanFull &m, const std::vector<int> &ein) {
        std::vector<int> eout(m.out.blocks.size(), kAllSteps);
        for (size_t j = 0; j < m.mix.jobs.size(); ++j)
            for (int t = m.mix.jobs[j].term_begin; t < m.mix.jobs[j].term_end; ++t) {
                const int e = ein[m.term_in[t]];
                m.mix.terms[t].entry = e;
                eout[j] = std::min(eout[j], e);
            }
        return eout;
    };
    const Meta *last = &H.p1.out;
    if (nsite >= 1) {
        H.m1 = plan_mix(*last, *W1, 1);
        e_last = mix_entries(H.m1, e_last);
        last = &H.m1.out;
    }
    if (nsite == 2) {
        H.m2 = plan_mix(*last, *W2, 2);
        e_last = mix_entries(H.m2, e_last);
        last = &H.m2.out;
    }
    H.p2 = plan_product(*last, R, 2, KV_OP_N, KV_OP_T);
    for (size_t x = 0; x < H.p2.segs.size(); ++x) H.p2.segs[x].entry = e_last[H.p2.pairs[x].first];
    // reference flops of iteration k: the pairs and terms live at k, MPO-mixing
    // outputs counted once per matched reference block (the reference does not
    // merge them, holstein/product.h:203-477)
    for (int k = 0; k < max_iter; ++k) {
        Flops f;
        std::vector<double> mult(H.p1.out.blocks.size(), 0.0);
        for (size_t b = 0; b < H.p1.out.blocks.size(); ++b)
            for (int x = H.p1.out_start[b]; x < H.p1.out_start[b + 1]; ++x)
                if (H.p1.segs[x].entry <= k) {
                    f.gemm += 8.0 * H.p1.mn[b].first * (double)H.p1.mn[b].second * H.p1.segs[x].K;
                    mult[b] = 1.0;
                }
        for (MixPlanFull *m : {nsite >= 1 ? &H.m1 : nullptr, nsite == 2 ? &H.m2 : nullptr}) {
            if (!m) continue;
            std::vector<double> mo(m->out.blocks.size(), 0.0);
            for (size_t j = 0; j < m->mix.jobs.size(); ++j)
                for (int t = m->mix.jobs[j].term_begin; t < m->mix.jobs[j].term_end; ++t)
                    if (m->mix.terms[t].entry <= k) {
                        const double mi = mult[m->term_in[t]];
                        mo[j] += mi;
                        f.mix += mi * m->term_coef[t];
                    }
            mult = std::move(mo);
        }
        for (size_t b = 0; b < H.p2.out.blocks.size(); ++b)
            for (int x = H.p2.out_start[b]; x < H.p2.out_start[b + 1]; ++x) {
                const GemmSeg &sg = H.p2.segs[x];
                if (sg.entry <= k)
                    f.gemm += mult[H.p2.pairs[x].first] * 8.0 * H.p2.mn[b].first * (double)H.p2.mn[b].second * sg.K;
            }
        H.iter_flops.push_back(f);
    }
    H.klayout = K;
    build_tiles(H.p1, own_offsets(H.p1.out), kTileM(precision), kTileN(precision));
    // intermediates: blocks with no live input are neither computed nor read
    H.p1.gemm.write_inactive = false;
    H.m1.mix.write_inactive = false;
    H.m2.mix.write_inactive = false;
    std::vector<int64_t> tgt;
    std::vector<char> produced(K.blocks.size(), 0);
    for (auto &b : H.p2.out.blocks) {
        int k = K.find(b);
        KV_REQUIRE(k >= 0, KV_EINVAL, "internal: H_eff output outside the Krylov layout");
        tgt.push_back(K.blocks[k].off);
        produced[k] = 1;
    }
    build_tiles(H.p2, tgt, kTileM(precision), kTileN(precision));
    // blocks of the layout that H_eff does not produce are written as zeros
    for (size_t k = 0; k < K.blocks.size(); ++k)
        if (!produced[k]) {
            const BlockMeta &b = K.blocks[k];
            int M = 1;
            for (int i = 0; i < K.rank - 1; ++i) M *= b.shape[i];
            add_zero_tiles(H.p2.gemm, b.off, M, b.shape[K.rank - 1], kTileM(precision), kTileN(precision));
        }
    // Both products contract indices along which the operands' magnitudes
    // span orders of magnitude: the first the bond index of psi (its entries
    // fall with the bond's Schmidt values), the second (MPO channel, bond)
    // (accumulated block energy against identity, and the other bond's
    // Schmidt values).  The mixed path balances those indices before slicing.
    H.p1.gemm.balance_k = true;
    H.p1.gemm.upload();
    H.p2.gemm.balance_k = true;
    H.p2.gemm.upload();
    if (nsite >= 1) H.m1.mix.upload();
    if (nsite == 2) H.m2.mix.upload();
    return H;
}

// ---------------------------------------------------------- plan cache
// H_eff plans depend only on the block structures (charges, shapes, order) of
// L, psi, W1, W2, R; in a steady sweep the same structures recur every time
// step, so plans (host task lists and their device copies, no data) are cached.
namespace {
void key_meta(std::vector<int> &v, const Meta *m) {
    if (!m) { v.push_back(-1); return; }
    v.push_back(m->rank);
    v.push_back((int)m->blocks.size());
    for (int i = 0; i < m->rank; ++i) v.push_back(m->dirs[i]);
    for (auto &b : m->blocks)
        for (int i = 0; i < m->rank; ++i) { v.push_back(b.shape[i]); v.push_back(b.qn[i]); }
}
struct VecHash {
    size_t operator()(const std::vector<int> &v) const {
        uint64_t h = 1469598103934665603ull;
        for (int x : v) { h ^= (uint64_t)(uint32_t)x; h *= 1099511628211ull; }
        return (size_t)h;
    }
};
constexpr size_t kPlanCacheMax = 16384;
}  // namespace

// Plans hold device buffers uploaded on their context's stream, so each
// context keeps its own cache and no plan is read on another stream.
struct PlanCache {
    std::unordered_map<std::vector<int>, std::shared_ptr<HeffPlan>, VecHash> map;
};

void clear_plan_cache() {
    delete ctx().plans;
    ctx().plans = nullptr;
}

void plan_stats(long long *built, double *ms) {
    *built = ctx().plans_built;
    *ms = ctx().plan_ms;
}

std::shared_ptr<HeffPlan> get_heff_plan(int nsite, const Meta &L, const Meta &psi, const Meta *W1, const Meta *W2,
                                        const Meta &R, int precision, int max_iter) {
    std::vector<int> key = {nsite, precision, max_iter};
    key_meta(key, &L);
    key_meta(key, &psi);
    key_meta(key, W1);
    key_meta(key, W2);
    key_meta(key, &R);
    Context &c = ctx();
    if (!c.plans) c.plans = new PlanCache;
    auto &cache = c.plans->map;
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    if (cache.size() >= kPlanCacheMax) cache.clear();
    const auto t0 = std::chrono::steady_clock::now();
    auto p = std::make_shared<HeffPlan>(plan_heff(nsite, L, psi, W1, W2, R, precision, max_iter));
    ++c.plans_built;
    c.plan_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    cache.emplace(std::move(key), p);
    return p;
}

// per-call intermediates of an H_eff application
struct HeffWork {
    DevBuf t1, t2, t3;
    explicit HeffWork(const HeffPlan &H) {
        t1 = DevBuf(std::max<int64_t>(1, H.p1.out.nelem) * sizeof(double2));
        if (H.nsite >= 1) t2 = DevBuf(std::max<int64_t>(1, H.m1.out.nelem) * sizeof(double2));
        if (H.nsite == 2) t3 = DevBuf(std::max<int64_t>(1, H.m2.out.nelem) * sizeof(double2));
    }
};

// out (Krylov layout) = scale * H_eff . v (Krylov layout)
void run_heff(const HeffPlan &H, HeffWork &w, const DTensor &L, const double2 *v, const DTensor *W1,
              const DTensor *W2, const DTensor &R, double2 *out, double scale, int precision, const int *skip,
              const KrylovState *st = nullptr, int k = -1) {
    // credit each launch with the reference flops of iteration k (all of the
    // product<> flops to the first GEMM of the pair; the second gets none)
    const double credit = (k >= 0 && k < (int)H.iter_flops.size()) ? H.iter_flops[k].gemm : -1.0;
    run_gemm(H.p1.gemm, L.data(), v, w.t1.as<double2>(), 1.0, precision, skip, st, k, credit);
    const double2 *last = w.t1.as<double2>();
    const int step = k >= 0 ? k : kAllSteps;
    if (H.nsite >= 1) {
        run_mix(H.m1.mix, last, W1->data(), w.t2.as<double2>(), skip, step, st, k);
        last = w.t2.as<double2>();
    }
    if (H.nsite == 2) {
        run_mix(H.m2.mix, last, W2->data(), w.t3.as<double2>(), skip, step, st, k);
        last = w.t3.as<double2>();
    }
    run_gemm(H.p2.gemm, last, R.data(), out, scale, precision, skip, st, k, credit >= 0.0 ? 0.0 : -1.0);
}

// scatter a tensor into a (superset) layout; blocks not present become zero
void scatter_into(const DTensor &src, const Meta &dst_meta, double2 *dst) {
    launch_zero(dst, dst_meta.nelem);
    std::vector<int64_t> desc;
    int nb = 0;
    for (auto &b : src.meta.blocks) {
        int k = dst_meta.find(b);
        KV_REQUIRE(k >= 0, KV_EINVAL, "internal: block missing from target layout");
        std::array<int64_t, 16> d{};
        d[0] = b.off;
        d[1] = dst_meta.blocks[k].off;
        d[2] = b.size;
        d[3] = src.meta.rank;
        for (int i = 0; i < src.meta.rank; ++i) { d[4 + i] = b.shape[i]; d[10 + i] = i; }
        desc.insert(desc.end(), d.begin(), d.end());
        ++nb;
    }
    launch_permute(src.data(), dst, desc, nb);
}

TensorP op_heff(int nsite, const DTensor &L, const DTensor &psi, const DTensor *W1, const DTensor *W2,
                const DTensor &R, double scale, int precision) {
    check_precision(precision);
    auto Hp = get_heff_plan(nsite, L.meta, psi.meta, W1 ? &W1->meta : nullptr, W2 ? &W2->meta : nullptr, R.meta,
                            precision, 1);
    const HeffPlan &H = *Hp;
    HeffWork w(H);
    DevBuf v(std::max<int64_t>(1, H.klayout.nelem) * sizeof(double2));
    scatter_into(psi, H.klayout, v.as<double2>());
    auto out = DTensor::make(H.klayout, false);
    run_heff(H, w, L, v.as<double2>(), W1, W2, R, out->data(), scale, precision, nullptr);
    return out;
}

// ------------------------------------------------------- local_krylov
TensorP op_lanczos(int nsite, const DTensor &L, const DTensor &psi, const DTensor *W1, const DTensor *W2,
                   const DTensor &R, double dt, int max_iter, double tol, bool reverse, int precision,
                   KrylovState *st_dev, std::vector<Flops> *per_iter, int *iters_out) {
    check_precision(precision);
    KV_REQUIRE(max_iter >= 2 && max_iter <= kMaxKrylov, KV_EINVAL, "max_iter must be in [2, 32]");
    KV_REQUIRE(tol < 1.0, KV_EINVAL, "Krylov tolerance must be < 1");
    auto Hp = get_heff_plan(nsite, L.meta, psi.meta, W1 ? &W1->meta : nullptr, W2 ? &W2->meta : nullptr, R.meta,
                            precision, max_iter);
    const HeffPlan &H = *Hp;
    HeffWork w(H);
    if (per_iter) *per_iter = H.iter_flops;
    // v_j lives on the first nl[j] elements of the layout; the vectors are packed
    KrylovLens nl{};
    for (int j = 0; j <= kMaxKrylov; ++j) nl.n[j] = H.prefix[std::min(j, H.napply)];
    const int64_t n = H.klayout.nelem;
    const int nvec = max_iter;  // V_0 .. V_{max_iter-1}
    std::vector<int64_t> voff(nvec + 1, 0);
    for (int j = 0; j < nvec; ++j) voff[j + 1] = voff[j] + nl.n[j];
    DevBuf Vbuf(std::max<int64_t>(1, voff[nvec]) * sizeof(double2));
    DevBuf hv(std::max<int64_t>(1, n) * sizeof(double2));
    DevBuf parts(2 * reduce_parts() * sizeof(double2));
    double2 *V = Vbuf.as<double2>();
    // psi's blocks are the layout's first blocks at the same offsets (both laid out in block order)
    KV_REQUIRE(psi.meta.nelem == nl.n[0], KV_EINVAL, "internal: Krylov layout does not start with psi");
    // The iterations are issued ahead of the device, and every kernel of an
    // iteration past the stop returns at once (skip).  Before issuing
    // iteration k the host waits for iteration k - kStopLag to finish and
    // stops if the recurrence had stopped by then, so at most kStopLag
    // iterations are issued in vain while the device stays kStopLag - 1
    // iterations ahead of the host.  No kernel of this context is running
    // here (the previous call on it synchronised), so the flag can be reset.
    constexpr int kStopLag = 2;
    Context &c = ctx();
    *reinterpret_cast<volatile int *>(c.stop_host) = 0;
    krylov_start(st_dev, psi.data(), V, nl.n[0], parts.as<double2>(), c.stop_dev);
    const int *skip = &st_dev->done;
    ++c.krylov_calls;
    for (int k = 0; k < max_iter - 1; ++k) {
        if (k >= kStopLag) {
            KV_CUDA(cudaEventSynchronize(c.iter_ev[k - kStopLag]));
            if (*reinterpret_cast<volatile int *>(c.stop_host)) break;
        }
        run_heff(H, w, L, V + voff[k], W1, W2, R, hv.as<double2>(), dt * 0.5, precision, skip, st_dev, k);
        ProfRec rec{};
        if (c.prof) {
            // algorithmic bytes, 16 B per element: overlap with v_{k-1} (hv,
            // v_{k-1} on its support), subtract it and overlap with v_k (hv, v_k;
            // v_{k-1} read and hv written on v_{k-1}'s support), subtract v_k
            // and take the norm (hv; v_k read and hv written on v_k's support),
            // normalise (hv read, v_{k+1} written)
            const double n_prev = k > 0 ? (double)nl.n[k - 1] : 0.0;
            rec = {prof_event(), prof_event(), 16.0 * (4 * n_prev + 4 * (double)nl.n[k] + 3 * (double)nl.n[k + 1]),
                   st_dev, k, kProfLanczos};
            KV_CUDA(cudaEventRecord(rec.a, c.stream));
        }
        krylov_step(st_dev, k, hv.as<double2>(), k > 0 ? V + voff[k - 1] : nullptr, V + voff[k], V + voff[k + 1], nl,
                    parts.as<double2>(), tol, max_iter, c.stop_dev);
        if (c.prof) {
            KV_CUDA(cudaEventRecord(rec.b, c.stream));
            c.prof_pending.push_back(rec);
        }
        KV_CUDA(cudaEventRecord(c.iter_ev[k], c.stream));
        ++c.krylov_issued;
    }
    std::vector<double2 *> ptrs(nvec);
    for (int i = 0; i < nvec; ++i) ptrs[i] = V + voff[i];
    DevBuf dptrs = upload_vec(ptrs);
    auto out = DTensor::make(H.klayout, false);
    krylov_finish(st_dev, dptrs.as<double2 *>(), out->data(), nl, reverse ? 1 : 0);
    // the result carries the blocks of v_0 .. v_{iters-1}, as the reference's
    // sum of Krylov vectors does: a prefix of the layout
    KrylovState h;
    KV_CUDA(cudaMemcpyAsync(&h, st_dev, sizeof(h), cudaMemcpyDeviceToHost, ctx().stream));
    KV_CUDA(cudaStreamSynchronize(ctx().stream));
    KV_REQUIRE(h.status == KV_OK, h.status, "non-finite norm in the Lanczos recurrence");
    KV_REQUIRE(h.iters >= 1 && h.iters <= max_iter, KV_EINVAL, "internal: Krylov dimension out of range");
    const int64_t keep = nl.n[h.iters - 1];
    size_t nb = 0;
    while (nb < out->meta.blocks.size() && out->meta.blocks[nb].off < keep) ++nb;
    out->meta.blocks.resize(nb);
    out->meta.layout();
    KV_REQUIRE(out->meta.nelem == keep, KV_EINVAL, "internal: Krylov prefix is not block aligned");
    if (iters_out) *iters_out = h.iters;
    c.krylov_used += h.iters;
    return out;
}

// ---------------------------------------------------------------- SVD
// mixed mode: FP32 singular values below this fraction of their sector's
// largest are treated as zero before ranking (a state dropped by this rule
// carries at most 1e-12 of the sector's weight).  FP32 values above it are
// only used to choose which columns get their value recomputed in FP64: an
// FP32 value that is rounding noise on an exact zero (up to ~1e-5 relative)
// comes back near zero from the FP64 rebuild and is dropped there.
constexpr double kMixedSvdFloor = 1e-6;
// mixed mode: the QR reduction stops once every remaining row of a sector is
// below this fraction of the sector's Frobenius norm (FP32 rounding level;
// the dropped part is below ~1e-7 sqrt(rows) of the sector's norm)
constexpr float kQrFloor = 1e-7f;

struct Micro {
    std::array<int, kMaxRank> shape{}, qn{};
    int pos = 0, len = 0;
    std::vector<int> idx;
};
struct Macro {
    int q = 0, len = 0, kept = 0;
    std::vector<Micro> subs;
};

// fill_block (holstein/svd.h:110-205): macro = total row (column) charge,
// micro = (shape, charges) of the row (column) legs, in first-appearance order
static void fill_side(std::vector<Macro> &info, int q, const BlockMeta &b, int lo, int hi, int k) {
    Micro m;
    int len = 1;
    for (int i = lo; i < hi; ++i) { m.shape[i - lo] = b.shape[i]; m.qn[i - lo] = b.qn[i]; len *= b.shape[i]; }
    for (auto &mac : info) {
        if (mac.q != q) continue;
        for (auto &s : mac.subs) {
            bool same = true;
            for (int i = 0; i < hi - lo; ++i) same = same && s.shape[i] == m.shape[i] && s.qn[i] == m.qn[i];
            if (same) { s.idx.push_back(k); return; }
        }
        m.pos = mac.len;
        m.len = len;
        m.idx = {k};
        mac.len += len;
        mac.subs.push_back(m);
        return;
    }
    Macro mac;
    mac.q = q;
    m.pos = 0;
    m.len = len;
    m.idx = {k};
    mac.len = len;
    mac.subs.push_back(m);
    info.push_back(mac);
}

// ---- SA-1TDVP helpers (util/allocation.h:232-256, holstein/svd.h:525-560),
// written as the reference writes them so the host draws and the synthetic
// spectrum agree with it value for value
static double quasi_gauss(double x, double bet) {
    double r = std::exp(-0.25 * bet * std::pow(x, 2.0)) * std::abs(0.25 * x / bet);
    r += (0.5 / bet - 0.25 * std::pow(x, 2.0)) * std::erfc(0.5 * std::pow(bet, 0.5) * std::abs(x)) * 0.5 *
         std::pow(3.1415926 / bet, 0.5);
    r *= std::exp(-0.25 * bet * std::pow(x, 2.0)) * 4.0 * bet * std::pow(bet / 3.1415926, 0.5);
    return r;
}

// the root of quasi_gauss(x) = y on [0, 2] by bisection to 1e-8
static double inv_quasi_gauss(double y, double bet) {
    double hi = 2.0, lo = 0.0, mid = 0.0;
    while (hi - lo > 1e-8) {
        mid = 0.5 * (hi + lo);
        if ((quasi_gauss(mid, bet) - y) * (quasi_gauss(lo, bet) - y) < 0) hi = mid;
        else lo = mid;
    }
    return mid;
}

// States the SA split adds: the descending spectrum's tail continued by
// s' = 10^(+-r) s_last^2 / s_prev with r = inv_quasi_gauss(u, beta), u uniform
// in [0, 1) from a fresh generator per value, the sign alternating, clamped
// to be non-increasing, until a value reaches thres or the spectrum max_dim;
// only spectra with 5 < n < max_dim values grow.
static int sa_added(const std::vector<double> &desc, int max_dim, double thres, double beta, std::mt19937 &seeds) {
    const int n = (int)desc.size();
    if (n < 2 || !(n < max_dim && n > 5)) return 0;
    std::vector<double> t = {desc[n - 2], desc[n - 1]};
    int added = 0;
    for (int i = n; i < max_dim; ++i) {
        std::mt19937 gen{(std::mt19937::result_type)(unsigned int)seeds()};
        std::uniform_real_distribution<double> u(0, 1);
        const double r = inv_quasi_gauss(u(gen), beta);
        const double f = (i + n) % 2 == 0 ? std::pow(10, r) : std::pow(10, -1.0 * r);
        t.push_back(f * std::pow(t[t.size() - 1], 2.0) / t[t.size() - 2]);
        if (t.back() <= thres) {
            t.pop_back();
            break;
        }
        if (t.back() > t[t.size() - 2]) t.back() = t[t.size() - 2];
        added = (int)t.size() - 2;
    }
    return added;
}

SvdOut op_svd(const DTensor &A, int r1, bool l2r, double thres, int max_dim, int precision, SaParams *sa) {
    const Meta &M = A.meta;
    KV_REQUIRE(r1 >= 1 && r1 < M.rank, KV_EINVAL, "svd split must be in [1, rank-1]");
    KV_REQUIRE(max_dim >= 1, KV_EINVAL, "max_dim must be >= 1");
    std::vector<Macro> rows, cols;
    for (int k = 0; k < (int)M.blocks.size(); ++k) {
        const BlockMeta &b = M.blocks[k];
        int qr = 0, qc = 0;
        for (int i = 0; i < r1; ++i) qr += b.qn[i] * M.dirs[i];
        for (int i = r1; i < M.rank; ++i) qc += b.qn[i] * M.dirs[i];
        fill_side(rows, qr, b, 0, r1, k);
        fill_side(cols, qc, b, r1, M.rank, k);
    }
    SvdPlan P;
    std::vector<std::pair<int, int>> sec_rc;
    const bool mixed = svd_mixed(precision) && !sa;
    for (int ri = 0; ri < (int)rows.size(); ++ri)
        for (int ci = 0; ci < (int)cols.size(); ++ci) {
            if (rows[ri].q + cols[ci].q != 0) continue;
            SvdSector s{};
            s.m = rows[ri].len;
            s.n = cols[ci].len;
            // FP64: tall T with accumulated V.  Mixed: T's columns are the
            // singular vectors the polish needs (right ones for L->R, left
            // ones for R->L), so no rotations are accumulated; T may be wide.
            s.transposed = mixed ? (l2r ? 1 : 0) : (s.m < s.n ? 1 : 0);
            s.p = s.transposed ? s.n : s.m;
            s.q = s.transposed ? s.m : s.n;
            s.t_off = P.t_elems;
            s.v_off = P.v_elems;
            s.s_off = P.s_elems;
            P.t_elems += (int64_t)s.p * s.q;
            if (!mixed) P.v_elems += (int64_t)s.q * s.q;
            P.s_elems += s.q;
            P.max_q = std::max(P.max_q, s.q);
            rows[ri].kept = std::min(s.m, s.n);
            cols[ci].kept = std::min(s.m, s.n);
            const int sid = (int)P.secs.size();
            for (auto &ra : rows[ri].subs)
                for (auto &ca : cols[ci].subs)
                    for (int x : ra.idx)
                        for (int y : ca.idx)
                            if (x == y) P.gathers.push_back({M.blocks[x].off, sid, ra.pos, ca.pos, ra.len, ca.len});
            P.secs.push_back(s);
            sec_rc.push_back({ri, ci});
        }
    P.upload();
    const size_t cb = mixed ? sizeof(float2) : sizeof(double2);
    DevBuf T(std::max<int64_t>(1, P.t_elems) * sizeof(double2));
    DevBuf Us(std::max<int64_t>(1, P.t_elems) * cb), V(std::max<int64_t>(1, P.v_elems) * cb);
    DevBuf Vs(std::max<int64_t>(1, P.v_elems) * cb);
    DevBuf S(std::max<int64_t>(1, P.s_elems) * sizeof(double));
    DevBuf status(std::max<size_t>(1, 2 * P.secs.size()) * sizeof(int));  // sweeps, then QR ranks
    svd_gather(P, A.data(), T.as<double2>());
    bool qr_ranks = false;
    if (mixed) {
        // tolerance 1e-5 on the columns' cosines: a residual c_ij <= 1e-5 s_i s_j
        // tilts the kept subspace by ~1e-5 s_j / s_i, and the FP64 polish
        // rebuilds the kept factor exactly from that subspace.  Sectors that
        // fit shared memory are first reduced to their numerical rank (rows
        // below 1e-7 ||T||_F dropped by a pivoted Householder QR).
        qr_ranks = svd_qrjacobi_f32(P, T.as<double2>(), Us.as<float2>(), S.as<double>(), status.as<int>(),
                                    status.as<int>() + P.secs.size(), 60, 1e-5f, kQrFloor);
        if (!qr_ranks) {
            // sectors beyond shared memory: the same QR reduction on an
            // L2-resident workspace, then the global-memory Jacobi on each
            // sector's rank-r factor (its columns beyond r are zero)
            DevBuf T32(std::max<int64_t>(1, P.t_elems) * cb);
            int *rk_dev = status.as<int>() + P.secs.size();
            svd_qr_global(P, T.as<double2>(), T32.as<float2>(), rk_dev, kQrFloor);
            std::vector<int> rk(P.secs.size());
            KV_CUDA(cudaMemcpyAsync(rk.data(), rk_dev, rk.size() * sizeof(int), cudaMemcpyDeviceToHost,
                                    ctx().stream));
            KV_CUDA(cudaStreamSynchronize(ctx().stream));
            SvdPlan Pr;
            Pr.secs = P.secs;
            for (size_t i = 0; i < rk.size(); ++i) Pr.secs[i].q = std::max(0, std::min(rk[i], P.secs[i].q));
            Pr.t_elems = P.t_elems;
            Pr.upload();
            svd_jacobi_f32(Pr, nullptr, T32.as<float2>(), status.as<int>(), 60, 1e-5f);
            svd_finalize_f32(P, T32.as<float2>(), Us.as<float2>(), S.as<double>());
            qr_ranks = true;
        }
    } else {
        svd_jacobi(P, T.as<double2>(), V.as<double2>(), status.as<int>(), 60, 1e-15);
        svd_finalize(P, T.as<double2>(), V.as<double2>(), Us.as<double2>(), Vs.as<double2>(), S.as<double>());
    }
    std::vector<double> sv(P.s_elems);
    std::vector<int> st(2 * P.secs.size());
    if (P.s_elems)
        KV_CUDA(cudaMemcpyAsync(sv.data(), S.p, P.s_elems * sizeof(double), cudaMemcpyDeviceToHost, ctx().stream));
    if (!st.empty())
        KV_CUDA(cudaMemcpyAsync(st.data(), status.p, st.size() * sizeof(int), cudaMemcpyDeviceToHost, ctx().stream));
    KV_CUDA(cudaStreamSynchronize(ctx().stream));
    {
        auto &c = ctx();
        for (size_t i = 0; i < P.secs.size(); ++i) {
            KV_REQUIRE(st[i] >= 0, KV_ETIMEOUT, "Jacobi SVD did not converge within the sweep limit");
            c.svd.sectors += 1;
            c.svd.columns += P.secs[i].q;
            c.svd.rank += qr_ranks ? st[P.secs.size() + i] : std::min(P.secs[i].p, P.secs[i].q);
            c.svd.sweeps += st[i];
            c.svd.max_sweeps = std::max(c.svd.max_sweeps, st[i]);
        }
    }
    for (double x : sv) KV_REQUIRE(std::isfinite(x), KV_ENONFINITE, "non-finite singular value");
    if (mixed) {
        // below kMixedSvdFloor of the sector's largest: zero
        for (auto &sc : P.secs) {
            const double smax = sc.q > 0 ? sv[sc.s_off] : 0.0;
            for (int i = 0; i < sc.q; ++i)
                if (sv[sc.s_off + i] <= kMixedSvdFloor * smax) sv[sc.s_off + i] = 0.0;
        }
    }
    const int nsec = (int)P.secs.size();
    // global ordering and truncation, holstein/svd.h:350-388: all singular
    // values sorted descending, dropped from the tail while i >= max_dim or
    // s <= thres (never the first); returns the kept count per sector
    auto truncate = [&](const std::vector<double> &vals, std::vector<double> *kept_vals, int *total) {
        std::vector<std::pair<int, double>> collect;
        std::vector<int> cnt(nsec, 0);
        for (int s_ = 0; s_ < nsec; ++s_) {
            // min(m, n) singular values (a wide mixed-mode T has q - p surplus zero columns, sorted last)
            cnt[s_] = std::min(P.secs[s_].m, P.secs[s_].n);
            for (int i = 0; i < cnt[s_]; ++i) collect.push_back({s_, vals[P.secs[s_].s_off + i]});
        }
        std::sort(collect.begin(), collect.end(),
                  [](const std::pair<int, double> &a, const std::pair<int, double> &b) { return a.second > b.second; });
        if (total) *total = (int)collect.size();
        for (int i = (int)collect.size() - 1; i > 0; --i) {
            if (!(i >= max_dim || collect[i].second <= thres)) break;
            --cnt[collect[i].first];
            collect.pop_back();
        }
        if (kept_vals)
            for (auto &c : collect) kept_vals->push_back(c.second);
        return cnt;
    };
    SvdOut out;
    std::vector<int> kfin = truncate(sv, &out.kept_s, &out.n_total);
    std::vector<int> ext(nsec, 0);  // SA: states added per sector
    if (sa) {
        // sa_svd_impl keeps min(m, n) states per sector; the added states go
        // to the sectors in order, each taking what its kept side has room for
        std::vector<double> all;
        for (int s_ = 0; s_ < nsec; ++s_) {
            const SvdSector &sc = P.secs[s_];
            kfin[s_] = std::min(sc.m, sc.n);
            for (int i = 0; i < kfin[s_]; ++i) all.push_back(sv[sc.s_off + i]);
        }
        std::sort(all.begin(), all.end(), std::greater<double>());
        out.kept_s = all;
        out.n_total = (int)all.size();
        int add = sa_added(all, max_dim, thres, sa->beta, *sa->seeds);
        sa->added = 0;
        for (int s_ = 0; s_ < nsec && add > 0; ++s_) {
            const SvdSector &sc = P.secs[s_];
            const int room = (l2r ? sc.m : sc.n) - kfin[s_];
            if (kfin[s_] <= 0 || room <= 0) continue;
            ext[s_] = std::min(add, room);
            add -= ext[s_];
            sa->added += ext[s_];
        }
    }
    // ---- mixed mode, part 1: FP64 rebuild of the candidate columns.  The
    // kept factor is rebuilt in FP64 from the sector matrix and the FP32
    // singular vectors of the other side,
    //   L->R: X = A_s V S^-1   R->L: X = A_s^H U S^-1,
    // over each sector's FP32-kept columns plus the candidates within 10%
    // below the cutoff.  The columns of X are orthonormal up to the FP32
    // error of W, so s_j |x_j| is column j's singular value with that error
    // entering only at second order -- accurate to FP64 where the FP32 value
    // is not (its error is ~1e-7 of the sector's largest).  The truncation is
    // redone with those values; the kept columns are a prefix of X.
    const int side = l2r ? 0 : 1;  // which factor is kept orthonormal
    std::vector<int> kc(nsec, 0);  // columns rebuilt per sector
    std::vector<SvdPolish> pol;
    std::vector<int> pol_of_sector(nsec, -1);
    DevBuf X, Gm, Wb, cst, cdiag;
    // the rebuild's FP64 products are small: 16 x 16 tiles spread them over more SMs
    const int tm = 16, tn = 16;
    auto add_gemm = [&](GemmPlan &g, int64_t c_off, int M, int N, GemmSeg seg) {
        const int sb = (int)g.segs.size();
        g.tile_m = tm;
        g.tile_n = tn;
        g.segs.push_back(seg);
        for (int m0 = 0; m0 < M; m0 += tm)
            for (int n0 = 0; n0 < N; n0 += tn) g.tiles.push_back({c_off, N, M, N, m0, n0, sb, sb + 1});
    };
    auto polish_pass = [&](const std::vector<SvdPolish> &pl_list, const DevBuf &dp, double shift) {
        GemmPlan gram;
        int kmax = 1;
        for (auto &pl : pl_list) {
            add_gemm(gram, pl.g_off, pl.k, pl.k, GemmSeg{pl.x_off, pl.x_off, pl.rows, pl.ldx, pl.ldx, 1, 0});
            kmax = std::max(kmax, pl.k);
        }
        gram.upload();
        std::vector<int> item_pol, item_row0;
        for (size_t i = 0; i < pl_list.size(); ++i)
            for (int r0 = 0; r0 < pl_list[i].rows; r0 += kTrsmRows) {
                item_pol.push_back((int)i);
                item_row0.push_back(r0);
            }
        launch_gemm_fp64(gram, X.as<double2>(), X.as<double2>(), Gm.as<double2>(), 1.0, nullptr);
        svd_chol(dp, (int)pl_list.size(), Gm.as<double2>(), cst.as<int>(), cdiag.as<double>(), shift);
        svd_trsm(dp, item_pol, item_row0, Gm.as<double2>(), X.as<double2>(), kmax);
    };
    if (mixed) {
        const double s_cut = out.kept_s.empty() ? 0.0 : out.kept_s.back();
        int64_t x_elems = 0, g_elems = 0, w_elems = 0;
        for (int s_ = 0; s_ < nsec; ++s_) {
            const SvdSector &sc = P.secs[s_];
            const int ns = std::min(sc.m, sc.n);
            int k = kfin[s_];
            while (k < ns && k < kfin[s_] + 64 && sv[sc.s_off + k] > 0.0 && sv[sc.s_off + k] >= 0.9 * s_cut) ++k;
            kc[s_] = k;
            if (k <= 0) continue;
            const int xr = side == 0 ? sc.m : sc.n;  // rows of the kept factor
            const int wr = side == 0 ? sc.n : sc.m;  // rows of the other side's vectors
            pol_of_sector[s_] = (int)pol.size();
            pol.push_back({x_elems, g_elems, w_elems, s_, xr, k, k});
            x_elems += (int64_t)xr * k;
            g_elems += (int64_t)k * k;
            w_elems += (int64_t)wr * k;
        }
        DevBuf dpol = upload_vec(pol);
        X = DevBuf(std::max<int64_t>(1, x_elems) * sizeof(double2));
        Gm = DevBuf(std::max<int64_t>(1, g_elems) * sizeof(double2));
        Wb = DevBuf(std::max<int64_t>(1, w_elems) * sizeof(double2));
        cst = DevBuf(std::max<size_t>(1, pol.size()) * sizeof(int));
        cdiag = DevBuf(std::max<size_t>(1, pol.size()) * sizeof(double));
        KV_CUDA(cudaMemsetAsync(cst.p, 0, std::max<size_t>(1, pol.size()) * sizeof(int), ctx().stream));
        svd_extract(dpol, (int)pol.size(), P, Us.as<float2>(), S.as<double>(), Wb.as<double2>());
        // X = A_s W (L->R, K = n) or A_s^H W (R->L, K = m), A_s from T:
        // A_s[i, j] = T[i + j p] (T = A_s) or conj(T[j + i p]) (T = A_s^H)
        GemmPlan build;
        for (auto &pl : pol) {
            const SvdSector &sc = P.secs[pl.sector];
            if (side == 0)
                add_gemm(build, pl.x_off, sc.m, pl.k,
                         GemmSeg{sc.t_off, pl.w_off, sc.n, sc.p, pl.k, sc.transposed ? 3 : 2, 0});
            else
                add_gemm(build, pl.x_off, sc.n, pl.k,
                         GemmSeg{sc.t_off, pl.w_off, sc.m, sc.p, pl.k, sc.transposed ? 2 : 3, 0});
        }
        build.upload();
        launch_gemm_fp64(build, T.as<double2>(), Wb.as<double2>(), X.as<double2>(), 1.0, nullptr);
        // refined singular values: x_j = A w_j / s~_j, so s_j = s~_j |x_j|.  W's
        // FP32 error enters |A w_j| only at second order (the columns of X are
        // orthogonal to that order), which is what the truncation needs.
        svd_col_norm2(dpol, (int)pol.size(), X.as<double2>(), Gm.as<double2>());
        std::vector<std::vector<double2>> diag(pol.size());
        for (size_t i = 0; i < pol.size(); ++i) {
            diag[i].resize(pol[i].k);
            KV_CUDA(cudaMemcpyAsync(diag[i].data(), Gm.as<double2>() + pol[i].g_off, pol[i].k * sizeof(double2),
                                    cudaMemcpyDeviceToHost, ctx().stream));
        }
        KV_CUDA(cudaStreamSynchronize(ctx().stream));
        std::vector<double> svr = sv;
        for (size_t i = 0; i < pol.size(); ++i) {
            const SvdSector &sc = P.secs[pol[i].sector];
            for (int j = 0; j < pol[i].k; ++j) svr[sc.s_off + j] = sv[sc.s_off + j] * std::sqrt(diag[i][j].x);
        }
        out.kept_s.clear();
        kfin = truncate(svr, nullptr, nullptr);
        for (int s_ = 0; s_ < nsec; ++s_) {
            kfin[s_] = std::min(kfin[s_], kc[s_]);
            for (int j = 0; j < kfin[s_]; ++j) out.kept_s.push_back(svr[P.secs[s_].s_off + j]);
        }
        std::sort(out.kept_s.begin(), out.kept_s.end(), std::greater<double>());
    }
    out.n_kept = 0;
    for (int s_ = 0; s_ < nsec; ++s_) {
        rows[sec_rc[s_].first].kept = kfin[s_] + ext[s_];
        cols[sec_rc[s_].second].kept = kfin[s_] + ext[s_];
        out.n_kept += kfin[s_] + ext[s_];
    }
    // redistribution, holstein/svd.h:405-428 with LeftDir = -1
    Meta mu, mv;
    mu.rank = r1 + 1;
    mv.rank = M.rank - r1 + 1;
    for (int i = 0; i < r1; ++i) mu.dirs[i] = M.dirs[i];
    mu.dirs[r1] = -1;
    mv.dirs[0] = 1;
    for (int i = r1; i < M.rank; ++i) mv.dirs[i - r1 + 1] = M.dirs[i];
    struct Pending { int sector, side, pos, len, kept; };
    std::vector<Pending> pu, pv;
    for (int s_ = 0; s_ < nsec; ++s_) {
        Macro &rw = rows[sec_rc[s_].first];
        Macro &cl = cols[sec_rc[s_].second];
        if (rw.kept <= 0 || cl.kept <= 0) continue;
        for (auto &ra : rw.subs) {
            BlockMeta b;
            for (int i = 0; i < r1; ++i) { b.shape[i] = ra.shape[i]; b.qn[i] = ra.qn[i]; }
            b.shape[r1] = rw.kept;
            b.qn[r1] = rw.q;
            mu.blocks.push_back(b);
            pu.push_back({s_, 0, ra.pos, ra.len, rw.kept});
        }
        for (auto &ca : cl.subs) {
            BlockMeta b;
            b.shape[0] = cl.kept;
            b.qn[0] = -cl.q;
            for (int i = 0; i < M.rank - r1; ++i) { b.shape[i + 1] = ca.shape[i]; b.qn[i + 1] = ca.qn[i]; }
            mv.blocks.push_back(b);
            pv.push_back({s_, 1, ca.pos, ca.len, cl.kept});
        }
    }
    const bool extended = sa && sa->added > 0;
    out.U = DTensor::make(mu, extended);  // the added states' other side stays zero
    out.V = DTensor::make(mv, extended);
    if (!mixed) {
        std::vector<SvdScatter> su, svs;
        for (size_t i = 0; i < pu.size(); ++i)
            su.push_back({out.U->meta.blocks[i].off, pu[i].sector, 0, pu[i].pos, pu[i].len, kfin[pu[i].sector],
                          l2r ? 0 : 1, pu[i].kept});
        for (size_t i = 0; i < pv.size(); ++i)
            svs.push_back({out.V->meta.blocks[i].off, pv[i].sector, 1, pv[i].pos, pv[i].len, kfin[pv[i].sector],
                           l2r ? 1 : 0, pv[i].kept});
        svd_scatter(su, P, Us.as<double2>(), Vs.as<double2>(), S.as<double>(), out.U->data());
        svd_scatter(svs, P, Us.as<double2>(), Vs.as<double2>(), S.as<double>(), out.V->data());
        if (!extended) return out;
        // ---- SA: the new directions of the kept side (gs_ortho,
        // util/allocation.h:260-320).  Each new vector's entries are drawn
        // uniform(-1, 1) (real) from a fresh generator seeded by the stream;
        // X = (I - B B^H) R twice and a Cholesky-QR twice give the vectors the
        // reference's one-at-a-time Gram-Schmidt gives (the Q factor of [B R]
        // beyond B), to rounding.
        std::vector<SaSector> sas;
        std::vector<int64_t> c_off;
        std::vector<int64_t> x_of_sector(nsec, -1);
        int64_t b_elems = 0, x_elems = 0, c_elems = 0;
        for (int s_ = 0; s_ < nsec; ++s_) {
            if (ext[s_] <= 0) continue;
            const SvdSector &sc = P.secs[s_];
            const int n = l2r ? sc.m : sc.n;
            sas.push_back({b_elems, x_elems, s_, l2r ? 0 : 1, n, kfin[s_], ext[s_]});
            c_off.push_back(c_elems);
            x_of_sector[s_] = x_elems;
            b_elems += (int64_t)n * kfin[s_];
            x_elems += (int64_t)n * ext[s_];
            c_elems += (int64_t)kfin[s_] * ext[s_];
        }
        std::vector<double2> xr(x_elems);
        for (auto &a : sas)
            for (int c = 0; c < a.ext; ++c) {
                std::mt19937 gen((std::mt19937::result_type)(unsigned int)(*sa->seeds)());
                std::uniform_real_distribution<double> dis(-1, 1);
                for (int r = 0; r < a.n; ++r) xr[a.x_off + (int64_t)r * a.ext + c] = make_double2(dis(gen), 0.0);
            }
        DevBuf Bd(std::max<int64_t>(1, b_elems) * sizeof(double2)), Cb(std::max<int64_t>(1, c_elems) * sizeof(double2));
        DevBuf Pb(std::max<int64_t>(1, x_elems) * sizeof(double2));
        X = DevBuf(std::max<int64_t>(1, x_elems) * sizeof(double2));
        upload_bytes(X.p, xr.data(), xr.size() * sizeof(double2));
        sa_basis(sas, P, Us.as<double2>(), Vs.as<double2>(), Bd.as<double2>());
        GemmPlan proj, back;  // C = B^H X, P = B C
        std::vector<SvdPolish> pl;
        int64_t g_elems = 0;
        for (size_t i = 0; i < sas.size(); ++i) {
            const SaSector &a = sas[i];
            add_gemm(proj, c_off[i], a.kept, a.ext, GemmSeg{a.b_off, a.x_off, a.n, a.kept, a.ext, 1, 0});
            add_gemm(back, a.x_off, a.n, a.ext, GemmSeg{a.b_off, c_off[i], a.kept, a.kept, a.ext, 0, 0});
            pl.push_back({a.x_off, g_elems, 0, a.sector, a.n, a.ext, a.ext});
            g_elems += (int64_t)a.ext * a.ext;
        }
        proj.upload();
        back.upload();
        for (int pass = 0; pass < 2; ++pass) {
            launch_gemm_fp64(proj, Bd.as<double2>(), X.as<double2>(), Cb.as<double2>(), 1.0, nullptr);
            launch_gemm_fp64(back, Bd.as<double2>(), Cb.as<double2>(), Pb.as<double2>(), 1.0, nullptr);
            sa_subtract(X.as<double2>(), Pb.as<double2>(), x_elems);
        }
        Gm = DevBuf(std::max<int64_t>(1, g_elems) * sizeof(double2));
        cst = DevBuf(std::max<size_t>(1, pl.size()) * sizeof(int));
        cdiag = DevBuf(std::max<size_t>(1, pl.size()) * sizeof(double));
        KV_CUDA(cudaMemsetAsync(cst.p, 0, std::max<size_t>(1, pl.size()) * sizeof(int), ctx().stream));
        DevBuf dpl = upload_vec(pl);
        polish_pass(pl, dpl, 0.0);
        polish_pass(pl, dpl, 0.0);
        std::vector<SaOut> so;
        if (l2r) {
            for (size_t i = 0; i < pu.size(); ++i)
                if (ext[pu[i].sector] > 0)
                    so.push_back({out.U->meta.blocks[i].off, x_of_sector[pu[i].sector], 0, pu[i].pos, pu[i].len,
                                  kfin[pu[i].sector], ext[pu[i].sector]});
        } else {
            for (size_t i = 0; i < pv.size(); ++i)
                if (ext[pv[i].sector] > 0)
                    so.push_back({out.V->meta.blocks[i].off, x_of_sector[pv[i].sector], 1, pv[i].pos, pv[i].len,
                                  kfin[pv[i].sector], ext[pv[i].sector]});
        }
        sa_scatter(so, X.as<double2>(), l2r ? out.U->data() : out.V->data());
        return out;
    }
    // ---- mixed mode, part 2: the kept prefix of each sector's X (row stride
    // kc), one Cholesky-QR pass for FP64 orthonormality (X's condition number
    // is 1 up to the FP32 error of W, so one pass reaches FP64 rounding), and
    // the other factor as the exact projection (Y = X^H A_s, or A_s X).  With
    // no truncation the factorisation is exact to FP64 rounding; the FP32
    // error only enters the choice of directions.
    std::vector<SvdPolish> pol2;
    std::vector<int> pol2_of_sector(nsec, -1);
    std::vector<int64_t> y_off(nsec, 0);
    int64_t y_elems = 0;
    for (auto pl : pol) {
        const int s_ = pl.sector;
        if (kfin[s_] <= 0) continue;
        const SvdSector &sc = P.secs[s_];
        pl.k = kfin[s_];
        pol2_of_sector[s_] = (int)pol2.size();
        pol2.push_back(pl);
        y_off[s_] = y_elems;
        y_elems += (int64_t)pl.k * (side == 0 ? sc.n : sc.m);
    }
    DevBuf dpol2 = upload_vec(pol2);
    if (!pol2.empty()) polish_pass(pol2, dpol2, 0.0);
    DevBuf Y(std::max<int64_t>(1, y_elems) * sizeof(double2));
    GemmPlan proj;
    for (auto &pl : pol2) {
        const SvdSector &sc = P.secs[pl.sector];
        const int64_t tof = sc.t_off;
        if (side == 0) {
            // Y = X^H A_s (k x n)
            add_gemm(proj, y_off[pl.sector], pl.k, sc.n,
                     GemmSeg{pl.x_off, tof, sc.m, pl.ldx, sc.p, 1, sc.transposed ? 3 : 1});
        } else {
            // Lef = A_s X (m x k)
            add_gemm(proj, y_off[pl.sector], sc.m, pl.k,
                     GemmSeg{tof, pl.x_off, sc.n, sc.p, pl.ldx, sc.transposed ? 3 : 2, 0});
        }
    }
    proj.upload();
    if (side == 0) launch_gemm_fp64(proj, X.as<double2>(), T.as<double2>(), Y.as<double2>(), 1.0, nullptr);
    else launch_gemm_fp64(proj, T.as<double2>(), X.as<double2>(), Y.as<double2>(), 1.0, nullptr);
    std::vector<SvdDense> du, dv;
    for (size_t i = 0; i < pu.size(); ++i) {
        const int s_ = pu[i].sector;
        const SvdPolish &pl = pol2[pol2_of_sector[s_]];
        if (side == 0) du.push_back({out.U->meta.blocks[i].off, pl.x_off, 0, pu[i].pos, pu[i].len, pl.k, pl.ldx, 0});
        else du.push_back({out.U->meta.blocks[i].off, y_off[s_], 0, pu[i].pos, pu[i].len, pl.k, pl.k, 0});
    }
    for (size_t i = 0; i < pv.size(); ++i) {
        const int s_ = pv[i].sector;
        const SvdPolish &pl = pol2[pol2_of_sector[s_]];
        if (side == 0)
            dv.push_back({out.V->meta.blocks[i].off, y_off[s_], 1, pv[i].pos, pv[i].len, pl.k, P.secs[s_].n, 0});
        else dv.push_back({out.V->meta.blocks[i].off, pl.x_off, 1, pv[i].pos, pv[i].len, pl.k, pl.ldx, 1});
    }
    svd_scatter_dense(du, side == 0 ? X.as<double2>() : Y.as<double2>(), out.U->data());
    svd_scatter_dense(dv, side == 0 ? Y.as<double2>() : X.as<double2>(), out.V->data());
    std::vector<int> ch(pol.size());
    std::vector<double> chd(pol.size());
    if (!ch.empty()) {
        KV_CUDA(cudaMemcpyAsync(ch.data(), cst.p, ch.size() * sizeof(int), cudaMemcpyDeviceToHost, ctx().stream));
        KV_CUDA(cudaMemcpyAsync(chd.data(), cdiag.p, chd.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                ctx().stream));
        KV_CUDA(cudaStreamSynchronize(ctx().stream));
        for (size_t i = 0; i < ch.size(); ++i) {
            if (ch[i] == 0) continue;
            const SvdSector &sc = P.secs[pol[i].sector];
            std::string msg = "Cholesky re-orthonormalisation failed: sector m=" + std::to_string(sc.m) +
                              " n=" + std::to_string(sc.n) + " kept=" + std::to_string(pol[i].k) +
                              " transposed=" + std::to_string(sc.transposed) + " l2r=" + std::to_string(l2r) +
                              " pivot=" + std::to_string(ch[i] - 1) + " value=" + std::to_string(chd[i]) + " s=[";
            for (int j = 0; j < std::min(sc.q, 12); ++j) msg += std::to_string(sv[sc.s_off + j]) + " ";
            throw Error(KV_ENONFINITE, msg + "]");
        }
    }
    return out;
}

// ---------------------------------------------------------- env update
TensorP op_permute(const DTensor &t, const std::vector<int> &ax) {
    Meta m;
    m.rank = t.meta.rank;
    for (int i = 0; i < m.rank; ++i) m.dirs[i] = t.meta.dirs[ax[i]];
    for (auto &b : t.meta.blocks) {
        BlockMeta o;
        for (int i = 0; i < m.rank; ++i) { o.shape[i] = b.shape[ax[i]]; o.qn[i] = b.qn[ax[i]]; }
        m.blocks.push_back(o);
    }
    auto out = DTensor::make(m, false);
    std::vector<int64_t> desc;
    for (size_t k = 0; k < t.meta.blocks.size(); ++k) {
        const BlockMeta &b = t.meta.blocks[k];
        std::array<int64_t, 16> d{};
        d[0] = b.off;
        d[1] = out->meta.blocks[k].off;
        d[2] = b.size;
        d[3] = m.rank;
        for (int i = 0; i < m.rank; ++i) { d[4 + i] = b.shape[i]; d[10 + i] = ax[i]; }
        desc.insert(desc.end(), d.begin(), d.end());
    }
    launch_permute(t.data(), out->data(), desc, (int)t.meta.blocks.size());
    return out;
}

// env_sweep(env, A, W, l2r) (holstein/product.h:488-503).  Wt, if given, is W
// already permuted {0,3,2,1} for the right-to-left case.
TensorP op_env(bool l2r, const DTensor &env, const DTensor &A, const DTensor &W, const DTensor *Wt, int precision,
               Flops *fl) {
    check_precision(precision);
    if (!l2r) {
        TensorP At = op_permute(A, {2, 1, 0});
        TensorP Wp;
        if (!Wt) { Wp = op_permute(W, {0, 3, 2, 1}); Wt = Wp.get(); }
        return op_env(true, env, *At, *Wt, nullptr, precision, fl);
    }
    ProductPlan P1 = plan_product(env.meta, A.meta, 1, KV_OP_N, KV_OP_N);
    auto t1 = DTensor::make(P1.out, false);
    build_tiles(P1, own_offsets(t1->meta), kTileM(precision), kTileN(precision));
    P1.gemm.upload();
    run_gemm(P1.gemm, env.data(), A.data(), t1->data(), 1.0, precision, nullptr);
    MixPlanFull M = plan_mix(t1->meta, W.meta, 1);
    M.mix.upload();
    auto t2 = DTensor::make(M.out, false);
    run_mix(M.mix, t1->data(), W.data(), t2->data(), nullptr, kAllSteps, nullptr, -1);
    ProductPlan P2 = plan_product(A.meta, t2->meta, 2, KV_OP_C, KV_OP_N);
    // A's blocks pair with every (reference-unmerged) copy of each mixed block
    const double f2 = ref_product_flops(A.meta, M.out, 2, KV_OP_C, KV_OP_N, nullptr, &M.mult);
    P2.gemm.ref_flops = f2;
    auto out = DTensor::make(P2.out, false);
    build_tiles(P2, own_offsets(out->meta), kTileM(precision), kTileN(precision));
    P2.gemm.upload();
    run_gemm(P2.gemm, A.data(), t2->data(), out->data(), 1.0, precision, nullptr);
    if (fl) {
        fl->gemm += P1.gemm.ref_flops + f2;
        fl->mix += M.ref_flops;
    }
    return out;
}

// =============================================================== TDVP
TensorP boundary_env(int dir0, int q) {
    Meta m;
    m.rank = 3;
    m.dirs = {dir0, -dir0, -dir0};
    BlockMeta b;
    b.shape = {1, 1, 1};
    b.qn = {q, 0, q};
    m.blocks.push_back(b);
    auto t = DTensor::make(m, false);
    double2 one = make_double2(1.0, 0.0);
    KV_CUDA(cudaMemcpyAsync(t->data(), &one, sizeof(one), cudaMemcpyHostToDevice, ctx().stream));
    KV_CUDA(cudaStreamSynchronize(ctx().stream));
    return t;
}

Tdvp::Tdvp(const std::vector<TensorP> &mps_in, const std::vector<TensorP> &mpo_in, double tol_svd_, double tol_exp_,
           int max_dim_, int max_iter_, double dt_, int precision_)
    : tol_svd(tol_svd_), tol_exp(tol_exp_), max_dim(max_dim_), max_iter(max_iter_), dt(dt_), precision(precision_) {
    check_precision(precision);
    KV_REQUIRE(mps_in.size() == mpo_in.size() && mps_in.size() >= 2, KV_EINVAL, "need >= 2 sites and one MPO tensor per site");
    for (auto &t : mps_in) mps.push_back(clone(*t));
    for (auto &t : mpo_in) { mpo.push_back(clone(*t)); mpo_t.push_back(op_permute(*t, {0, 3, 2, 1})); }
    KV_REQUIRE(!mps.back()->meta.blocks.empty(), KV_EINVAL, "empty last site tensor");
    kstate = DevBuf(sizeof(KrylovState) * kStateSlots);
    events.resize(2 * kMaxEvents);
    for (auto &e : events) KV_CUDA(cudaEventCreate(&e));
    for (auto &e : sweep_ev) KV_CUDA(cudaEventCreate(&e));
    init_envs();
}

// holstein/tdvp.h:303-316
void Tdvp::init_envs() {
    const int ns = (int)mps.size();
    envL = {boundary_env(1, 0)};
    envR = {boundary_env(-1, mps[ns - 1]->meta.blocks[0].qn[2])};
    for (int i = ns - 1; i > 0; --i)
        envR.push_back(op_env(false, *envR.back(), *mps[i], *mpo[i], mpo_t[i].get(), precision, nullptr));
    KV_CUDA(cudaStreamSynchronize(ctx().stream));
}

// holstein/tdvp.h:318-327: the MPO scaled by dt on its first site
// (Operator::operator*=, holstein/operator.h:66-70), one global_main.  The
// reference builds the sweep environments once, before this stage, so its
// next sweep contracts the new state with environments of the old one (a
// result that depends on the phases of singular vectors, i.e. on rounding);
// here they are rebuilt from the new state.
void Tdvp::global_krylov() {
    KV_REQUIRE(window_at < 0, KV_EINVAL, "the chain is inside a timed window; it cannot sweep");
    std::vector<TensorP> Hc = mpo;
    Hc[0] = op_scale(*mpo[0], dt);
    global_main(Hc, mps, max_iter, tol_exp, tol_svd, max_dim, precision);
    init_envs();
}

Tdvp::~Tdvp() {
    for (auto &e : events) cudaEventDestroy(e);
    for (auto &e : sweep_ev) cudaEventDestroy(e);
}

void Tdvp::mark(int module, bool start) {
    const auto now = std::chrono::steady_clock::now();
    if (start) host_t0 = now;
    else module_host_ms[module] += std::chrono::duration<double, std::milli>(now - host_t0).count();
    if (n_marks >= kMaxEvents) return;
    KV_CUDA(cudaEventRecord(events[2 * n_marks + (start ? 0 : 1)], ctx().stream));
    if (!start) { mark_module[n_marks] = module; ++n_marks; }
}

KrylovState *Tdvp::next_state() {
    KrylovState *s = kstate.as<KrylovState>() + (n_krylov % kStateSlots);
    ++n_krylov;
    return s;
}

TensorP Tdvp::krylov(int nsite, const DTensor &L, const DTensor &psi, const DTensor *W1, const DTensor *W2,
                     const DTensor &R, bool reverse, int module) {
    mark(module, true);
    std::vector<Flops> f;
    KrylovState *st = next_state();
    TensorP r = op_lanczos(nsite, L, psi, W1, W2, R, dt, max_iter, tol_exp, reverse, precision, st, &f);
    krylov_flops.push_back({st, f});
    mark(module, false);
    return r;
}

void Tdvp::begin_sweep() {
    n_marks = 0;
    n_krylov = 0;
    krylov_flops.clear();
    other = Flops{};
    for (auto &m : module_host_ms) m = 0.0;
    plan_stats(&plans0, &plan_ms0);
    sweep_t0 = std::chrono::steady_clock::now();
    KV_CUDA(cudaEventRecord(sweep_ev[0], ctx().stream));
}

static int tdvp_iters_of(const KrylovState *st, void *arg) {
    auto *p = static_cast<std::pair<const KrylovState *, const std::vector<KrylovState> *> *>(arg);
    size_t idx = (size_t)(st - p->first);
    return idx < p->second->size() ? (*p->second)[idx].iters : kMaxKrylov;
}

void Tdvp::end_sweep() {
    KV_CUDA(cudaEventRecord(sweep_ev[1], ctx().stream));
    KV_CUDA(cudaStreamSynchronize(ctx().stream));
    sweep_host_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - sweep_t0).count();
    {
        long long b = 0;
        double ms = 0.0;
        plan_stats(&b, &ms);
        plans_built = b - plans0;
        plan_ms = ms - plan_ms0;
    }
    float sms = 0.f;
    KV_CUDA(cudaEventElapsedTime(&sms, sweep_ev[0], sweep_ev[1]));
    sweep_ms = sms;
    {
        const int st = mixed_gemm_status();
        KV_REQUIRE(st == KV_OK, st, st == KV_ETIMEOUT ? "a tensor-core GEMM wait timed out"
                                                      : "a tensor-core GEMM operand holds Inf or NaN");
    }
    for (auto &m : module_ms) m = 0.0;
    for (int i = 0; i < n_marks; ++i) {
        float ms = 0.f;
        KV_CUDA(cudaEventElapsedTime(&ms, events[2 * i], events[2 * i + 1]));
        module_ms[mark_module[i]] += ms;
    }
    // Krylov iterations actually run, read back once per sweep
    KV_REQUIRE(n_krylov <= kStateSlots, KV_EINVAL, "internal: too many Krylov calls in one sweep");
    std::vector<KrylovState> host(std::min<int>(n_krylov, kStateSlots));
    if (!host.empty())
        KV_CUDA(cudaMemcpy(host.data(), kstate.p, host.size() * sizeof(KrylovState), cudaMemcpyDeviceToHost));
    double f = other.gemm + other.mix, fg = other.gemm;
    for (auto &kf : krylov_flops) {
        const KrylovState &h = host[kf.first - kstate.as<KrylovState>()];
        KV_REQUIRE(h.status == KV_OK, h.status, "non-finite norm in the Lanczos recurrence");
        for (int k = 0; k < h.iters && k < (int)kf.second.size(); ++k) {
            f += kf.second[k].gemm + kf.second[k].mix;
            fg += kf.second[k].gemm;
        }
    }
    last_ref_flops = f;
    last_gemm_flops = fg;
    std::pair<const KrylovState *, const std::vector<KrylovState> *> arg{kstate.as<KrylovState>(), &host};
    prof_resolve(tdvp_iters_of, &arg);
}

// TDVP::one_site (holstein/tdvp.h:78-141)
void Tdvp::one_site() {
    KV_REQUIRE(window_at < 0, KV_EINVAL, "the chain is inside a timed window; it cannot sweep");
    begin_sweep();
    const int ns = (int)mps.size();
    for (int i = 0; i < ns; ++i) {
        mps[i] = krylov(1, *envL.back(), *mps[i], mpo[i].get(), nullptr, *envR.back(), false, MOD_EVL1);
        if (i < ns - 1) {
            mark(MOD_SVD, true);
            SvdOut r = op_svd(*mps[i], 2, true, tol_svd, max_dim, precision);
            mark(MOD_SVD, false);
            mps[i] = r.U;
            mark(MOD_UPDATE, true);
            envL.push_back(op_env(true, *envL.back(), *mps[i], *mpo[i], nullptr, precision, &other));
            mark(MOD_UPDATE, false);
            TensorP c = krylov(0, *envL.back(), *r.V, nullptr, nullptr, *envR.back(), true, MOD_EVL0);
            mark(MOD_SWEEP, true);
            mps[i + 1] = op_product(*c, *mps[i + 1], 1, KV_OP_N, KV_OP_N, precision, &other);
            mark(MOD_SWEEP, false);
            envR.pop_back();
        }
    }
    for (int i = ns - 1; i >= 0; --i) {
        mps[i] = krylov(1, *envL.back(), *mps[i], mpo[i].get(), nullptr, *envR.back(), false, MOD_EVL1);
        if (i > 0) {
            mark(MOD_SVD, true);
            SvdOut r = op_svd(*mps[i], 1, false, tol_svd, max_dim, precision);
            mark(MOD_SVD, false);
            mps[i] = r.V;
            mark(MOD_UPDATE, true);
            envR.push_back(op_env(false, *envR.back(), *mps[i], *mpo[i], mpo_t[i].get(), precision, &other));
            mark(MOD_UPDATE, false);
            TensorP c = krylov(0, *envL.back(), *r.U, nullptr, nullptr, *envR.back(), true, MOD_EVL0);
            mark(MOD_SWEEP, true);
            mps[i - 1] = op_product(*mps[i - 1], *c, 1, KV_OP_N, KV_OP_N, precision, &other);
            mark(MOD_SWEEP, false);
            envL.pop_back();
        }
    }
    end_sweep();
}

void Tdvp::set_sa(const double *beta, int nbeta, unsigned long long seed) {
    KV_REQUIRE(nbeta >= 0 && (nbeta == 0 || beta), KV_EINVAL, "null width array");
    sa_beta.assign(beta, beta + nbeta);
    sa_seeds.seed((std::mt19937::result_type)seed);
}

// TDVP::sa_site (holstein/tdvp.h:230-294): one_site with the SA split in place
// of svd_impl; bond i (between sites i and i+1) takes width sa_beta[i]
void Tdvp::sa_site() {
    KV_REQUIRE(window_at < 0, KV_EINVAL, "the chain is inside a timed window; it cannot sweep");
    const int ns = (int)mps.size();
    KV_REQUIRE((int)sa_beta.size() >= ns - 1, KV_EINVAL, "SA-1TDVP needs one width per bond (kv_tdvp_set_sa)");
    begin_sweep();
    sa_added = 0;
    for (int i = 0; i < ns; ++i) {
        mps[i] = krylov(1, *envL.back(), *mps[i], mpo[i].get(), nullptr, *envR.back(), false, MOD_EVL1);
        if (i < ns - 1) {
            SaParams sp;
            sp.beta = sa_beta[i];
            sp.seeds = &sa_seeds;
            mark(MOD_SVD, true);
            SvdOut r = op_svd(*mps[i], 2, true, tol_svd, max_dim, precision, &sp);
            mark(MOD_SVD, false);
            sa_added += sp.added;
            mps[i] = r.U;
            mark(MOD_UPDATE, true);
            envL.push_back(op_env(true, *envL.back(), *mps[i], *mpo[i], nullptr, precision, &other));
            mark(MOD_UPDATE, false);
            TensorP c = krylov(0, *envL.back(), *r.V, nullptr, nullptr, *envR.back(), true, MOD_EVL0);
            mark(MOD_SWEEP, true);
            mps[i + 1] = op_product(*c, *mps[i + 1], 1, KV_OP_N, KV_OP_N, precision, &other);
            mark(MOD_SWEEP, false);
            envR.pop_back();
        }
    }
    for (int i = ns - 1; i >= 0; --i) {
        mps[i] = krylov(1, *envL.back(), *mps[i], mpo[i].get(), nullptr, *envR.back(), false, MOD_EVL1);
        if (i > 0) {
            SaParams sp;
            sp.beta = sa_beta[i - 1];
            sp.seeds = &sa_seeds;
            mark(MOD_SVD, true);
            SvdOut r = op_svd(*mps[i], 1, false, tol_svd, max_dim, precision, &sp);
            mark(MOD_SVD, false);
            sa_added += sp.added;
            mps[i] = r.V;
            mark(MOD_UPDATE, true);
            envR.push_back(op_env(false, *envR.back(), *mps[i], *mpo[i], mpo_t[i].get(), precision, &other));
            mark(MOD_UPDATE, false);
            TensorP c = krylov(0, *envL.back(), *r.U, nullptr, nullptr, *envR.back(), true, MOD_EVL0);
            mark(MOD_SWEEP, true);
            mps[i - 1] = op_product(*mps[i - 1], *c, 1, KV_OP_N, KV_OP_N, precision, &other);
            mark(MOD_SWEEP, false);
            envL.pop_back();
        }
    }
    end_sweep();
}

// one local update of TDVP::two_site's left-to-right pass at sites (i, i+1)
// (holstein/tdvp.h:150-185)
void Tdvp::two_site_lr(int i) {
    const int ns = (int)mps.size();
    mark(MOD_SWEEP, true);
    TensorP mm = op_product(*mps[i], *mps[i + 1], 1, KV_OP_N, KV_OP_N, precision, &other);
    mark(MOD_SWEEP, false);
    mm = krylov(2, *envL.back(), *mm, mpo[i].get(), mpo[i + 1].get(), *envR.back(), false, MOD_EVL2);
    mark(MOD_SVD, true);
    SvdOut r = op_svd(*mm, 2, true, tol_svd, max_dim, precision);
    mark(MOD_SVD, false);
    if (svs_on) svs.push_back(r.kept_s);
    if (i < ns - 2) {
        mps[i] = r.U;
        mark(MOD_UPDATE, true);
        envL.push_back(op_env(true, *envL.back(), *mps[i], *mpo[i], nullptr, precision, &other));
        mark(MOD_UPDATE, false);
        mps[i + 1] = krylov(1, *envL.back(), *r.V, mpo[i + 1].get(), nullptr, *envR.back(), true, MOD_EVL1);
        envR.pop_back();
    } else {
        mps[i] = r.U;
        mps[i + 1] = r.V;
    }
}

// A window of the two-site left-to-right pass: the pass is advanced (without
// the sweep statistics) to site i0, then n local updates are run as one timed
// "sweep" (module times, reference flops).  Chains too long to sweep in a
// benchmark run are measured this way; afterwards the handle is inside the
// pass and can only take further windows.
void Tdvp::window(int i0, int n) {
    const int ns = (int)mps.size();
    KV_REQUIRE(n >= 0 && i0 >= 0 && i0 + n <= ns - 2, KV_EINVAL, "window outside the two-site pass");
    if (window_at < 0) {
        envR.pop_back();
        window_at = 0;
    }
    KV_REQUIRE(i0 >= window_at, KV_EINVAL, "window behind the pass already advanced");
    for (; window_at < i0; ++window_at) {
        n_marks = 0;  // the advance keeps no statistics
        n_krylov = 0;
        krylov_flops.clear();
        two_site_lr(window_at);
    }
    KV_CUDA(cudaStreamSynchronize(ctx().stream));
    if (n == 0) return;
    begin_sweep();
    for (int i = i0; i < i0 + n; ++i) two_site_lr(i);
    window_at = i0 + n;
    end_sweep();
}

// TDVP::two_site (holstein/tdvp.h:144-227)
void Tdvp::two_site() {
    KV_REQUIRE(window_at < 0, KV_EINVAL, "the chain is inside a timed window; it cannot sweep");
    begin_sweep();
    const int ns = (int)mps.size();
    envR.pop_back();
    for (int i = 0; i < ns - 1; ++i) two_site_lr(i);
    for (int i = ns - 1; i > 0; --i) {
        mark(MOD_SWEEP, true);
        TensorP mm = op_product(*mps[i - 1], *mps[i], 1, KV_OP_N, KV_OP_N, precision, &other);
        mark(MOD_SWEEP, false);
        mm = krylov(2, *envL.back(), *mm, mpo[i - 1].get(), mpo[i].get(), *envR.back(), false, MOD_EVL2);
        mark(MOD_SVD, true);
        SvdOut r = op_svd(*mm, 2, false, tol_svd, max_dim, precision);
        mark(MOD_SVD, false);
        if (svs_on) svs.push_back(r.kept_s);
        if (i > 1) {
            mps[i] = r.V;
            mark(MOD_UPDATE, true);
            envR.push_back(op_env(false, *envR.back(), *mps[i], *mpo[i], mpo_t[i].get(), precision, &other));
            mark(MOD_UPDATE, false);
            mps[i - 1] = krylov(1, *envL.back(), *r.U, mpo[i - 1].get(), nullptr, *envR.back(), true, MOD_EVL1);
            envL.pop_back();
        } else {
            mps[i] = r.V;
            mps[i - 1] = r.U;
        }
    }
    envR.push_back(op_env(false, *envR.back(), *mps[1], *mpo[1], mpo_t[1].get(), precision, &other));
    end_sweep();
}

// State::canonicalize (holstein/state.h:166-185): an L->R sweep of svd_impl<2,1>
// carrying S.V^H into the next site, then an R->L sweep of svd_impl<1,2>
// carrying U.S into the previous one; the orthogonality centre ends on site 0.
std::vector<TensorP> op_canonicalize(const std::vector<TensorP> &in, double tol, int max_dim, int precision) {
    check_precision(precision);
    KV_REQUIRE(!in.empty(), KV_EINVAL, "empty MPS");
    std::vector<TensorP> t(in.begin(), in.end());
    const int ns = (int)t.size();
    for (int i = 0; i < ns - 1; ++i) {
        SvdOut r = op_svd(*t[i], 2, true, tol, max_dim, precision);
        t[i] = r.U;
        t[i + 1] = op_product(*r.V, *t[i + 1], 1, KV_OP_N, KV_OP_N, precision);
    }
    for (int i = ns - 1; i > 0; --i) {
        SvdOut r = op_svd(*t[i], 1, false, tol, max_dim, precision);
        t[i] = r.V;
        t[i - 1] = op_product(*t[i - 1], *r.U, 1, KV_OP_N, KV_OP_N, precision);
    }
    return t;
}

// sum_k E[k] R[k] over the blocks of two environments of one bond that carry
// the same (shape, charges): the value of <a|O|b> where the left part's
// environment E meets the right part's R
static cplx env_meet(const DTensor &E, const DTensor &R) {
    std::vector<double2> he(std::max<int64_t>(1, E.meta.nelem)), hr(std::max<int64_t>(1, R.meta.nelem));
    if (E.meta.nelem)
        KV_CUDA(cudaMemcpyAsync(he.data(), E.data(), E.meta.nelem * sizeof(double2), cudaMemcpyDeviceToHost,
                                ctx().stream));
    if (R.meta.nelem)
        KV_CUDA(cudaMemcpyAsync(hr.data(), R.data(), R.meta.nelem * sizeof(double2), cudaMemcpyDeviceToHost,
                                ctx().stream));
    KV_CUDA(cudaStreamSynchronize(ctx().stream));
    cplx v = 0.0;
    for (auto &b : E.meta.blocks) {
        const int k = R.meta.find(b);
        if (k < 0) continue;
        const BlockMeta &r = R.meta.blocks[k];
        for (int64_t i = 0; i < b.size; ++i)
            v += cplx(he[b.off + i].x, he[b.off + i].y) * cplx(hr[r.off + i].x, hr[r.off + i].y);
    }
    return v;
}

// <psi|O_k|psi> for operators O_k that are the identity except on one site
// (Operator::join, holstein/operator.h:178-198, with such an MPO): the
// identity environments from the left (L_s) and from the right (R_s) are
// built once, then each operator costs one environment update at its site,
// E = env_sweep(L_s, A_s, O_k), met with R_{s+1} -- all site populations of a
// chain in about three passes instead of one full contraction each.
std::vector<cplx> op_local_expectations(const std::vector<DTensor *> &mps, const std::vector<DTensor *> &ident,
                                        const std::vector<int> &op_site, const std::vector<DTensor *> &op) {
    const int ns = (int)mps.size();
    KV_REQUIRE(ns >= 1 && (int)ident.size() == ns, KV_EINVAL, "one identity MPO tensor per site is required");
    KV_REQUIRE(op_site.size() == op.size(), KV_EINVAL, "one site per local operator");
    for (int s : op_site) KV_REQUIRE(s >= 0 && s < ns, KV_EINVAL, "local operator site out of range");
    KV_REQUIRE(!mps.back()->meta.blocks.empty(), KV_EINVAL, "empty last site tensor");
    std::vector<TensorP> L(ns + 1), R(ns + 1);
    L[0] = boundary_env(1, 0);
    for (int s = 0; s < ns; ++s) L[s + 1] = op_env(true, *L[s], *mps[s], *ident[s], nullptr, KV_FP64, nullptr);
    R[ns] = boundary_env(-1, mps[ns - 1]->meta.blocks[0].qn[2]);
    for (int s = ns - 1; s >= 0; --s) R[s] = op_env(false, *R[s + 1], *mps[s], *ident[s], nullptr, KV_FP64, nullptr);
    std::vector<cplx> out;
    for (size_t k = 0; k < op.size(); ++k) {
        const int s = op_site[k];
        TensorP E = op_env(true, *L[s], *mps[s], *op[k], nullptr, KV_FP64, nullptr);
        out.push_back(env_meet(*E, *R[s + 1]));
    }
    return out;
}

// Operator::join (holstein/operator.h:178-198)
cplx op_expectation(const std::vector<DTensor *> &a, const std::vector<DTensor *> &w, const std::vector<DTensor *> &b) {
    TensorP env = boundary_env(1, 0);
    for (size_t i = 0; i < a.size(); ++i) {
        TensorP t1 = op_product(*env, *b[i], 1, KV_OP_N, KV_OP_N, KV_FP64);
        MixPlanFull M = plan_mix(t1->meta, w[i]->meta, 1);
        M.mix.upload();
        auto t2 = DTensor::make(M.out, false);
        launch_mix(M.mix, t1->data(), w[i]->data(), t2->data(), nullptr);
        env = op_product(*a[i], *t2, 2, KV_OP_C, KV_OP_N, KV_FP64);
    }
    if (env->meta.blocks.empty()) return 0.0;
    std::vector<double2> h(env->meta.nelem);
    KV_CUDA(cudaMemcpyAsync(h.data(), env->data(), env->meta.nelem * sizeof(double2), cudaMemcpyDeviceToHost,
                            ctx().stream));
    KV_CUDA(cudaStreamSynchronize(ctx().stream));
    const int q = env->meta.blocks[0].qn[0];
    cplx r = 0.0;
    for (auto &blk : env->meta.blocks)
        if (blk.size == 1 && blk.qn[0] == q && blk.qn[1] == 0 && blk.qn[2] == q) r += cplx(h[blk.off].x, h[blk.off].y);
    return r;
}

}  // namespace kv
