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

#include "kv_engine.h"
#include "kv_svd.h"

namespace kv {

// ================================================================ runtime
static Context g_ctx;
Context &ctx() { return g_ctx; }
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
ProductPlan plan_product(const Meta &A, const Meta &B, int nc, int opA, int opB) {
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
    std::vector<std::vector<GemmSeg>> per_out;
    std::vector<std::pair<int, int>> mn;  // M, N per output block
    // index B blocks by the charges of their contracted legs for fast matching
    for (size_t i = 0; i < A.blocks.size(); ++i) {
        const BlockMeta &a = A.blocks[i];
        for (size_t j = 0; j < B.blocks.size(); ++j) {
            const BlockMeta &b = B.blocks[j];
            bool match = true;
            for (int ax = 0; ax < nc && match; ++ax)
                match = a.shape[iax1 + ax] == b.shape[iax2 + ax] && a.qn[iax1 + ax] == b.qn[iax2 + ax];
            if (!match) continue;
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
            int pos = P.out.find(o);
            if (pos < 0) {
                pos = (int)P.out.blocks.size();
                P.out.blocks.push_back(o);
                per_out.emplace_back();
                mn.push_back({nrow, ncol});
            }
            GemmSeg s;
            s.a_off = a.off;
            s.b_off = b.off;
            s.K = nk;
            s.opa = (opA == KV_OP_N) ? 0 : 1;
            s.opb = (opB == KV_OP_N) ? 0 : 1;
            s.lda = (opA == KV_OP_N) ? nk : nrow;
            s.ldb = (opB == KV_OP_N) ? ncol : nk;
            per_out[pos].push_back(s);
            P.gemm.ref_flops += 8.0 * nrow * (double)ncol * nk;
            P.gemm.max_k = std::max(P.gemm.max_k, nk);
        }
    }
    P.out.layout();
    P.per_out = std::move(per_out);
    P.mn = std::move(mn);
    return P;
}

// Tiles of the grouped GEMM: output block b of the plan is written at
// target_off[b] (complex elements) of the destination buffer.
void build_tiles(ProductPlan &P, const std::vector<int64_t> &target_off, int tile_m, int tile_n) {
    GemmPlan &g = P.gemm;
    g.tiles.clear();
    g.segs.clear();
    for (size_t b = 0; b < P.per_out.size(); ++b) {
        const int M = P.mn[b].first, N = P.mn[b].second;
        const int sb = (int)g.segs.size();
        for (auto &s : P.per_out[b]) g.segs.push_back(s);
        const int se = (int)g.segs.size();
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

// Reference flop count of a product<> on a given (unmerged) operand structure.
double ref_product_flops(const Meta &A, const Meta &B, int nc, int opA, int opB) {
    const int n1 = A.rank, n2 = B.rank;
    const int iax1 = (opA == KV_OP_N) ? n1 - nc : 0;
    const int iax2 = (opB == KV_OP_N) ? 0 : n2 - nc;
    double f = 0.0;
    for (auto &a : A.blocks)
        for (auto &b : B.blocks) {
            bool match = true;
            for (int ax = 0; ax < nc && match; ++ax)
                match = a.shape[iax1 + ax] == b.shape[iax2 + ax] && a.qn[iax1 + ax] == b.qn[iax2 + ax];
            if (match) f += 8.0 * (double)a.size * (double)(b.size / prod_range(b, iax2, iax2 + nc));
        }
    return f;
}

// ============================================================ mix plans
// env_mps_mpo / env_mps2_mpo1 / env_mps2_mpo2 (holstein/product.h:203-477):
// legs lead, lead+1 of lm (w_l, sigma) contract with legs 1, 2 of W; W's legs
// 0, 3 (sigma', w_r) replace them.  Equal output blocks are merged here (the
// reference keeps them apart and the following product<> sums them).
MixPlanFull plan_mix(const Meta &lm, const Meta &W, int lead) {
    MixPlanFull R;
    R.out.rank = lm.rank;
    R.out.dirs = lm.dirs;
    R.out.dirs[lead] = W.dirs[0];
    R.out.dirs[lead + 1] = W.dirs[3];
    R.unmerged = R.out;
    std::vector<std::vector<MixTerm>> terms;
    std::vector<std::array<int, 3>> geo;  // so, wr, rest
    for (auto &a : lm.blocks)
        for (auto &w : W.blocks) {
            if (!(a.shape[lead] == w.shape[1] && a.shape[lead + 1] == w.shape[2] && a.qn[lead] == w.qn[1] &&
                  a.qn[lead + 1] == w.qn[2]))
                continue;
            BlockMeta o = a;
            o.shape[lead] = w.shape[0];
            o.qn[lead] = w.qn[0];
            o.shape[lead + 1] = w.shape[3];
            o.qn[lead + 1] = w.qn[3];
            R.unmerged.blocks.push_back(o);
            int pos = R.out.find(o);
            const int rest = (int)prod_range(a, lead + 2, lm.rank);
            if (pos < 0) {
                pos = (int)R.out.blocks.size();
                R.out.blocks.push_back(o);
                terms.emplace_back();
                geo.push_back({w.shape[0], w.shape[3], rest});
            }
            const int K = a.shape[lead] * a.shape[lead + 1];
            terms[pos].push_back({a.off, w.off, K});
            const double nk = (double)prod_range(a, 0, lead);
            R.ref_flops += 8.0 * nk * w.shape[0] * (double)w.shape[3] * rest * K;
        }
    R.out.layout();
    R.unmerged.layout();
    for (size_t b = 0; b < R.out.blocks.size(); ++b) {
        MixJob j;
        j.out_off = R.out.blocks[b].off;
        j.count = R.out.blocks[b].size;
        j.nk_unused = 0;
        j.so = geo[b][0];
        j.wr = geo[b][1];
        j.rest = geo[b][2];
        j.term_begin = (int)R.mix.terms.size();
        for (auto &t : terms[b]) R.mix.terms.push_back(t);
        j.term_end = (int)R.mix.terms.size();
        const int job = (int)R.mix.jobs.size();
        R.mix.jobs.push_back(j);
        for (int64_t s = 0; s < j.count; s += 1024) R.mix.items.push_back({job, s});
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
        c.prof_ms += ms;
        c.prof_launches += 1;
        if (!r.st || (iters_of && r.k < iters_of(r.st, arg))) c.prof_flops += r.flops;
        c.ev_free.push_back(r.a);
        c.ev_free.push_back(r.b);
    }
    c.prof_pending.clear();
}

void run_gemm(const GemmPlan &g, const double2 *A, const double2 *B, double2 *C, double alpha, int precision,
              const int *skip, const KrylovState *st, int k) {
    if (g.tiles.empty()) return;
    auto &c = ctx();
    ProfRec rec{};
    if (c.prof) {
        rec = {prof_event(), prof_event(), g.ref_flops, st, k};
        KV_CUDA(cudaEventRecord(rec.a, c.stream));
    }
    if (precision == KV_FP64) launch_gemm_fp64(g, A, B, C, alpha, skip);
    else if (precision == KV_MIXED_TF32) launch_gemm_mixed(g, A, B, C, alpha, skip);
    else throw Error(KV_EINVAL, "unknown precision mode");
    if (c.prof) {
        KV_CUDA(cudaEventRecord(rec.b, c.stream));
        c.prof_pending.push_back(rec);
    }
}

static void check_precision(int precision) {
    KV_REQUIRE(precision == KV_FP64 || precision == KV_MIXED_TF32, KV_EINVAL, "unknown precision mode");
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
// Krylov layout: the closure of psi's blocks under H_eff (union of input and
// output block sets until stable), so every Lanczos vector and H_eff . v share
// one layout; blocks absent from the reference's tensors are zero.
HeffPlan plan_heff(int nsite, const Meta &L, const Meta &psi, const Meta *W1, const Meta *W2, const Meta &R,
                   int precision) {
    HeffPlan H;
    H.nsite = nsite;
    Meta K = psi;
    K.layout();
    for (int iter = 0; iter < 8; ++iter) {
        ProductPlan P1 = plan_product(L, K, 1, KV_OP_N, KV_OP_N);
        Meta last = P1.out;
        if (nsite >= 1) last = plan_mix(last, *W1, 1).out;
        if (nsite == 2) last = plan_mix(last, *W2, 2).out;
        ProductPlan P2 = plan_product(last, R, 2, KV_OP_N, KV_OP_T);
        bool grew = false;
        for (auto &b : P2.out.blocks)
            if (K.find(b) < 0) { K.blocks.push_back(b); grew = true; }
        if (!grew) break;
        K.layout();
        KV_REQUIRE(iter < 7, KV_EINVAL, "H_eff block closure did not converge");
    }
    K.layout();
    H.klayout = K;
    // final plans on the closed layout
    H.p1 = plan_product(L, K, 1, KV_OP_N, KV_OP_N);
    build_tiles(H.p1, own_offsets(H.p1.out), kTileM(precision), kTileN(precision));
    Meta last = H.p1.out;
    Meta last_unmerged = H.p1.out;
    H.ref_flops = H.p1.gemm.ref_flops;
    H.gemm_flops = H.p1.gemm.ref_flops;
    if (nsite >= 1) {
        H.m1 = plan_mix(last, *W1, 1);
        H.ref_flops += H.m1.ref_flops;
        last = H.m1.out;
        last_unmerged = H.m1.unmerged;
    }
    if (nsite == 2) {
        // the reference mixes W2 into every unmerged W1 block; count its flops on that structure
        MixPlanFull ref2 = plan_mix(last_unmerged, *W2, 2);
        H.m2 = plan_mix(last, *W2, 2);
        H.ref_flops += ref2.ref_flops;
        last = H.m2.out;
        last_unmerged = ref2.unmerged;
    }
    H.p2 = plan_product(last, R, 2, KV_OP_N, KV_OP_T);
    const double f2 = ref_product_flops(last_unmerged, R, 2, KV_OP_N, KV_OP_T);
    H.ref_flops += f2;
    H.gemm_flops += f2;
    // the grouped GEMM is credited with the reference flops of the pairs it replaces
    H.p2.gemm.ref_flops = f2;
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
    H.p1.gemm.upload();
    H.p2.gemm.upload();
    if (nsite >= 1) H.m1.mix.upload();
    if (nsite == 2) H.m2.mix.upload();
    H.t1 = DevBuf(std::max<int64_t>(1, H.p1.out.nelem) * sizeof(double2));
    if (nsite >= 1) H.t2 = DevBuf(std::max<int64_t>(1, H.m1.out.nelem) * sizeof(double2));
    if (nsite == 2) H.t3 = DevBuf(std::max<int64_t>(1, H.m2.out.nelem) * sizeof(double2));
    return H;
}

// out (Krylov layout) = scale * H_eff . v (Krylov layout)
void run_heff(HeffPlan &H, const DTensor &L, const double2 *v, const DTensor *W1, const DTensor *W2,
              const DTensor &R, double2 *out, double scale, int precision, const int *skip,
              const KrylovState *st = nullptr, int k = -1) {
    run_gemm(H.p1.gemm, L.data(), v, H.t1.as<double2>(), 1.0, precision, skip, st, k);
    const double2 *last = H.t1.as<double2>();
    if (H.nsite >= 1) {
        launch_mix(H.m1.mix, last, W1->data(), H.t2.as<double2>(), skip);
        last = H.t2.as<double2>();
    }
    if (H.nsite == 2) {
        launch_mix(H.m2.mix, last, W2->data(), H.t3.as<double2>(), skip);
        last = H.t3.as<double2>();
    }
    run_gemm(H.p2.gemm, last, R.data(), out, scale, precision, skip, st, k);
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
    HeffPlan H = plan_heff(nsite, L.meta, psi.meta, W1 ? &W1->meta : nullptr, W2 ? &W2->meta : nullptr, R.meta,
                           precision);
    DevBuf v(std::max<int64_t>(1, H.klayout.nelem) * sizeof(double2));
    scatter_into(psi, H.klayout, v.as<double2>());
    auto out = DTensor::make(H.klayout, false);
    run_heff(H, L, v.as<double2>(), W1, W2, R, out->data(), scale, precision, nullptr);
    return out;
}

// ------------------------------------------------------- local_krylov
TensorP op_lanczos(int nsite, const DTensor &L, const DTensor &psi, const DTensor *W1, const DTensor *W2,
                   const DTensor &R, double dt, int max_iter, double tol, bool reverse, int precision,
                   KrylovState *st_dev, Flops *per_iter) {
    check_precision(precision);
    KV_REQUIRE(max_iter >= 2 && max_iter <= kMaxKrylov, KV_EINVAL, "max_iter must be in [2, 32]");
    KV_REQUIRE(tol < 1.0, KV_EINVAL, "Krylov tolerance must be < 1");
    HeffPlan H = plan_heff(nsite, L.meta, psi.meta, W1 ? &W1->meta : nullptr, W2 ? &W2->meta : nullptr, R.meta,
                           precision);
    if (per_iter) { per_iter->gemm = H.gemm_flops; per_iter->mix = H.ref_flops - H.gemm_flops; }
    const int64_t n = H.klayout.nelem;
    const int nvec = max_iter;  // V_0 .. V_{max_iter-1}
    DevBuf Vbuf(std::max<int64_t>(1, n) * nvec * sizeof(double2));
    DevBuf hv(std::max<int64_t>(1, n) * sizeof(double2));
    DevBuf parts(2 * reduce_parts() * sizeof(double2));
    DevBuf tmp(std::max<int64_t>(1, n) * sizeof(double2));
    double2 *V = Vbuf.as<double2>();
    scatter_into(psi, H.klayout, tmp.as<double2>());
    krylov_start(st_dev, tmp.as<double2>(), V, n, parts.as<double2>());
    const int *skip = &st_dev->done;
    for (int k = 0; k < max_iter - 1; ++k) {
        run_heff(H, L, V + (int64_t)k * n, W1, W2, R, hv.as<double2>(), dt * 0.5, precision, skip, st_dev, k);
        krylov_step(st_dev, k, hv.as<double2>(), k > 0 ? V + (int64_t)(k - 1) * n : nullptr, V + (int64_t)k * n,
                    V + (int64_t)(k + 1) * n, n, parts.as<double2>(), tol, max_iter);
    }
    std::vector<double2 *> ptrs(nvec);
    for (int i = 0; i < nvec; ++i) ptrs[i] = V + (int64_t)i * n;
    DevBuf dptrs = upload_vec(ptrs);
    auto out = DTensor::make(H.klayout, false);
    krylov_finish(st_dev, dptrs.as<double2 *>(), out->data(), n, reverse ? 1 : 0);
    return out;
}

// ---------------------------------------------------------------- SVD
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

SvdOut op_svd(const DTensor &A, int r1, bool l2r, double thres, int max_dim) {
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
    for (int ri = 0; ri < (int)rows.size(); ++ri)
        for (int ci = 0; ci < (int)cols.size(); ++ci) {
            if (rows[ri].q + cols[ci].q != 0) continue;
            SvdSector s{};
            s.m = rows[ri].len;
            s.n = cols[ci].len;
            s.transposed = s.m < s.n ? 1 : 0;
            s.p = std::max(s.m, s.n);
            s.q = std::min(s.m, s.n);
            s.t_off = P.t_elems;
            s.v_off = P.v_elems;
            s.s_off = P.s_elems;
            P.t_elems += (int64_t)s.p * s.q;
            P.v_elems += (int64_t)s.q * s.q;
            P.s_elems += s.q;
            P.max_q = std::max(P.max_q, s.q);
            rows[ri].kept = s.q;
            cols[ci].kept = s.q;
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
    DevBuf T(std::max<int64_t>(1, P.t_elems) * sizeof(double2)), Us(std::max<int64_t>(1, P.t_elems) * sizeof(double2));
    DevBuf V(std::max<int64_t>(1, P.v_elems) * sizeof(double2)), Vs(std::max<int64_t>(1, P.v_elems) * sizeof(double2));
    DevBuf S(std::max<int64_t>(1, P.s_elems) * sizeof(double));
    DevBuf status(std::max<size_t>(1, P.secs.size()) * sizeof(int));
    svd_gather(P, A.data(), T.as<double2>());
    svd_jacobi(P, T.as<double2>(), V.as<double2>(), status.as<int>(), 60, 1e-15);
    svd_finalize(P, T.as<double2>(), V.as<double2>(), Us.as<double2>(), Vs.as<double2>(), S.as<double>());
    std::vector<double> sv(P.s_elems);
    std::vector<int> st(P.secs.size());
    if (P.s_elems)
        KV_CUDA(cudaMemcpyAsync(sv.data(), S.p, P.s_elems * sizeof(double), cudaMemcpyDeviceToHost, ctx().stream));
    if (!st.empty())
        KV_CUDA(cudaMemcpyAsync(st.data(), status.p, st.size() * sizeof(int), cudaMemcpyDeviceToHost, ctx().stream));
    KV_CUDA(cudaStreamSynchronize(ctx().stream));
    for (int x : st) KV_REQUIRE(x >= 0, KV_ETIMEOUT, "Jacobi SVD did not converge within the sweep limit");
    for (double x : sv) KV_REQUIRE(std::isfinite(x), KV_ENONFINITE, "non-finite singular value");
    // global ordering and truncation, holstein/svd.h:350-388
    std::vector<std::pair<int, double>> collect;
    for (size_t s = 0; s < P.secs.size(); ++s) {
        const int q = l2r ? rows[sec_rc[s].first].q : cols[sec_rc[s].second].q;
        for (int i = 0; i < P.secs[s].q; ++i) collect.push_back({q, sv[P.secs[s].s_off + i]});
    }
    std::sort(collect.begin(), collect.end(), [](const std::pair<int, double> &a, const std::pair<int, double> &b) {
        return a.second > b.second;
    });
    SvdOut out;
    out.n_total = (int)collect.size();
    for (int i = (int)collect.size() - 1; i > 0; --i) {
        if (!(i >= max_dim || collect[i].second <= thres)) break;
        const int q = collect[i].first;
        for (auto &rw : rows) if (rw.q == (l2r ? q : -q)) { rw.kept -= 1; break; }
        for (auto &cl : cols) if (cl.q == (l2r ? -q : q)) { cl.kept -= 1; break; }
        collect.pop_back();
    }
    out.n_kept = (int)collect.size();
    for (auto &c : collect) out.kept_s.push_back(c.second);
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
    for (size_t s = 0; s < P.secs.size(); ++s) {
        Macro &rw = rows[sec_rc[s].first];
        Macro &cl = cols[sec_rc[s].second];
        if (rw.kept <= 0 || cl.kept <= 0) continue;
        for (auto &ra : rw.subs) {
            BlockMeta b;
            for (int i = 0; i < r1; ++i) { b.shape[i] = ra.shape[i]; b.qn[i] = ra.qn[i]; }
            b.shape[r1] = rw.kept;
            b.qn[r1] = rw.q;
            mu.blocks.push_back(b);
            pu.push_back({(int)s, 0, ra.pos, ra.len, rw.kept});
        }
        for (auto &ca : cl.subs) {
            BlockMeta b;
            b.shape[0] = cl.kept;
            b.qn[0] = -cl.q;
            for (int i = 0; i < M.rank - r1; ++i) { b.shape[i + 1] = ca.shape[i]; b.qn[i + 1] = ca.qn[i]; }
            mv.blocks.push_back(b);
            pv.push_back({(int)s, 1, ca.pos, ca.len, cl.kept});
        }
    }
    out.U = DTensor::make(mu, false);
    out.V = DTensor::make(mv, false);
    std::vector<SvdScatter> su, svs;
    for (size_t i = 0; i < pu.size(); ++i)
        su.push_back({out.U->meta.blocks[i].off, pu[i].sector, 0, pu[i].pos, pu[i].len, pu[i].kept, l2r ? 0 : 1});
    for (size_t i = 0; i < pv.size(); ++i)
        svs.push_back({out.V->meta.blocks[i].off, pv[i].sector, 1, pv[i].pos, pv[i].len, pv[i].kept, l2r ? 1 : 0});
    svd_scatter(su, P, Us.as<double2>(), Vs.as<double2>(), S.as<double>(), out.U->data());
    svd_scatter(svs, P, Us.as<double2>(), Vs.as<double2>(), S.as<double>(), out.V->data());
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
    launch_mix(M.mix, t1->data(), W.data(), t2->data(), nullptr);
    ProductPlan P2 = plan_product(A.meta, t2->meta, 2, KV_OP_C, KV_OP_N);
    const double f2 = ref_product_flops(A.meta, M.unmerged, 2, KV_OP_C, KV_OP_N);
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
    // holstein/tdvp.h:303-316
    const int ns = (int)mps.size();
    envL = {boundary_env(1, 0)};
    envR = {boundary_env(-1, mps[ns - 1]->meta.blocks[0].qn[2])};
    for (int i = ns - 1; i > 0; --i)
        envR.push_back(op_env(false, *envR.back(), *mps[i], *mpo[i], mpo_t[i].get(), precision, nullptr));
    KV_CUDA(cudaStreamSynchronize(ctx().stream));
}

Tdvp::~Tdvp() {
    for (auto &e : events) cudaEventDestroy(e);
    for (auto &e : sweep_ev) cudaEventDestroy(e);
}

void Tdvp::mark(int module, bool start) {
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
    Flops f;
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
    float sms = 0.f;
    KV_CUDA(cudaEventElapsedTime(&sms, sweep_ev[0], sweep_ev[1]));
    sweep_ms = sms;
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
        f += (kf.second.gemm + kf.second.mix) * h.iters;
        fg += kf.second.gemm * h.iters;
    }
    last_ref_flops = f;
    last_gemm_flops = fg;
    std::pair<const KrylovState *, const std::vector<KrylovState> *> arg{kstate.as<KrylovState>(), &host};
    prof_resolve(tdvp_iters_of, &arg);
}

// TDVP::one_site (holstein/tdvp.h:78-141)
void Tdvp::one_site() {
    begin_sweep();
    const int ns = (int)mps.size();
    for (int i = 0; i < ns; ++i) {
        mps[i] = krylov(1, *envL.back(), *mps[i], mpo[i].get(), nullptr, *envR.back(), false, MOD_EVL1);
        if (i < ns - 1) {
            mark(MOD_SVD, true);
            SvdOut r = op_svd(*mps[i], 2, true, tol_svd, max_dim);
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
            SvdOut r = op_svd(*mps[i], 1, false, tol_svd, max_dim);
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

// TDVP::two_site (holstein/tdvp.h:144-227)
void Tdvp::two_site() {
    begin_sweep();
    const int ns = (int)mps.size();
    envR.pop_back();
    for (int i = 0; i < ns - 1; ++i) {
        mark(MOD_SWEEP, true);
        TensorP mm = op_product(*mps[i], *mps[i + 1], 1, KV_OP_N, KV_OP_N, precision, &other);
        mark(MOD_SWEEP, false);
        mm = krylov(2, *envL.back(), *mm, mpo[i].get(), mpo[i + 1].get(), *envR.back(), false, MOD_EVL2);
        mark(MOD_SVD, true);
        SvdOut r = op_svd(*mm, 2, true, tol_svd, max_dim);
        mark(MOD_SVD, false);
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
    for (int i = ns - 1; i > 0; --i) {
        mark(MOD_SWEEP, true);
        TensorP mm = op_product(*mps[i - 1], *mps[i], 1, KV_OP_N, KV_OP_N, precision, &other);
        mark(MOD_SWEEP, false);
        mm = krylov(2, *envL.back(), *mm, mpo[i - 1].get(), mpo[i].get(), *envR.back(), false, MOD_EVL2);
        mark(MOD_SVD, true);
        SvdOut r = op_svd(*mm, 2, false, tol_svd, max_dim);
        mark(MOD_SVD, false);
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
