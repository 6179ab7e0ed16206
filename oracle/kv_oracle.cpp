/*
 * kv_oracle.cpp -- CPU restatement of Kylin-V's Holstein TDVP hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the GPU library is checked
 * against (tests, smoke check) and the CPU baseline bench.py times; it is
 * never linked into or called by the GPU library.  It restates the
 * reference's algorithm step by step (block matching rules, output block
 * order, Lanczos recurrence, SVD sector assembly and truncation, sweep
 * schedule) on the same BLAS/LAPACK calls the reference makes
 * (zgemm/zgesvd/zheevd), taken from scipy's OpenBLAS.  Each function cites
 * the reference file:line it follows.  It is pinned against golden vectors
 * produced by the compiled reference (oracle/_ref, tests/golden/).
 *
 * C API (all functions return 0 on success, nonzero on error):
 *   tensors: kvo_tensor_new / kvo_tensor_info / kvo_tensor_get / kvo_tensor_free
 *   ops:     kvo_product, kvo_apply_zero/single/double, kvo_env_sweep,
 *            kvo_local_krylov, kvo_svd
 *   sweep:   kvo_tdvp_new / kvo_tdvp_sweep (mode 0: one global-Krylov step,
 *            1: one_site, 2: two_site, 3: one SA-1TDVP sweep with the widths
 *            and seed of kvo_tdvp_set_sa) / kvo_tdvp_site / kvo_tdvp_free;
 *            kvo_tdvp_window times a window of two-site local updates
 *            (CPU-baseline timing)
 *   observable: kvo_join
 */
#include <algorithm>
#include <chrono>
#include <array>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

using cplx = std::complex<double>;

extern "C" {
void scipy_cblas_zgemm(int layout, int ta, int tb, int m, int n, int k, const void *alpha,
                       const void *a, int lda, const void *b, int ldb, const void *beta, void *c,
                       int ldc);
int scipy_LAPACKE_zgesvd(int layout, char jobu, char jobvt, int m, int n, void *a, int lda,
                         double *s, void *u, int ldu, void *vt, int ldvt, double *superb);
int scipy_LAPACKE_zheevd(int layout, char jobz, char uplo, int n, void *a, int lda, double *w);
}

namespace {

enum Op { OP_N = 111, OP_T = 112, OP_C = 113 };
constexpr int kRowMajor = 101;
constexpr int kMaxRank = 6;

// ---------------------------------------------------------------- tensors
// Block<Rank> (holstein/block.h:23-166): dense row-major complex block with a
// U(1) charge per leg.
struct Block {
    int rank = 0;
    std::array<int, kMaxRank> shape{}, qn{};
    std::vector<cplx> data;
    size_t size() const {
        size_t s = 1;
        for (int i = 0; i < rank; ++i) s *= shape[i];
        return s;
    }
    bool same_key(const Block &o) const {
        for (int i = 0; i < rank; ++i)
            if (shape[i] != o.shape[i] || qn[i] != o.qn[i]) return false;
        return true;
    }
};

// Tensor<Rank> (holstein/tensor.h:16-209): leg directions + block list.
struct Tensor {
    int rank = 0;
    std::array<int, kMaxRank> dirs{};
    std::vector<Block> blocks;

    // push_back_ch: merge into an existing block of equal shape and charges
    // (holstein/tensor.h:172-185)
    void push_merge(const Block &b) {
        for (auto &x : blocks)
            if (x.same_key(b)) {
                for (size_t i = 0; i < x.data.size(); ++i) x.data[i] += b.data[i];
                return;
            }
        blocks.push_back(b);
    }
};

double tnorm(const Tensor &t) {  // holstein/tensor.h:211-219
    double s = 0.0;
    for (auto &b : t.blocks)
        for (auto &v : b.data) s += std::norm(v);
    return std::sqrt(s);
}

// overlap(ori, oth) = sum over blocks with equal shape and charges of
// <oth|ori> (zdotc(oth, ori)), holstein/tensor.h:221-237
cplx overlap(const Tensor &ori, const Tensor &oth) {
    cplx r = 0.0;
    for (auto &a : ori.blocks)
        for (auto &b : oth.blocks)
            if (a.same_key(b))
                for (size_t i = 0; i < a.data.size(); ++i) r += std::conj(b.data[i]) * a.data[i];
    return r;
}

void scale(Tensor &t, cplx v) {
    for (auto &b : t.blocks)
        for (auto &x : b.data) x *= v;
}

// t += v * s  with push_back_ch semantics (holstein/tensor.h:87-104, block.h:98-103)
void add_scaled(Tensor &t, const Tensor &s, cplx v) {
    for (auto &b : s.blocks) {
        Block c = b;
        for (auto &x : c.data) x *= v;
        t.push_merge(c);
    }
}

// transpose (holstein/tensor.h:242-257, block.h:166-210): permute legs by ax
Tensor transpose(const Tensor &t, const std::vector<int> &ax) {
    Tensor r;
    r.rank = t.rank;
    for (int i = 0; i < t.rank; ++i) r.dirs[i] = t.dirs[ax[i]];
    for (auto &b : t.blocks) {
        Block c;
        c.rank = b.rank;
        for (int i = 0; i < b.rank; ++i) { c.shape[i] = b.shape[ax[i]]; c.qn[i] = b.qn[ax[i]]; }
        c.data.resize(b.size());
        std::array<size_t, kMaxRank> sd{}, cd{};
        sd[b.rank - 1] = cd[b.rank - 1] = 1;
        for (int i = b.rank - 2; i >= 0; --i) {
            sd[i] = sd[i + 1] * b.shape[i + 1];
            cd[i] = cd[i + 1] * c.shape[i + 1];
        }
        for (size_t e = 0; e < b.size(); ++e) {
            size_t dst = 0;
            for (int j = 0; j < b.rank; ++j) dst += ((e / sd[ax[j]]) % b.shape[ax[j]]) * cd[j];
            c.data[dst] = b.data[e];
        }
        r.blocks.push_back(std::move(c));
    }
    return r;
}

// algorithmic flop counter: 8*M*N*K per complex GEMM the reference issues
double g_flops = 0.0;

// row-major complex GEMM with the reference's zdot conventions
// (util/allocation.h:186-205)
void zdot(const cplx *a, const cplx *b, int m, int n, int k, cplx *c, Op ta, Op tb) {
    const cplx one(1.0, 0.0), zero(0.0, 0.0);
    g_flops += 8.0 * m * (double)n * k;
    int lda = (ta == OP_N) ? k : m;
    int ldb = (tb == OP_N) ? n : k;
    scipy_cblas_zgemm(kRowMajor, ta, tb, m, n, k, &one, a, lda, b, ldb, &zero, c, n);
}

// ------------------------------------------------------------- product<>
// Generic block-sparse contraction of the last nc legs of op(A) with the first
// nc legs of op(B), holstein/product.h:61-201.  Pairs are matched on equal
// shape AND charge of every contracted leg; output blocks are created in
// first-appearance order of (shape, charge) and matched pairs accumulate.
Tensor product(const Tensor &m1, const Tensor &m2, int nc, Op t1, Op t2) {
    const int n1 = m1.rank, n2 = m2.rank, nr = n1 + n2 - 2 * nc;
    Tensor res;
    res.rank = nr;
    for (int i = 0; i < n1 - nc; ++i) {
        int src = (t1 == OP_N) ? i : nc + i;
        res.dirs[i] = m1.dirs[src] * (t1 == OP_C ? -1 : 1);
    }
    for (int i = 0; i < n2 - nc; ++i) {
        int src = (t2 == OP_N) ? nc + i : i;
        res.dirs[n1 - nc + i] = m2.dirs[src] * (t2 == OP_C ? -1 : 1);
    }
    const int iax1 = (t1 == OP_N) ? n1 - nc : 0;
    const int iax2 = (t2 == OP_N) ? 0 : n2 - nc;
    const int f1 = (t1 == OP_C) ? -1 : 1, f2 = (t2 == OP_C) ? -1 : 1;
    for (int ax = 0; ax < nc; ++ax)  // holstein/product.h:102-110
        if (m1.dirs[iax1 + ax] * f1 != -m2.dirs[iax2 + ax] * f2)
            throw std::runtime_error("contracted legs' directions mismatch");
    struct Pair { int x, y, pos, nrow, ncol, nk; };
    std::vector<Pair> pairs;
    std::vector<Block> outs;
    for (int i = 0; i < (int)m1.blocks.size(); ++i) {
        const Block &a = m1.blocks[i];
        for (int j = 0; j < (int)m2.blocks.size(); ++j) {
            const Block &b = m2.blocks[j];
            bool match = true;
            for (int ax = 0; ax < nc && match; ++ax)
                match = a.shape[iax1 + ax] == b.shape[iax2 + ax] && a.qn[iax1 + ax] == b.qn[iax2 + ax];
            if (!match) continue;
            Block o;
            o.rank = nr;
            int nrow = 1, ncol = 1;
            for (int u = 0; u < n1 - nc; ++u) {
                int src = (t1 == OP_N) ? u : nc + u;
                o.shape[u] = a.shape[src];
                o.qn[u] = a.qn[src];
                nrow *= a.shape[src];
            }
            for (int u = 0; u < n2 - nc; ++u) {
                int src = (t2 == OP_N) ? nc + u : u;
                o.shape[n1 - nc + u] = b.shape[src];
                o.qn[n1 - nc + u] = b.qn[src];
                ncol *= b.shape[src];
            }
            int nk = (int)(a.size() / nrow);
            int pos = -1;
            for (int p = 0; p < (int)outs.size(); ++p)
                if (outs[p].same_key(o)) { pos = p; break; }
            if (pos < 0) {
                pos = (int)outs.size();
                o.data.assign(o.size(), cplx(0.0, 0.0));
                outs.push_back(std::move(o));
            }
            pairs.push_back({i, j, pos, nrow, ncol, nk});
        }
    }
    std::vector<cplx> tmp;
    for (auto &p : pairs) {
        Block &o = outs[p.pos];
        tmp.assign(o.size(), cplx(0.0, 0.0));
        zdot(m1.blocks[p.x].data.data(), m2.blocks[p.y].data.data(), p.nrow, p.ncol, p.nk,
             tmp.data(), t1, t2);
        for (size_t e = 0; e < tmp.size(); ++e) o.data[e] += tmp[e];
    }
    res.blocks = std::move(outs);
    return res;
}

// ----------------------------------------------------- MPO application
// Shared kernel of env_mps_mpo / env_mps2_mpo1 / env_mps2_mpo2
// (holstein/product.h:203-230, 321-348, 399-429): for every matched
// (lm block, W block), out[k, s', wr, rest] = sum_{(wl, s)} W[s', wl, s, wr] lm[k, wl, s, rest]
// where `lead` leading legs of lm form k, legs lead, lead+1 are contracted
// with W's legs 1,2, and the remaining legs of lm are carried.  One output
// block per matched pair, no merging (push_back).
Tensor mpo_mix(const Tensor &lm, const Tensor &mpo, int lead) {
    Tensor res;
    res.rank = lm.rank;
    for (int i = 0; i < lead; ++i) res.dirs[i] = lm.dirs[i];
    res.dirs[lead] = mpo.dirs[0];
    res.dirs[lead + 1] = mpo.dirs[3];
    for (int i = lead + 2; i < lm.rank; ++i) res.dirs[i] = lm.dirs[i];
    for (auto &a : lm.blocks)
        for (auto &w : mpo.blocks) {
            if (!(a.shape[lead] == w.shape[1] && a.shape[lead + 1] == w.shape[2] &&
                  a.qn[lead] == w.qn[1] && a.qn[lead + 1] == w.qn[2]))
                continue;
            Block o;
            o.rank = lm.rank;
            o.shape = a.shape;
            o.qn = a.qn;
            o.shape[lead] = w.shape[0];
            o.qn[lead] = w.qn[0];
            o.shape[lead + 1] = w.shape[3];
            o.qn[lead + 1] = w.qn[3];
            o.data.assign(o.size(), cplx(0.0, 0.0));
            size_t nk = 1, rest = 1;
            for (int i = 0; i < lead; ++i) nk *= a.shape[i];
            for (int i = lead + 2; i < lm.rank; ++i) rest *= a.shape[i];
            const int K = a.shape[lead] * a.shape[lead + 1];
            const int so = w.shape[0], wr = w.shape[3];
            for (size_t k = 0; k < nk; ++k)
                for (int k2 = 0; k2 < so; ++k2)
                    zdot(w.data.data() + (size_t)k2 * K * wr, a.data.data() + k * K * rest, wr,
                         (int)rest, K, o.data.data() + (k * so + k2) * wr * rest, OP_T, OP_N);
            res.blocks.push_back(std::move(o));
        }
    return res;
}

Tensor env_mps_mpo(const Tensor &env, const Tensor &mps, const Tensor &mpo) {
    return mpo_mix(product(env, mps, 1, OP_N, OP_N), mpo, 1);  // holstein/product.h:250-275
}

// apply_single (holstein/product.h:547-553)
Tensor apply_single(const Tensor &L, const Tensor &A, const Tensor &W, const Tensor &R) {
    return product(env_mps_mpo(L, A, W), R, 2, OP_N, OP_T);
}

// apply_double (holstein/product.h:478-486; 372-397, 451-477)
Tensor apply_double(const Tensor &L, const Tensor &A, const Tensor &W1, const Tensor &W2,
                    const Tensor &R) {
    Tensor lm = product(L, A, 1, OP_N, OP_N);
    Tensor o1 = mpo_mix(lm, W1, 1);
    Tensor o2 = mpo_mix(o1, W2, 2);
    return product(o2, R, 2, OP_N, OP_T);
}

// apply_zero (holstein/product.h:540-545)
Tensor apply_zero(const Tensor &L, const Tensor &C, const Tensor &R) {
    return product(product(L, C, 1, OP_N, OP_N), R, 2, OP_N, OP_T);
}

// env_sweep (holstein/product.h:488-503): R->L transposes A {2,1,0}, W {0,3,2,1}
Tensor env_sweep(const Tensor &env, const Tensor &A, const Tensor &W, bool l2r) {
    if (l2r) return product(A, env_mps_mpo(env, A, W), 2, OP_C, OP_N);
    return env_sweep(env, transpose(A, {2, 1, 0}), transpose(W, {0, 3, 2, 1}), true);
}

// 4-argument env_sweep for <a|O|b> (holstein/product.h:505-521)
Tensor env_sweep2(const Tensor &env, const Tensor &A1, const Tensor &W, const Tensor &A2) {
    return product(A1, env_mps_mpo(env, A2, W), 2, OP_C, OP_N);
}

// --------------------------------------------------------- local_krylov
struct KrylovExit { int iters; double err; int converged; };

// local_krylov<Rank> (holstein/exponential.h:92-190).  H_eff is scaled by
// dt/2; beta and alpha are overlap(V, hv) = <hv|V>; the loop runs while
// k < maxIter-1 and the product of Lanczos norms exceeds tol; T (diag alpha,
// upper beta) is diagonalised by zheevd('V','U'); psi = sum_i c_i V_i with
// c = Z exp(-+i Lambda) Z^H e0 (+i for the reverse, zero-site step).
KrylovExit local_krylov(int nsite, const Tensor &L, Tensor &psi, const Tensor *W1,
                        const Tensor *W2, const Tensor &R, double dt, int max_iter, double tol,
                        bool reverse) {
    scale(psi, 1.0 / tnorm(psi));
    std::vector<Tensor> V = {psi};
    std::vector<cplx> alp, bet;
    int k = 0;
    double err = 1.0;
    KrylovExit ex{0, 0.0, 0};
    while (k < max_iter - 1 && err > tol) {
        Tensor hv = nsite == 0 ? apply_zero(L, V[k], R)
                  : nsite == 1 ? apply_single(L, V[k], *W1, R)
                               : apply_double(L, V[k], *W1, *W2, R);
        scale(hv, dt * 0.5);
        if (k > 0) {
            cplx b = overlap(V[k - 1], hv);
            bet.push_back(b);
            add_scaled(hv, V[k - 1], -b);
        }
        cplx a = overlap(V[k], hv);
        alp.push_back(a);
        add_scaled(hv, V[k], -a);
        double nh = tnorm(hv);
        err *= nh;
        if (err < tol) { ex.converged = 1; break; }
        scale(hv, 1.0 / nh);
        V.push_back(std::move(hv));
        ++k;
    }
    const int n = (int)alp.size();
    ex.iters = n;
    ex.err = err;
    std::vector<cplx> T((size_t)n * n, cplx(0.0, 0.0));
    for (int i = 0; i < n; ++i) {
        T[(size_t)i * n + i] = alp[i];
        if (i < n - 1) T[(size_t)i * n + i + 1] = bet[i];
    }
    std::vector<double> lam(n);
    if (scipy_LAPACKE_zheevd(kRowMajor, 'V', 'U', n, T.data(), n, lam.data()) != 0)
        throw std::runtime_error("zheevd failed");
    const cplx img = reverse ? cplx(0.0, 1.0) : cplx(0.0, -1.0);
    std::vector<cplx> c(n, cplx(0.0, 0.0));
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) c[i] += T[(size_t)i * n + j] * std::exp(img * lam[j]) * std::conj(T[j]);
    Tensor out = V[0];
    scale(out, c[0]);
    for (int i = 1; i < n; ++i) add_scaled(out, V[i], c[i]);
    psi = std::move(out);
    return ex;
}

// ---------------------------------------------------------------- SVD
// svd_impl<R1,R2> (holstein/svd.h:296-440) with fill_block (:110-205),
// copy_to_mat (:219-247) and redist_row/col (:250-293).
struct Micro { std::array<int, kMaxRank> shape{}, qn{}; int pos; int len; std::vector<int> idx; };
struct Macro { int q; int len = 0; int kept = 0; std::vector<Micro> subs; };

void fill_side(std::vector<Macro> &info, int q, const Block &b, int lo, int hi, int k) {
    Micro m;
    int len = 1;
    for (int i = lo; i < hi; ++i) { m.shape[i - lo] = b.shape[i]; m.qn[i - lo] = b.qn[i]; len *= b.shape[i]; }
    for (auto &mac : info) {
        if (mac.q != q) continue;
        for (auto &s : mac.subs) {
            bool same = true;
            for (int i = 0; i < hi - lo; ++i)
                same = same && s.shape[i] == m.shape[i] && s.qn[i] == m.qn[i];
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

struct SvdResult { Tensor U, V; std::vector<double> kept_s; int total = 0; };

SvdResult svd_impl(const Tensor &A, int r1, bool l2r, double thres, int max_dim) {
    const int rank = A.rank;
    std::vector<Macro> rows, cols;
    for (int k = 0; k < (int)A.blocks.size(); ++k) {
        const Block &b = A.blocks[k];
        int qr = 0, qc = 0;
        for (int i = 0; i < r1; ++i) qr += b.qn[i] * A.dirs[i];
        for (int i = r1; i < rank; ++i) qc += b.qn[i] * A.dirs[i];
        fill_side(rows, qr, b, 0, r1, k);
        fill_side(cols, qc, b, r1, rank, k);
    }
    struct Sector { int r, c, m, n, ldu; std::vector<cplx> U, Vt; };
    std::vector<Sector> secs;
    std::vector<std::pair<int, double>> svals;  // (charge, s)
    for (int ri = 0; ri < (int)rows.size(); ++ri)
        for (int ci = 0; ci < (int)cols.size(); ++ci) {
            Macro &rw = rows[ri], &cl = cols[ci];
            if (rw.q + cl.q != 0) continue;
            const int m = rw.len, n = cl.len, ldu = std::min(m, n);
            rw.kept = ldu;
            cl.kept = ldu;
            std::vector<cplx> Ar((size_t)m * n, cplx(0.0, 0.0));
            for (auto &ra : rw.subs)
                for (auto &ca : cl.subs)
                    for (int x : ra.idx)
                        for (int y : ca.idx) {
                            if (x != y) continue;
                            const Block &b = A.blocks[x];
                            for (int i = 0; i < ra.len; ++i)
                                for (int j = 0; j < ca.len; ++j)
                                    Ar[(size_t)(ra.pos + i) * n + ca.pos + j] = b.data[(size_t)i * ca.len + j];
                        }
            Sector s{ri, ci, m, n, ldu, std::vector<cplx>((size_t)m * ldu), std::vector<cplx>((size_t)ldu * n)};
            std::vector<double> sv(ldu), sup(std::max(1, ldu - 1));
            if (scipy_LAPACKE_zgesvd(kRowMajor, 'S', 'S', m, n, Ar.data(), n, sv.data(), s.U.data(), ldu,
                                     s.Vt.data(), n, sup.data()) != 0)
                throw std::runtime_error("zgesvd failed");
            for (int i = 0; i < ldu; ++i) {
                if (l2r) {
                    for (int j = 0; j < n; ++j) s.Vt[(size_t)i * n + j] *= sv[i];
                    svals.push_back({rw.q, sv[i]});
                } else {
                    for (int j = 0; j < m; ++j) s.U[(size_t)j * ldu + i] *= sv[i];
                    svals.push_back({cl.q, sv[i]});
                }
            }
            secs.push_back(std::move(s));
        }
    std::sort(svals.begin(), svals.end(), [](auto &a, auto &b) { return a.second > b.second; });
    SvdResult out;
    out.total = (int)svals.size();
    for (int i = (int)svals.size() - 1; i > 0; --i) {  // holstein/svd.h:361-388
        if (!(i >= max_dim || svals[i].second <= thres)) break;
        const int q = svals[i].first;
        for (auto &rw : rows) if (rw.q == (l2r ? q : -q)) { rw.kept -= 1; break; }
        for (auto &cl : cols) if (cl.q == (l2r ? -q : q)) { cl.kept -= 1; break; }
        svals.pop_back();
    }
    for (auto &p : svals) out.kept_s.push_back(p.second);
    const int left_dir = -1;
    out.U.rank = r1 + 1;
    out.V.rank = rank - r1 + 1;
    for (int i = 0; i < r1; ++i) out.U.dirs[i] = A.dirs[i];
    out.U.dirs[r1] = left_dir;
    out.V.dirs[0] = -left_dir;
    for (int i = r1; i < rank; ++i) out.V.dirs[i - r1 + 1] = A.dirs[i];
    for (auto &s : secs) {
        Macro &rw = rows[s.r], &cl = cols[s.c];
        if (rw.kept <= 0 || cl.kept <= 0) continue;
        const int ns = rw.kept;
        for (auto &ra : rw.subs) {  // redist_row
            Block b;
            b.rank = r1 + 1;
            for (int i = 0; i < r1; ++i) { b.shape[i] = ra.shape[i]; b.qn[i] = ra.qn[i]; }
            b.shape[r1] = ns;
            b.qn[r1] = -left_dir * rw.q;
            b.data.resize((size_t)ra.len * ns);
            for (int i = 0; i < ra.len; ++i)
                for (int j = 0; j < ns; ++j) b.data[(size_t)i * ns + j] = s.U[(size_t)(ra.pos + i) * s.ldu + j];
            out.U.push_merge(b);
        }
        const int nsc = cl.kept;
        for (auto &ca : cl.subs) {  // redist_col
            Block b;
            b.rank = rank - r1 + 1;
            b.shape[0] = nsc;
            b.qn[0] = left_dir * cl.q;
            for (int i = 0; i < rank - r1; ++i) { b.shape[i + 1] = ca.shape[i]; b.qn[i + 1] = ca.qn[i]; }
            b.data.resize((size_t)ca.len * nsc);
            for (int j = 0; j < nsc; ++j)
                for (int c = 0; c < ca.len; ++c) b.data[(size_t)j * ca.len + c] = s.Vt[(size_t)j * s.n + ca.pos + c];
            out.V.push_merge(b);
        }
    }
    return out;
}

// ------------------------------------------------------------ SA-1TDVP SVD
// The reference seeds a fresh mt19937 from std::random_device before every
// group of draws (one synthetic value; one new vector), a different sequence
// every run.  Here each group's mt19937 is seeded by the next value of a seed
// stream (an mt19937 seeded by the caller), the order of
// oracle/shim/seeded_device.h, under which the compiled reference repeats
// the same run: golden SA trajectories come from it.

// quasi-Gaussian density and its inversion by bisection on [0, 2]
// (util/allocation.h:232-256), written as the reference writes them
double quasi_gauss(double x, double bet) {
    double r = std::exp(-0.25 * bet * std::pow(x, 2.0)) * std::abs(0.25 * x / bet);
    r += (0.5 / bet - 0.25 * std::pow(x, 2.0)) * std::erfc(0.5 * std::pow(bet, 0.5) * std::abs(x)) * 0.5 *
         std::pow(3.1415926 / bet, 0.5);
    r *= std::exp(-0.25 * bet * std::pow(x, 2.0)) * 4.0 * bet * std::pow(bet / 3.1415926, 0.5);
    return r;
}

double inv_quasi_gauss(double y, double bet) {
    double hi = 2.0, lo = 0.0, res = 0.0;
    while (hi - lo > 1e-8) {
        res = 0.5 * (hi + lo);
        if ((quasi_gauss(res, bet) - y) * (quasi_gauss(lo, bet) - y) < 0) hi = res;
        else lo = res;
    }
    return res;
}

// Number of synthetic states sa_svd_impl adds (holstein/svd.h:525-560): the
// sorted spectrum's tail is continued by s_new = 10^(+-r) s_last^2 / s_prev,
// r = inv_quasi_gauss(u, beta), sign alternating, clamped to non-increasing,
// until a value falls to the threshold or the spectrum reaches max_dim; only
// for spectra with 5 < n < max_dim values.
int sa_added(const std::vector<double> &sorted_desc, int max_dim, double thres, double beta, std::mt19937 &seeds) {
    const int n = (int)sorted_desc.size();
    if (n < 2) return 0;
    std::vector<double> t = {sorted_desc[n - 2], sorted_desc[n - 1]};
    int added = 0;
    if (n < max_dim && n > 5) {
        for (int i = n; i < max_dim; ++i) {
            std::mt19937 gen{(std::mt19937::result_type)(unsigned int)seeds()};
            std::uniform_real_distribution<double> d(0, 1);
            const double rds = inv_quasi_gauss(d(gen), beta);
            const double f = (i + n) % 2 == 0 ? std::pow(10, rds) : std::pow(10, -1.0 * rds);
            t.push_back(f * std::pow(t[t.size() - 1], 2.0) / t[t.size() - 2]);
            if (t.back() <= thres) {
                t.pop_back();
                break;
            }
            if (t.back() > t[t.size() - 2]) t.back() = t[t.size() - 2];
            added = (int)t.size() - 2;
        }
    }
    return added;
}

// gs_ortho (util/allocation.h:260-320) on a row-major matrix a (nrow x ncol):
// extend_rows appends `inc` rows, else `inc` columns; fill_zero leaves them 0,
// else each new vector is drawn uniform(-1, 1) (real parts), normalised,
// orthogonalised one after another against every earlier vector (modified
// Gram-Schmidt, zdotc / zaxpy) and normalised again.
void gs_ortho(int nrow, int ncol, std::vector<cplx> &a, bool extend_rows, int inc, bool fill_zero,
              std::mt19937 &seeds) {
    if (extend_rows) {
        std::vector<cplx> b((size_t)(nrow + inc) * ncol, cplx(0.0, 0.0));
        std::copy(a.begin(), a.begin() + (size_t)nrow * ncol, b.begin());
        a.swap(b);
        if (fill_zero) return;
        auto row = [&](int r) { return a.data() + (size_t)r * ncol; };
        for (int i = 0; i < inc; ++i) {
            std::mt19937 gen((std::mt19937::result_type)(unsigned int)seeds());
            std::uniform_real_distribution<double> dis(-1, 1);
            cplx *v = row(nrow + i);
            for (int k = 0; k < ncol; ++k) v[k] = dis(gen);
            double nrm = 0.0;
            for (int k = 0; k < ncol; ++k) nrm += std::norm(v[k]);
            nrm = std::sqrt(nrm);
            for (int k = 0; k < ncol; ++k) v[k] *= 1.0 / nrm;
            for (int j = 0; j < nrow + i; ++j) {
                cplx d(0.0, 0.0);
                for (int k = 0; k < ncol; ++k) d += std::conj(row(j)[k]) * v[k];
                for (int k = 0; k < ncol; ++k) v[k] -= d * row(j)[k];
            }
            nrm = 0.0;
            for (int k = 0; k < ncol; ++k) nrm += std::norm(v[k]);
            nrm = std::sqrt(nrm);
            for (int k = 0; k < ncol; ++k) v[k] *= 1.0 / nrm;
        }
    } else {
        const int ld = ncol + inc;
        std::vector<cplx> b((size_t)nrow * ld, cplx(0.0, 0.0));
        for (int r = 0; r < nrow; ++r)
            for (int c = 0; c < ncol; ++c) b[(size_t)r * ld + c] = a[(size_t)r * ncol + c];
        a.swap(b);
        if (fill_zero) return;
        auto at = [&](int r, int c) -> cplx & { return a[(size_t)r * ld + c]; };
        for (int i = 0; i < inc; ++i) {
            std::mt19937 gen((std::mt19937::result_type)(unsigned int)seeds());
            std::uniform_real_distribution<double> dis(-1, 1);
            const int c = ncol + i;
            for (int r = 0; r < nrow; ++r) at(r, c) = dis(gen);
            double nrm = 0.0;
            for (int r = 0; r < nrow; ++r) nrm += std::norm(at(r, c));
            nrm = std::sqrt(nrm);
            for (int r = 0; r < nrow; ++r) at(r, c) *= 1.0 / nrm;
            for (int j = 0; j < c; ++j) {
                cplx d(0.0, 0.0);
                for (int r = 0; r < nrow; ++r) d += std::conj(at(r, j)) * at(r, c);
                for (int r = 0; r < nrow; ++r) at(r, c) -= d * at(r, j);
            }
            nrm = 0.0;
            for (int r = 0; r < nrow; ++r) nrm += std::norm(at(r, c));
            nrm = std::sqrt(nrm);
            for (int r = 0; r < nrow; ++r) at(r, c) *= 1.0 / nrm;
        }
    }
}

// sa_svd_impl (holstein/svd.h:443-614): every sector's full SVD is kept (no
// truncation); if the spectrum is short of max_dim, sa_added states are given
// to the sectors in order, each taking as many as its kept side has room for:
// new orthonormal directions on the kept side (U for left-to-right, V^H
// for right-to-left), zero rows / columns on the other, so the state is
// unchanged and only the bond grows.
SvdResult sa_svd_impl(const Tensor &A, int r1, bool l2r, double thres, int max_dim, double beta,
                      std::mt19937 &seeds) {
    const int rank = A.rank;
    std::vector<Macro> rows, cols;
    for (int k = 0; k < (int)A.blocks.size(); ++k) {
        const Block &b = A.blocks[k];
        int qr = 0, qc = 0;
        for (int i = 0; i < r1; ++i) qr += b.qn[i] * A.dirs[i];
        for (int i = r1; i < rank; ++i) qc += b.qn[i] * A.dirs[i];
        fill_side(rows, qr, b, 0, r1, k);
        fill_side(cols, qc, b, r1, rank, k);
    }
    struct Sector { int r, c, m, n, ldu; std::vector<cplx> U, Vt; };
    std::vector<Sector> secs;
    std::vector<double> svals;
    for (int ri = 0; ri < (int)rows.size(); ++ri)
        for (int ci = 0; ci < (int)cols.size(); ++ci) {
            Macro &rw = rows[ri], &cl = cols[ci];
            if (rw.q + cl.q != 0) continue;
            const int m = rw.len, n = cl.len, ldu = std::min(m, n);
            rw.kept = ldu;
            cl.kept = ldu;
            std::vector<cplx> Ar((size_t)m * n, cplx(0.0, 0.0));
            for (auto &ra : rw.subs)
                for (auto &ca : cl.subs)
                    for (int x : ra.idx)
                        for (int y : ca.idx) {
                            if (x != y) continue;
                            const Block &b = A.blocks[x];
                            for (int i = 0; i < ra.len; ++i)
                                for (int j = 0; j < ca.len; ++j)
                                    Ar[(size_t)(ra.pos + i) * n + ca.pos + j] = b.data[(size_t)i * ca.len + j];
                        }
            Sector s{ri, ci, m, n, ldu, std::vector<cplx>((size_t)m * ldu), std::vector<cplx>((size_t)ldu * n)};
            std::vector<double> sv(ldu), sup(std::max(1, ldu - 1));
            if (scipy_LAPACKE_zgesvd(kRowMajor, 'S', 'S', m, n, Ar.data(), n, sv.data(), s.U.data(), ldu,
                                     s.Vt.data(), n, sup.data()) != 0)
                throw std::runtime_error("zgesvd failed");
            for (int i = 0; i < ldu; ++i) {
                if (l2r) for (int j = 0; j < n; ++j) s.Vt[(size_t)i * n + j] *= sv[i];
                else for (int j = 0; j < m; ++j) s.U[(size_t)j * ldu + i] *= sv[i];
                svals.push_back(sv[i]);
            }
            secs.push_back(std::move(s));
        }
    std::sort(svals.begin(), svals.end(), std::greater<double>());
    SvdResult out;
    out.total = (int)svals.size();
    int add = sa_added(svals, max_dim, thres, beta, seeds);
    for (auto &s : secs) {
        Macro &rw = rows[s.r], &cl = cols[s.c];
        if (rw.kept <= 0 || cl.kept <= 0 || add == 0) continue;
        const int room = l2r ? rw.len - rw.kept : cl.len - cl.kept;
        if (room <= 0) continue;
        const int a = std::min(add, room);
        if (l2r) {
            gs_ortho(s.m, rw.kept, s.U, false, a, false, seeds);
            gs_ortho(cl.kept, s.n, s.Vt, true, a, true, seeds);
        } else {
            gs_ortho(s.m, rw.kept, s.U, false, a, true, seeds);
            gs_ortho(cl.kept, s.n, s.Vt, true, a, false, seeds);
        }
        rw.kept += a;
        cl.kept += a;
        s.ldu += a;
        add -= a;
    }
    out.kept_s = svals;
    const int left_dir = -1;
    out.U.rank = r1 + 1;
    out.V.rank = rank - r1 + 1;
    for (int i = 0; i < r1; ++i) out.U.dirs[i] = A.dirs[i];
    out.U.dirs[r1] = left_dir;
    out.V.dirs[0] = -left_dir;
    for (int i = r1; i < rank; ++i) out.V.dirs[i - r1 + 1] = A.dirs[i];
    for (auto &s : secs) {
        Macro &rw = rows[s.r], &cl = cols[s.c];
        if (rw.kept <= 0 || cl.kept <= 0) continue;
        for (auto &ra : rw.subs) {  // redist_row
            Block b;
            b.rank = r1 + 1;
            for (int i = 0; i < r1; ++i) { b.shape[i] = ra.shape[i]; b.qn[i] = ra.qn[i]; }
            b.shape[r1] = rw.kept;
            b.qn[r1] = -left_dir * rw.q;
            b.data.resize((size_t)ra.len * rw.kept);
            for (int i = 0; i < ra.len; ++i)
                for (int j = 0; j < rw.kept; ++j) b.data[(size_t)i * rw.kept + j] = s.U[(size_t)(ra.pos + i) * s.ldu + j];
            out.U.push_merge(b);
        }
        for (auto &ca : cl.subs) {  // redist_col
            Block b;
            b.rank = rank - r1 + 1;
            b.shape[0] = cl.kept;
            b.qn[0] = left_dir * cl.q;
            for (int i = 0; i < rank - r1; ++i) { b.shape[i + 1] = ca.shape[i]; b.qn[i + 1] = ca.qn[i]; }
            b.data.resize((size_t)ca.len * cl.kept);
            for (int j = 0; j < cl.kept; ++j)
                for (int c = 0; c < ca.len; ++c) b.data[(size_t)j * ca.len + c] = s.Vt[(size_t)j * s.n + ca.pos + c];
            out.V.push_merge(b);
        }
    }
    return out;
}

// --------------------------------------------------------------- TDVP
struct Tdvp {
    std::vector<Tensor> mps, mpo;
    std::vector<Tensor> envL, envR;
    double tol_svd, tol_exp, dt;
    int max_dim, max_iter;
    int window_at = -1;  // two-site L->R pass advanced to this site by kvo_tdvp_window (-1: not started)
    std::vector<double> sa_beta;  // SA-1TDVP widths per bond (kvo_tdvp_set_sa)
    std::mt19937 sa_seeds;        // the seed stream of the SA draws
};

Tensor boundary(int rank3_dirs0, int q) {
    Tensor t;
    t.rank = 3;
    t.dirs = {rank3_dirs0, -rank3_dirs0, -rank3_dirs0};
    Block b;
    b.rank = 3;
    b.shape = {1, 1, 1};
    b.qn = {q, 0, q};
    b.data = {cplx(1.0, 0.0)};
    t.blocks.push_back(b);
    return t;
}

// environment initialisation of TDVP::total_start (holstein/tdvp.h:303-316)
void tdvp_init(Tdvp &s) {
    const int ns = (int)s.mps.size();
    s.envL = {boundary(1, 0)};
    s.envR = {boundary(-1, s.mps[ns - 1].blocks.at(0).qn[2])};
    for (int i = ns - 1; i > 0; --i) s.envR.push_back(env_sweep(s.envR.back(), s.mps[i], s.mpo[i], false));
}

// TDVP::one_site (holstein/tdvp.h:78-141)
void one_site(Tdvp &s) {
    const int ns = (int)s.mps.size();
    for (int i = 0; i < ns; ++i) {
        local_krylov(1, s.envL.back(), s.mps[i], &s.mpo[i], nullptr, s.envR.back(), s.dt, s.max_iter, s.tol_exp, false);
        if (i < ns - 1) {
            SvdResult r = svd_impl(s.mps[i], 2, true, s.tol_svd, s.max_dim);
            s.mps[i] = std::move(r.U);
            s.envL.push_back(env_sweep(s.envL.back(), s.mps[i], s.mpo[i], true));
            local_krylov(0, s.envL.back(), r.V, nullptr, nullptr, s.envR.back(), s.dt, s.max_iter, s.tol_exp, true);
            s.mps[i + 1] = product(r.V, s.mps[i + 1], 1, OP_N, OP_N);
            s.envR.pop_back();
        }
    }
    for (int i = ns - 1; i >= 0; --i) {
        local_krylov(1, s.envL.back(), s.mps[i], &s.mpo[i], nullptr, s.envR.back(), s.dt, s.max_iter, s.tol_exp, false);
        if (i > 0) {
            SvdResult r = svd_impl(s.mps[i], 1, false, s.tol_svd, s.max_dim);
            s.mps[i] = std::move(r.V);
            s.envR.push_back(env_sweep(s.envR.back(), s.mps[i], s.mpo[i], false));
            local_krylov(0, s.envL.back(), r.U, nullptr, nullptr, s.envR.back(), s.dt, s.max_iter, s.tol_exp, true);
            s.mps[i - 1] = product(s.mps[i - 1], r.U, 1, OP_N, OP_N);
            s.envL.pop_back();
        }
    }
}

// TDVP::sa_site (holstein/tdvp.h:230-294): one_site with sa_svd_impl in
// place of svd_impl, bond i taking width beta[i]
void sa_site(Tdvp &s) {
    const int ns = (int)s.mps.size();
    if ((int)s.sa_beta.size() < ns - 1) throw std::runtime_error("SA-1TDVP needs one width per bond");
    for (int i = 0; i < ns; ++i) {
        local_krylov(1, s.envL.back(), s.mps[i], &s.mpo[i], nullptr, s.envR.back(), s.dt, s.max_iter, s.tol_exp, false);
        if (i < ns - 1) {
            SvdResult r = sa_svd_impl(s.mps[i], 2, true, s.tol_svd, s.max_dim, s.sa_beta[i], s.sa_seeds);
            s.mps[i] = std::move(r.U);
            s.envL.push_back(env_sweep(s.envL.back(), s.mps[i], s.mpo[i], true));
            local_krylov(0, s.envL.back(), r.V, nullptr, nullptr, s.envR.back(), s.dt, s.max_iter, s.tol_exp, true);
            s.mps[i + 1] = product(r.V, s.mps[i + 1], 1, OP_N, OP_N);
            s.envR.pop_back();
        }
    }
    for (int i = ns - 1; i >= 0; --i) {
        local_krylov(1, s.envL.back(), s.mps[i], &s.mpo[i], nullptr, s.envR.back(), s.dt, s.max_iter, s.tol_exp, false);
        if (i > 0) {
            SvdResult r = sa_svd_impl(s.mps[i], 1, false, s.tol_svd, s.max_dim, s.sa_beta[i - 1], s.sa_seeds);
            s.mps[i] = std::move(r.V);
            s.envR.push_back(env_sweep(s.envR.back(), s.mps[i], s.mpo[i], false));
            local_krylov(0, s.envL.back(), r.U, nullptr, nullptr, s.envR.back(), s.dt, s.max_iter, s.tol_exp, true);
            s.mps[i - 1] = product(s.mps[i - 1], r.U, 1, OP_N, OP_N);
            s.envL.pop_back();
        }
    }
}

// one local update of TDVP::two_site's left-to-right pass at sites (i, i+1)
// (holstein/tdvp.h:150-185)
void two_site_lr(Tdvp &s, int i) {
    const int ns = (int)s.mps.size();
    Tensor mm = product(s.mps[i], s.mps[i + 1], 1, OP_N, OP_N);
    local_krylov(2, s.envL.back(), mm, &s.mpo[i], &s.mpo[i + 1], s.envR.back(), s.dt, s.max_iter, s.tol_exp, false);
    SvdResult r = svd_impl(mm, 2, true, s.tol_svd, s.max_dim);
    if (i < ns - 2) {
        s.mps[i] = std::move(r.U);
        s.envL.push_back(env_sweep(s.envL.back(), s.mps[i], s.mpo[i], true));
        local_krylov(1, s.envL.back(), r.V, &s.mpo[i + 1], nullptr, s.envR.back(), s.dt, s.max_iter, s.tol_exp, true);
        s.mps[i + 1] = std::move(r.V);
        s.envR.pop_back();
    } else {
        s.mps[i] = std::move(r.U);
        s.mps[i + 1] = std::move(r.V);
    }
}

// TDVP::two_site (holstein/tdvp.h:144-227)
void two_site(Tdvp &s) {
    const int ns = (int)s.mps.size();
    s.envR.pop_back();
    for (int i = 0; i < ns - 1; ++i) two_site_lr(s, i);
    for (int i = ns - 1; i > 0; --i) {
        Tensor mm = product(s.mps[i - 1], s.mps[i], 1, OP_N, OP_N);
        local_krylov(2, s.envL.back(), mm, &s.mpo[i - 1], &s.mpo[i], s.envR.back(), s.dt, s.max_iter, s.tol_exp, false);
        SvdResult r = svd_impl(mm, 2, false, s.tol_svd, s.max_dim);
        if (i > 1) {
            s.mps[i] = std::move(r.V);
            s.envR.push_back(env_sweep(s.envR.back(), s.mps[i], s.mpo[i], false));
            local_krylov(1, s.envL.back(), r.U, &s.mpo[i - 1], nullptr, s.envR.back(), s.dt, s.max_iter, s.tol_exp, true);
            s.mps[i - 1] = std::move(r.U);
            s.envL.pop_back();
        } else {
            s.mps[i] = std::move(r.V);
            s.mps[i - 1] = std::move(r.U);
        }
    }
    s.envR.push_back(env_sweep(s.envR.back(), s.mps[1], s.mpo[1], false));
}

// Operator::join (holstein/operator.h:178-198)
cplx join(const std::vector<Tensor> &a, const std::vector<Tensor> &w, const std::vector<Tensor> &b) {
    Tensor env = boundary(1, 0);
    for (size_t i = 0; i < a.size(); ++i) env = env_sweep2(env, a[i], w[i], b[i]);
    if (env.blocks.empty()) return 0.0;
    const int q = env.blocks[0].qn[0];
    cplx r = 0.0;
    for (auto &blk : env.blocks)
        if (blk.rank == 3 && blk.shape[0] == 1 && blk.shape[1] == 1 && blk.shape[2] == 1 && blk.qn[0] == q &&
            blk.qn[1] == 0 && blk.qn[2] == q)
            r += blk.data[0];
    return r;
}

// ------------------------------------------------------- global Krylov
// The nK stage of TDVP::total_start (holstein/tdvp.h:318-327):
// global_main (holstein/krylov.h:199-283) on the MPO scaled by dt.
using State = std::vector<Tensor>;

Tensor boundary2(int dir0, int q) {  // rank-2 boundary environment {dir0, -dir0}, (q, q) = 1
    Tensor t;
    t.rank = 2;
    t.dirs = {dir0, -dir0};
    Block b;
    b.rank = 2;
    b.shape = {1, 1};
    b.qn = {q, q};
    b.data = {cplx(1.0, 0.0)};
    t.blocks.push_back(b);
    return t;
}

// leg dimension per charge of axis `ax`, from the blocks (holstein/tensor.h:187-196)
std::map<int, int> leg_dims(const Tensor &t, int ax) {
    std::map<int, int> m;
    for (auto &b : t.blocks) m[b.qn[ax]] = b.shape[ax];
    return m;
}

// b placed at offset `pos` inside a zero block of shape `sh` (holstein/block.h:181-197)
Block pad_block(const Block &b, const std::array<int, kMaxRank> &sh, const std::array<int, kMaxRank> &pos) {
    Block r;
    r.rank = b.rank;
    r.shape = sh;
    r.qn = b.qn;
    r.data.assign(r.size(), cplx(0.0, 0.0));
    std::array<size_t, kMaxRank> sd{}, rd{};
    sd[b.rank - 1] = rd[b.rank - 1] = 1;
    for (int i = b.rank - 2; i >= 0; --i) {
        sd[i] = sd[i + 1] * b.shape[i + 1];
        rd[i] = rd[i + 1] * sh[i + 1];
    }
    for (size_t e = 0; e < b.size(); ++e) {
        size_t dst = 0;
        for (int j = 0; j < b.rank; ++j) dst += ((e / sd[j]) % b.shape[j] + pos[j]) * rd[j];
        r.data[dst] = b.data[e];
    }
    return r;
}

// stack (holstein/tensor.h:262-317): direct sum of om2 into om1 on the legs
// in `ax`; om1's blocks keep offset 0, om2's go after om1's dimension of the
// same charge, equal keys merge.
void stack(Tensor &om1, const Tensor &om2, const std::vector<int> &ax) {
    std::vector<std::map<int, int>> comb(kMaxRank);
    for (int a : ax) {
        comb[a] = leg_dims(om1, a);
        for (auto &kv : leg_dims(om2, a)) comb[a][kv.first] += kv.second;
    }
    for (auto &b : om1.blocks) {
        std::array<int, kMaxRank> sh = b.shape, pos{};
        for (int a : ax) sh[a] = comb[a][b.qn[a]];
        if (sh != b.shape) b = pad_block(b, sh, pos);
    }
    for (auto &b : om2.blocks) {
        std::array<int, kMaxRank> sh = b.shape, pos{};
        for (int a : ax) {
            sh[a] = comb[a][b.qn[a]];
            pos[a] = sh[a] - b.shape[a];
        }
        om1.push_merge(sh != b.shape ? pad_block(b, sh, pos) : b);
    }
}

// State += (holstein/state.h:54-64)
void state_add(State &a, const State &b) {
    const int ns = (int)a.size();
    stack(a[0], b[0], {2});
    for (int i = 1; i < ns - 1; ++i) stack(a[i], b[i], {0, 2});
    stack(a[ns - 1], b[ns - 1], {0});
}

// overlap(State, State) (holstein/state.h:206-227)
cplx state_overlap(const State &s1, const State &s2) {
    Tensor env = boundary2(1, 0);
    for (size_t i = 0; i < s1.size(); ++i) env = product(s1[i], product(env, s2[i], 1, OP_N, OP_N), 2, OP_C, OP_N);
    if (env.blocks.empty()) return 0.0;
    const int q = env.blocks[0].qn[0];
    cplx r = 0.0;
    for (auto &b : env.blocks)
        if (b.shape[0] == 1 && b.shape[1] == 1 && b.qn[0] == q && b.qn[1] == q) r += b.data[0];
    return r;
}

// State::canonicalize (holstein/state.h:166-185)
void canonicalize(State &s, double tol, int maxd) {
    const int ns = (int)s.size();
    for (int i = 0; i < ns - 1; ++i) {
        SvdResult r = svd_impl(s[i], 2, true, tol, maxd);
        s[i] = std::move(r.U);
        s[i + 1] = product(r.V, s[i + 1], 1, OP_N, OP_N);
    }
    for (int i = ns - 1; i > 0; --i) {
        SvdResult r = svd_impl(s[i], 1, false, tol, maxd);
        s[i] = std::move(r.V);
        s[i - 1] = product(s[i - 1], r.U, 1, OP_N, OP_N);
    }
}

// env_mps_mpo(..., Chk = true) (holstein/product.h:278-319): equal blocks merged
Tensor env_mps_mpo_merged(const Tensor &env, const Tensor &mps, const Tensor &mpo) {
    Tensor raw = env_mps_mpo(env, mps, mpo), r;
    r.rank = raw.rank;
    r.dirs = raw.dirs;
    for (auto &b : raw.blocks) r.push_merge(b);
    return r;
}

// apply_operator (holstein/operator.h:232-269)
State apply_operator(const State &op, const State &wf, double tol, int maxd) {
    const int ns = (int)op.size();
    Tensor envl = boundary(1, 0);
    State res(ns);
    const int lastB = wf[ns - 1].blocks.at(0).qn[2], lastw = op[ns - 1].blocks.at(0).qn[3];
    for (int i = 0; i < ns; ++i) {
        Tensor lmo = env_mps_mpo_merged(envl, wf[i], op[i]);
        if (i == ns - 1) {
            Tensor envr = boundary(-1, lastB);
            envr.blocks[0].qn = {lastB, lastw, lastB};
            res[i] = product(lmo, envr, 2, OP_N, OP_T);
        } else {
            SvdResult r = svd_impl(lmo, 2, true, tol, maxd);
            res[i] = std::move(r.U);
            envl = std::move(r.V);
        }
    }
    for (int i = ns - 1; i > 0; --i) {
        SvdResult r = svd_impl(res[i], 1, false, tol, maxd);
        res[i] = std::move(r.V);
        res[i - 1] = product(res[i - 1], r.U, 1, OP_N, OP_N);
    }
    return res;
}

// apply_ortho_site (holstein/krylov.h:13-45): Nh minus its projection on La, Lb
Tensor apply_ortho_site(const Tensor &Nh, const Tensor &La, const Tensor &Lb) {
    const cplx LNa = overlap(La, Nh), LNb = overlap(Lb, Nh);
    const cplx aa = std::pow(tnorm(La), 2.0), bb = std::pow(tnorm(Lb), 2.0);
    const cplx ab = overlap(La, Lb), ba = std::conj(ab);
    const cplx cc = ab * ba - aa * bb;
    Tensor res = Nh;
    if (std::abs(cc) < 1e-17) {
        if (std::abs(aa) < 1e-17) return res;
        add_scaled(res, La, -1.0 * LNa / aa);
    } else {
        add_scaled(res, La, (bb * LNa - ab * LNb) / cc);
        add_scaled(res, Lb, (aa * LNb - ba * LNa) / cc);
    }
    return res;
}

// 4-argument env_sweep (holstein/product.h:505-521), both directions
Tensor env_sweep4(const Tensor &env, const Tensor &a1, const Tensor &W, const Tensor &a2, bool l2r) {
    if (l2r) return env_sweep2(env, a1, W, a2);
    return env_sweep2(env, transpose(a1, {2, 1, 0}), transpose(W, {0, 3, 2, 1}), transpose(a2, {2, 1, 0}));
}

// 2-leg env_sweep <a1|a2> (holstein/product.h:523-538), both directions
Tensor env_state(const Tensor &env, const Tensor &a1, const Tensor &a2, bool l2r) {
    if (l2r) return product(a1, product(env, a2, 1, OP_N, OP_N), 2, OP_C, OP_N);
    return env_state(env, transpose(a1, {2, 1, 0}), transpose(a2, {2, 1, 0}), true);
}

// apply_double_state (holstein/krylov.h:125-131)
Tensor apply_double_state(const Tensor &envl, const Tensor &M, const Tensor &envr) {
    return product(product(envl, M, 1, OP_N, OP_N), envr, 1, OP_N, OP_T);
}

// apply_ortho(H, Va) (holstein/krylov.h:133-142)
State apply_ortho1(const State &H, const State &Va, double tol, int maxd) {
    State gss = apply_operator(H, Va, tol, maxd);
    const cplx ovp = state_overlap(gss, Va);
    State vac = Va;
    scale(vac[0], -1.0 * ovp);
    state_add(gss, vac);
    canonicalize(gss, 0.0, 1000);
    return gss;
}

// apply_ortho(H, Va, Vb) (holstein/krylov.h:145-197): H Va minus its
// components on Va and Vb, fitted two sites at a time, both directions
State apply_ortho2(const State &H, const State &Va, const State &Vb, double tol, int maxd) {
    const int ns = (int)H.size();
    State gss = apply_operator(H, Va, tol, maxd);
    const int tot = gss[ns - 1].blocks.at(0).qn[2];
    std::vector<Tensor> eLH = {boundary(1, 0)}, eRH = {boundary(-1, tot)};
    std::vector<Tensor> eLa = {boundary2(1, 0)}, eRa = {boundary2(-1, tot)};
    std::vector<Tensor> eLb = {boundary2(1, 0)}, eRb = {boundary2(-1, tot)};
    for (int i = ns - 1; i > 1; --i) {  // init_env_op / init_env_state (holstein/krylov.h:48-94)
        eRH.push_back(env_sweep4(eRH.back(), gss[i], H[i], Va[i], false));
        eRa.push_back(env_state(eRa.back(), gss[i], Va[i], false));
        eRb.push_back(env_state(eRb.back(), gss[i], Vb[i], false));
    }
    auto site = [&](int a, int b, bool l2r) {
        Tensor Ta = product(Va[a], Va[b], 1, OP_N, OP_N), Tb = product(Vb[a], Vb[b], 1, OP_N, OP_N);
        Tensor Nh = apply_double(eLH.back(), Ta, H[a], H[b], eRH.back());
        Tensor La = apply_double_state(eLa.back(), Ta, eRa.back());
        Tensor Lb = apply_double_state(eLb.back(), Tb, eRb.back());
        SvdResult r = svd_impl(apply_ortho_site(Nh, La, Lb), 2, l2r, tol, maxd);
        gss[a] = std::move(r.U);
        gss[b] = std::move(r.V);
    };
    for (int i = 0; i < ns - 1; ++i) {
        site(i, i + 1, true);
        if (i < ns - 2) {  // update_env_op / update_env_state (holstein/krylov.h:97-124)
            eLH.push_back(env_sweep4(eLH.back(), gss[i], H[i], Va[i], true));
            eLa.push_back(env_state(eLa.back(), gss[i], Va[i], true));
            eLb.push_back(env_state(eLb.back(), gss[i], Vb[i], true));
            eRH.pop_back();
            eRa.pop_back();
            eRb.pop_back();
        }
    }
    for (int i = ns - 1; i > 0; --i) {
        site(i - 1, i, false);
        if (i > 1) {
            eRH.push_back(env_sweep4(eRH.back(), gss[i], H[i], Va[i], false));
            eRa.push_back(env_state(eRa.back(), gss[i], Va[i], false));
            eRb.push_back(env_state(eRb.back(), gss[i], Vb[i], false));
            eLH.pop_back();
            eLa.pop_back();
            eLb.pop_back();
        }
    }
    return gss;
}

// global_main (holstein/krylov.h:199-283): Krylov basis of MPSs with the MPO
// (already scaled by dt), exp(-i Hm) e0 on the Hessenberg matrix of joins,
// mps = sum_i c_i V_i with a canonicalisation after every addition
void global_main(const State &Hc, State &mps, int max_iter, double tol_exp, double tol_svd, int maxd) {
    scale(mps[0], 1.0 / tnorm(mps[0]));
    std::vector<State> Vm = {mps};
    int k = 0;
    double err = 1.0;
    while (k < max_iter - 1 && err > tol_exp) {
        State hv = k > 0 ? apply_ortho2(Hc, Vm[k], Vm[k - 1], tol_svd, maxd) : apply_ortho1(Hc, Vm[k], tol_svd, maxd);
        const double nmhv = tnorm(hv[0]);
        err *= nmhv;
        if (err < tol_exp || nmhv > 1.0) break;
        scale(hv[0], 1.0 / nmhv);
        Vm.push_back(std::move(hv));
        ++k;
    }
    const int ld = (int)Vm.size();
    std::vector<cplx> Hm((size_t)ld * ld, cplx(0.0, 0.0)), c(ld, cplx(0.0, 0.0));
    std::vector<double> ev(ld);
    for (int i = 0; i < ld; ++i) {
        Hm[(size_t)i * ld + i] = join(Vm[i], Hc, Vm[i]);
        if (i < ld - 1) Hm[(size_t)i * ld + i + 1] = join(Vm[i], Hc, Vm[i + 1]);
    }
    if (scipy_LAPACKE_zheevd(kRowMajor, 'V', 'U', ld, Hm.data(), ld, ev.data()) != 0)
        throw std::runtime_error("zheevd failed");
    const cplx img(0.0, -1.0);
    for (int i = 0; i < ld; ++i)
        for (int j = 0; j < ld; ++j) c[i] += Hm[(size_t)i * ld + j] * std::exp(img * ev[j]) * std::conj(Hm[j]);
    mps = Vm[0];
    scale(mps[0], c[0]);
    for (int i = 1; i < ld; ++i) {
        State t = Vm[i];
        scale(t[0], c[i]);
        state_add(mps, t);
        canonicalize(mps, tol_svd, maxd);
    }
}

// one step of the nK stage: the MPO scaled by dt on its first site
// (Operator::operator*=, holstein/operator.h:66-70).  Deviation: the sweep
// driver's environments are rebuilt from the new state afterwards.
// total_start builds them once, before this stage (holstein/tdvp.h:303-316),
// so its first sweep after a global step contracts the new MPS with
// environments of the old one; that result depends on the phases of the
// singular vectors the step leaves, which rounding decides.
void global_step(Tdvp &s) {
    State Hc = s.mpo;
    scale(Hc[0], s.dt);
    global_main(Hc, s.mps, s.max_iter, s.tol_exp, s.tol_svd, s.max_dim);
    tdvp_init(s);
}

thread_local std::string g_err;

template <class F>
int guarded(F &&f) {
    try {
        f();
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return 1;
    }
}

}  // namespace

// =================================================================== C API
extern "C" {

const char *kvo_last_error() { return g_err.c_str(); }

// complex-GEMM flops (8*M*N*K) issued since the last reset
double kvo_flops(int reset) {
    double f = g_flops;
    if (reset) g_flops = 0.0;
    return f;
}

int kvo_tensor_new(int rank, const int *dirs, int nblocks, const int *shapes, const int *qns,
                   const double *data, void **out) {
    return guarded([&] {
        if (rank < 1 || rank > kMaxRank) throw std::runtime_error("bad rank");
        auto *t = new Tensor;
        t->rank = rank;
        for (int i = 0; i < rank; ++i) t->dirs[i] = dirs[i];
        size_t off = 0;
        for (int b = 0; b < nblocks; ++b) {
            Block blk;
            blk.rank = rank;
            for (int i = 0; i < rank; ++i) { blk.shape[i] = shapes[b * rank + i]; blk.qn[i] = qns[b * rank + i]; }
            blk.data.resize(blk.size());
            for (size_t e = 0; e < blk.size(); ++e) blk.data[e] = cplx(data[2 * (off + e)], data[2 * (off + e) + 1]);
            off += blk.size();
            t->blocks.push_back(std::move(blk));
        }
        *out = t;
    });
}

int kvo_tensor_info(void *h, int *rank, int *nblocks, long long *nelem) {
    auto *t = static_cast<Tensor *>(h);
    *rank = t->rank;
    *nblocks = (int)t->blocks.size();
    long long n = 0;
    for (auto &b : t->blocks) n += (long long)b.size();
    *nelem = n;
    return 0;
}

int kvo_tensor_get(void *h, int *dirs, int *shapes, int *qns, double *data) {
    auto *t = static_cast<Tensor *>(h);
    for (int i = 0; i < t->rank; ++i) dirs[i] = t->dirs[i];
    size_t off = 0;
    for (size_t b = 0; b < t->blocks.size(); ++b) {
        auto &blk = t->blocks[b];
        for (int i = 0; i < t->rank; ++i) { shapes[b * t->rank + i] = blk.shape[i]; qns[b * t->rank + i] = blk.qn[i]; }
        std::memcpy(data + 2 * off, blk.data.data(), blk.size() * sizeof(cplx));
        off += blk.size();
    }
    return 0;
}

void kvo_tensor_free(void *h) { delete static_cast<Tensor *>(h); }

int kvo_product(void *a, void *b, int nc, int ta, int tb, void **out) {
    return guarded([&] {
        *out = new Tensor(product(*static_cast<Tensor *>(a), *static_cast<Tensor *>(b), nc, (Op)ta, (Op)tb));
    });
}

int kvo_apply(int nsite, void *L, void *psi, void *W1, void *W2, void *R, void **out) {
    return guarded([&] {
        auto &l = *static_cast<Tensor *>(L);
        auto &p = *static_cast<Tensor *>(psi);
        auto &r = *static_cast<Tensor *>(R);
        Tensor res = nsite == 0 ? apply_zero(l, p, r)
                   : nsite == 1 ? apply_single(l, p, *static_cast<Tensor *>(W1), r)
                                : apply_double(l, p, *static_cast<Tensor *>(W1), *static_cast<Tensor *>(W2), r);
        *out = new Tensor(std::move(res));
    });
}

int kvo_env_sweep(void *env, void *A, void *W, int l2r, void **out) {
    return guarded([&] {
        *out = new Tensor(env_sweep(*static_cast<Tensor *>(env), *static_cast<Tensor *>(A),
                                    *static_cast<Tensor *>(W), l2r != 0));
    });
}

int kvo_local_krylov(int nsite, void *L, void *psi, void *W1, void *W2, void *R, double dt, int max_iter,
                     double tol, int reverse, int *iters, void **out) {
    return guarded([&] {
        Tensor p = *static_cast<Tensor *>(psi);
        KrylovExit ex = local_krylov(nsite, *static_cast<Tensor *>(L), p, static_cast<Tensor *>(W1),
                                     static_cast<Tensor *>(W2), *static_cast<Tensor *>(R), dt, max_iter, tol,
                                     reverse != 0);
        *iters = ex.iters;
        *out = new Tensor(std::move(p));
    });
}

int kvo_svd(void *A, int r1, int l2r, double tol, int max_dim, void **U, void **V, double *svals,
            int *nkept, int *ntotal) {
    return guarded([&] {
        SvdResult r = svd_impl(*static_cast<Tensor *>(A), r1, l2r != 0, tol, max_dim);
        *U = new Tensor(std::move(r.U));
        *V = new Tensor(std::move(r.V));
        *nkept = (int)r.kept_s.size();
        *ntotal = r.total;
        if (svals) std::memcpy(svals, r.kept_s.data(), r.kept_s.size() * sizeof(double));
    });
}

int kvo_tdvp_new(int ns, void **mps, void **mpo, double tol_svd, double tol_exp, int max_dim, int max_iter,
                 double dt, void **out) {
    return guarded([&] {
        auto *s = new Tdvp;
        for (int i = 0; i < ns; ++i) {
            s->mps.push_back(*static_cast<Tensor *>(mps[i]));
            s->mpo.push_back(*static_cast<Tensor *>(mpo[i]));
        }
        s->tol_svd = tol_svd;
        s->tol_exp = tol_exp;
        s->max_dim = max_dim;
        s->max_iter = max_iter;
        s->dt = dt;
        tdvp_init(*s);
        *out = s;
    });
}

int kvo_tdvp_sweep(void *h, int mode) {
    return guarded([&] {
        auto *s = static_cast<Tdvp *>(h);
        if (s->window_at >= 0) throw std::runtime_error("the handle is inside a timed window; it cannot sweep");
        if (mode == 1) one_site(*s);
        else if (mode == 2) two_site(*s);
        else if (mode == 0) global_step(*s);
        else if (mode == 3) sa_site(*s);
        else throw std::runtime_error("mode must be 0, 1, 2 or 3");
    });
}

// SA-1TDVP widths (one per bond: beta, as betaSet holds it) and the seed of
// the generator every SA draw comes from
int kvo_tdvp_set_sa(void *h, const double *beta, int nbeta, unsigned long long seed) {
    return guarded([&] {
        auto *s = static_cast<Tdvp *>(h);
        s->sa_beta.assign(beta, beta + nbeta);
        s->sa_seeds.seed((std::mt19937::result_type)seed);
    });
}

// Timing hook of the CPU baseline (no reference counterpart): the two-site
// left-to-right pass is advanced (once, untimed) to site i0, then n local
// updates from there are run on a copy of that state and timed; the handle
// stays at i0, so every call with the same (i0, n) repeats the same work.
int kvo_tdvp_window(void *h, int i0, int n, double *seconds) {
    return guarded([&] {
        auto *s = static_cast<Tdvp *>(h);
        const int ns = (int)s->mps.size();
        if (n < 1 || i0 < 0 || i0 + n > ns - 2) throw std::runtime_error("window outside the two-site pass");
        if (s->window_at < 0) {
            s->envR.pop_back();
            s->window_at = 0;
        }
        if (i0 < s->window_at) throw std::runtime_error("window behind the pass already advanced");
        for (; s->window_at < i0; ++s->window_at) two_site_lr(*s, s->window_at);
        Tdvp c = *s;
        const auto t0 = std::chrono::steady_clock::now();
        for (int i = i0; i < i0 + n; ++i) two_site_lr(c, i);
        *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    });
}

int kvo_tdvp_site(void *h, int i, void **out) {
    return guarded([&] { *out = new Tensor(static_cast<Tdvp *>(h)->mps.at(i)); });
}

void kvo_tdvp_free(void *h) { delete static_cast<Tdvp *>(h); }

int kvo_join(int ns, void **a, void **w, void **b, double *re, double *im) {
    return guarded([&] {
        std::vector<Tensor> va, vw, vb;
        for (int i = 0; i < ns; ++i) {
            va.push_back(*static_cast<Tensor *>(a[i]));
            vw.push_back(*static_cast<Tensor *>(w[i]));
            vb.push_back(*static_cast<Tensor *>(b[i]));
        }
        cplx r = join(va, vw, vb);
        *re = r.real();
        *im = r.imag();
    });
}

}  // extern "C"
