// Global-Krylov stage (the nK stage of TDVP::total_start,
// holstein/tdvp.h:318-327): a Krylov basis of whole MPSs built with the MPO
// scaled by dt (global_main, holstein/krylov.h:199-283), each new vector the
// MPO applied to the last with compression (apply_operator,
// holstein/operator.h:232-269) and made orthogonal to the previous two by a
// two-site fitting sweep (apply_ortho, holstein/krylov.h:133-197); the state
// becomes sum_i c_i V_i, c = exp(-i Hm) e0 on the matrix of joins.
//
// Everything runs on the device through the engine's block-sparse products,
// MPO mixing, permutations, SVD and H_eff apply; the kernels below add the
// whole-tensor pieces the stage needs: scaling, overlaps in a fixed
// reduction order, scaled accumulation with the reference's merge rule, and
// the direct sum of two tensors (State::operator+=).  The host reads back
// only the scalars the reference's control flow branches on.
#include <map>

#include "kv_engine.h"

namespace kv {

namespace {

using State = std::vector<TensorP>;
constexpr int kN = KV_OP_N, kT = KV_OP_T, kC = KV_OP_C;
constexpr int GT = 256;

int grid(int64_t n) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + GT - 1) / GT, (int64_t)ctx().num_sms * 8));
}

__global__ void k_scale_c(const double2 *__restrict__ in, double2 *__restrict__ out, int64_t n, double sr,
                          double si) {
    for (int64_t i = blockIdx.x * (int64_t)GT + threadIdx.x; i < n; i += (int64_t)gridDim.x * GT) {
        const double2 v = in[i];
        out[i] = make_double2(sr * v.x - si * v.y, sr * v.y + si * v.x);
    }
}

// parts[p] = sum_i conj(B[b_off + i]) A[a_off + i] over pair p's block; one
// CTA per pair, a fixed-order tree in shared memory
__global__ void __launch_bounds__(GT) k_pair_dot(const int64_t *__restrict__ desc, const double2 *__restrict__ A,
                                                 const double2 *__restrict__ B, double2 *__restrict__ parts) {
    __shared__ double2 red[GT];
    const int64_t ao = desc[3 * blockIdx.x], bo = desc[3 * blockIdx.x + 1], n = desc[3 * blockIdx.x + 2];
    double sr = 0.0, si = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += GT) {
        const double2 a = A[ao + i], b = B[bo + i];
        sr += b.x * a.x + b.y * a.y;
        si += b.x * a.y - b.y * a.x;
    }
    red[threadIdx.x] = make_double2(sr, si);
    __syncthreads();
    for (int o = GT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            red[threadIdx.x].x += red[threadIdx.x + o].x;
            red[threadIdx.x].y += red[threadIdx.x + o].y;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) parts[blockIdx.x] = red[0];
}

// out[dst + i] += (ar + i ai) in[src + i] for each (src, dst, size) triple; one CTA per block
__global__ void __launch_bounds__(GT) k_pair_axpy(const int64_t *__restrict__ desc, const double2 *__restrict__ in,
                                                  double2 *__restrict__ out, double ar, double ai) {
    const int64_t so = desc[3 * blockIdx.x], dst = desc[3 * blockIdx.x + 1], n = desc[3 * blockIdx.x + 2];
    for (int64_t i = threadIdx.x; i < n; i += GT) {
        const double2 v = in[so + i];
        double2 &o = out[dst + i];
        o.x += ar * v.x - ai * v.y;
        o.y += ar * v.y + ai * v.x;
    }
}

// a block placed at offset `pos` inside a larger (zeroed) block of the same rank
struct Embed {
    int64_t src_off, dst_off, size;
    int rank;
    int sshape[kMaxRank], dshape[kMaxRank], pos[kMaxRank];
};

__global__ void __launch_bounds__(GT) k_embed_add(const Embed *__restrict__ em, const double2 *__restrict__ in,
                                                  double2 *__restrict__ out) {
    const Embed e = em[blockIdx.x];
    for (int64_t i = threadIdx.x; i < e.size; i += GT) {
        int64_t rem = i, dst = 0, stride = 1;
        for (int d = e.rank - 1; d >= 0; --d) {
            const int64_t c = rem % e.sshape[d];
            rem /= e.sshape[d];
            dst += (c + e.pos[d]) * stride;
            stride *= e.dshape[d];
        }
        const double2 v = in[e.src_off + i];
        double2 &o = out[e.dst_off + dst];
        o.x += v.x;
        o.y += v.y;
    }
}

void check_launch() {
    counted();
    KV_CUDA(cudaGetLastError());
}

TensorP tscale(const DTensor &t, cplx s) { return op_scale(t, s); }

// overlap(ori, oth) = sum over blocks of equal shape and charges of
// <oth|ori> (holstein/tensor.h:221-237); partial sums per block, added on the
// host in block order
cplx toverlap(const DTensor &ori, const DTensor &oth) {
    std::vector<int64_t> desc;
    for (auto &a : ori.meta.blocks) {
        const int j = oth.meta.find(a);
        if (j >= 0) desc.insert(desc.end(), {a.off, oth.meta.blocks[j].off, a.size});
    }
    const int np = (int)(desc.size() / 3);
    if (np == 0) return 0.0;
    DevBuf d = upload_vec(desc), parts((size_t)np * sizeof(double2));
    k_pair_dot<<<np, GT, 0, ctx().stream>>>(d.as<int64_t>(), ori.data(), oth.data(), parts.as<double2>());
    check_launch();
    std::vector<double2> h(np);
    KV_CUDA(cudaMemcpyAsync(h.data(), parts.p, np * sizeof(double2), cudaMemcpyDeviceToHost, ctx().stream));
    KV_CUDA(cudaStreamSynchronize(ctx().stream));
    cplx r = 0.0;
    for (auto &x : h) r += cplx(x.x, x.y);
    return r;
}

double tnorm(const DTensor &t) { return std::sqrt(std::max(0.0, toverlap(t, t).real())); }

TensorP add_scaled(const DTensor &t, const DTensor &s, cplx v) { return op_add_scaled(t, s, v); }

}  // namespace

// t + v s with the merge rule of push_back_ch (holstein/tensor.h:172-185):
// blocks of t in order, then the new keys of s appended
TensorP op_add_scaled(const DTensor &t, const DTensor &s, cplx v) {
    Meta m = t.meta;
    for (auto &b : s.meta.blocks) m.add(b);
    auto out = DTensor::make(m, true);
    for (int pass = 0; pass < 2; ++pass) {
        const DTensor &x = pass == 0 ? t : s;
        const cplx f = pass == 0 ? cplx(1.0, 0.0) : v;
        std::vector<int64_t> desc;
        for (auto &b : x.meta.blocks) desc.insert(desc.end(), {b.off, out->meta.blocks[out->meta.find(b)].off, b.size});
        if (desc.empty()) continue;
        DevBuf d = upload_vec(desc);
        k_pair_axpy<<<(unsigned)(desc.size() / 3), GT, 0, ctx().stream>>>(d.as<int64_t>(), x.data(), out->data(),
                                                                          f.real(), f.imag());
        check_launch();
    }
    return out;
}

namespace {

std::map<int, int> leg_dims(const Meta &m, int ax) {
    std::map<int, int> r;
    for (auto &b : m.blocks) r[b.qn[ax]] = b.shape[ax];
    return r;
}

// stack (holstein/tensor.h:262-317): the direct sum of om1 and om2 on the legs
// in `ax`; om1's blocks at offset 0, om2's after om1's dimension of their
// charge, equal keys merged
TensorP stack(const DTensor &om1, const DTensor &om2, const std::vector<int> &ax) {
    std::vector<std::map<int, int>> comb(kMaxRank);
    for (int a : ax) {
        comb[a] = leg_dims(om1.meta, a);
        for (auto &kv : leg_dims(om2.meta, a)) comb[a][kv.first] += kv.second;
    }
    Meta m;
    m.rank = om1.meta.rank;
    m.dirs = om1.meta.dirs;
    std::vector<Embed> em;
    auto place = [&](const DTensor &x, bool second) {
        for (auto &b : x.meta.blocks) {
            BlockMeta o;
            o.shape = b.shape;
            o.qn = b.qn;
            Embed e{};
            e.src_off = b.off;
            e.size = b.size;
            e.rank = m.rank;
            for (int i = 0; i < m.rank; ++i) {
                e.sshape[i] = b.shape[i];
                e.pos[i] = 0;
            }
            for (int a : ax) {
                o.shape[a] = comb[a][b.qn[a]];
                if (second) e.pos[a] = o.shape[a] - b.shape[a];
            }
            for (int i = 0; i < m.rank; ++i) e.dshape[i] = o.shape[i];
            e.dst_off = m.add(o);  // block index for now
            em.push_back(e);
        }
    };
    place(om1, false);
    place(om2, true);
    auto out = DTensor::make(m, true);
    for (auto &e : em) e.dst_off = out->meta.blocks[e.dst_off].off;
    const size_t n1 = om1.meta.blocks.size();
    for (int pass = 0; pass < 2; ++pass) {  // om1 first, then om2 (accumulating)
        std::vector<Embed> part(em.begin() + (pass ? n1 : 0), pass ? em.end() : em.begin() + n1);
        if (part.empty()) continue;
        DevBuf d = upload_vec(part);
        k_embed_add<<<(unsigned)part.size(), GT, 0, ctx().stream>>>(d.as<Embed>(), (pass ? om2 : om1).data(),
                                                                    out->data());
        check_launch();
    }
    return out;
}

TensorP boundary3(int dir0, int q0, int q1, int q2) {
    TensorP t = boundary_env(dir0, q0);
    t->meta.blocks[0].qn = {q0, q1, q2};
    t->meta.rebuild_index();
    return t;
}

TensorP boundary2(int dir0, int q) {
    Meta m;
    m.rank = 2;
    m.dirs = {dir0, -dir0};
    BlockMeta b;
    b.shape = {1, 1};
    b.qn = {q, q};
    m.blocks.push_back(b);
    auto t = DTensor::make(m, false);
    const double2 one = make_double2(1.0, 0.0);
    upload_bytes(t->data(), &one, sizeof(one));
    return t;
}

TensorP P(const DTensor &a, const DTensor &b, int nc, int oa, int ob, int prec) {
    return op_product(a, b, nc, oa, ob, prec);
}

// State::operator+= (holstein/state.h:54-64)
State state_add(const State &a, const State &b) {
    const int ns = (int)a.size();
    State r(ns);
    r[0] = stack(*a[0], *b[0], {2});
    for (int i = 1; i < ns - 1; ++i) r[i] = stack(*a[i], *b[i], {0, 2});
    r[ns - 1] = stack(*a[ns - 1], *b[ns - 1], {0});
    return r;
}

// overlap(State, State) (holstein/state.h:206-227)
cplx state_overlap(const State &s1, const State &s2, int prec) {
    TensorP env = boundary2(1, 0);
    for (size_t i = 0; i < s1.size(); ++i) env = P(*s1[i], *P(*env, *s2[i], 1, kN, kN, prec), 2, kC, kN, prec);
    if (env->meta.blocks.empty()) return 0.0;
    const int q = env->meta.blocks[0].qn[0];
    TensorP ref = boundary2(1, q);
    ref->meta.dirs = env->meta.dirs;
    return toverlap(*env, *ref);
}

State scaled_first(const State &s, cplx v) {
    State r = s;
    r[0] = tscale(*s[0], v);
    return r;
}

// env_mps_mpo(env, mps, mpo, true) (holstein/product.h:278-319): equal output blocks merged
TensorP env_mps_mpo_merged(const DTensor &env, const DTensor &mps, const DTensor &mpo, int prec) {
    return op_mix(*P(env, mps, 1, kN, kN, prec), mpo, 1);
}

// apply_operator (holstein/operator.h:232-269)
State apply_operator(const State &op, const State &wf, double tol, int maxd, int prec) {
    const int ns = (int)op.size();
    TensorP envl = boundary_env(1, 0);
    State res(ns);
    const int lastB = wf[ns - 1]->meta.blocks.at(0).qn[2], lastw = op[ns - 1]->meta.blocks.at(0).qn[3];
    for (int i = 0; i < ns; ++i) {
        TensorP lmo = env_mps_mpo_merged(*envl, *wf[i], *op[i], prec);
        if (i == ns - 1) {
            res[i] = P(*lmo, *boundary3(-1, lastB, lastw, lastB), 2, kN, kT, prec);
        } else {
            SvdOut r = op_svd(*lmo, 2, true, tol, maxd, prec);
            res[i] = r.U;
            envl = r.V;
        }
    }
    for (int i = ns - 1; i > 0; --i) {
        SvdOut r = op_svd(*res[i], 1, false, tol, maxd, prec);
        res[i] = r.V;
        res[i - 1] = P(*res[i - 1], *r.U, 1, kN, kN, prec);
    }
    return res;
}

// apply_ortho_site (holstein/krylov.h:13-45)
TensorP apply_ortho_site(const TensorP &Nh, const DTensor &La, const DTensor &Lb) {
    const cplx LNa = toverlap(La, *Nh), LNb = toverlap(Lb, *Nh);
    const cplx aa = std::pow(tnorm(La), 2.0), bb = std::pow(tnorm(Lb), 2.0);
    const cplx ab = toverlap(La, Lb), ba = std::conj(ab);
    const cplx cc = ab * ba - aa * bb;
    if (std::abs(cc) < 1e-17) {
        if (std::abs(aa) < 1e-17) return Nh;
        return add_scaled(*Nh, La, -1.0 * LNa / aa);
    }
    TensorP r = add_scaled(*Nh, La, (bb * LNa - ab * LNb) / cc);
    return add_scaled(*r, Lb, (aa * LNb - ba * LNa) / cc);
}

// apply_double (holstein/product.h:478-486) as a plain chain of products and
// mixes: here the bra and ket states differ, so the apply maps one block
// structure to another
TensorP apply_double(const DTensor &L, const DTensor &M, const DTensor &W1, const DTensor &W2, const DTensor &R,
                     int prec) {
    TensorP o = op_mix(*op_mix(*P(L, M, 1, kN, kN, prec), W1, 1), W2, 2);
    return P(*o, R, 2, kN, kT, prec);
}

// 4-argument env_sweep (holstein/product.h:505-521)
TensorP env4(const DTensor &env, const DTensor &a1, const DTensor &W, const DTensor &a2, bool l2r, int prec) {
    if (!l2r)
        return env4(env, *op_permute(a1, {2, 1, 0}), *op_permute(W, {0, 3, 2, 1}), *op_permute(a2, {2, 1, 0}),
                    true, prec);
    return P(a1, *op_mix(*P(env, a2, 1, kN, kN, prec), W, 1), 2, kC, kN, prec);
}

// two-leg env_sweep <a1|a2> (holstein/product.h:523-538)
TensorP env_state(const DTensor &env, const DTensor &a1, const DTensor &a2, bool l2r, int prec) {
    if (!l2r) return env_state(env, *op_permute(a1, {2, 1, 0}), *op_permute(a2, {2, 1, 0}), true, prec);
    return P(a1, *P(env, a2, 1, kN, kN, prec), 2, kC, kN, prec);
}

// apply_ortho(H, Va) (holstein/krylov.h:133-142)
State apply_ortho1(const State &H, const State &Va, double tol, int maxd, int prec) {
    State gss = apply_operator(H, Va, tol, maxd, prec);
    const cplx ovp = state_overlap(gss, Va, prec);
    return op_canonicalize(state_add(gss, scaled_first(Va, -1.0 * ovp)), 0.0, 1000, prec);
}

// apply_ortho(H, Va, Vb) (holstein/krylov.h:145-197)
State apply_ortho2(const State &H, const State &Va, const State &Vb, double tol, int maxd, int prec) {
    const int ns = (int)H.size();
    State gss = apply_operator(H, Va, tol, maxd, prec);
    const int tot = gss[ns - 1]->meta.blocks.at(0).qn[2];
    std::vector<TensorP> eLH = {boundary_env(1, 0)}, eRH = {boundary_env(-1, tot)};
    std::vector<TensorP> eLa = {boundary2(1, 0)}, eRa = {boundary2(-1, tot)};
    std::vector<TensorP> eLb = {boundary2(1, 0)}, eRb = {boundary2(-1, tot)};
    for (int i = ns - 1; i > 1; --i) {
        eRH.push_back(env4(*eRH.back(), *gss[i], *H[i], *Va[i], false, prec));
        eRa.push_back(env_state(*eRa.back(), *gss[i], *Va[i], false, prec));
        eRb.push_back(env_state(*eRb.back(), *gss[i], *Vb[i], false, prec));
    }
    auto site = [&](int a, int b, bool l2r) {
        TensorP Ta = P(*Va[a], *Va[b], 1, kN, kN, prec), Tb = P(*Vb[a], *Vb[b], 1, kN, kN, prec);
        TensorP Nh = apply_double(*eLH.back(), *Ta, *H[a], *H[b], *eRH.back(), prec);
        TensorP La = P(*P(*eLa.back(), *Ta, 1, kN, kN, prec), *eRa.back(), 1, kN, kT, prec);
        TensorP Lb = P(*P(*eLb.back(), *Tb, 1, kN, kN, prec), *eRb.back(), 1, kN, kT, prec);
        SvdOut r = op_svd(*apply_ortho_site(Nh, *La, *Lb), 2, l2r, tol, maxd, prec);
        gss[a] = r.U;
        gss[b] = r.V;
    };
    for (int i = 0; i < ns - 1; ++i) {
        site(i, i + 1, true);
        if (i < ns - 2) {
            eLH.push_back(env4(*eLH.back(), *gss[i], *H[i], *Va[i], true, prec));
            eLa.push_back(env_state(*eLa.back(), *gss[i], *Va[i], true, prec));
            eLb.push_back(env_state(*eLb.back(), *gss[i], *Vb[i], true, prec));
            eRH.pop_back();
            eRa.pop_back();
            eRb.pop_back();
        }
    }
    for (int i = ns - 1; i > 0; --i) {
        site(i - 1, i, false);
        if (i > 1) {
            eRH.push_back(env4(*eRH.back(), *gss[i], *H[i], *Va[i], false, prec));
            eRa.push_back(env_state(*eRa.back(), *gss[i], *Va[i], false, prec));
            eRb.push_back(env_state(*eRb.back(), *gss[i], *Vb[i], false, prec));
            eLH.pop_back();
            eLa.pop_back();
            eLb.pop_back();
        }
    }
    return gss;
}

cplx join(const State &a, const State &w, const State &b) {
    std::vector<DTensor *> pa, pw, pb;
    for (size_t i = 0; i < a.size(); ++i) {
        pa.push_back(a[i].get());
        pw.push_back(w[i].get());
        pb.push_back(b[i].get());
    }
    return op_expectation(pa, pw, pb);
}

}  // namespace

// global_main (holstein/krylov.h:199-283)
void global_main(const std::vector<TensorP> &Hc, std::vector<TensorP> &mps, int max_iter, double tol_exp,
                 double tol_svd, int maxd, int precision) {
    // contractions in the sweep's precision, every SVD in FP64: the stage
    // canonicalises without truncation, below any FP32 resolution floor
    const int prec = gemm_mixed(precision) ? KV_MIXED_GEMM : KV_FP64;
    KV_REQUIRE(max_iter >= 1 && max_iter <= kMaxKrylov, KV_EINVAL,
               "global Krylov: maxIter outside the supported Krylov dimension");
    mps[0] = tscale(*mps[0], 1.0 / tnorm(*mps[0]));
    std::vector<State> Vm = {mps};
    int k = 0;
    double err = 1.0;
    while (k < max_iter - 1 && err > tol_exp) {
        State hv = k > 0 ? apply_ortho2(Hc, Vm[k], Vm[k - 1], tol_svd, maxd, prec)
                         : apply_ortho1(Hc, Vm[k], tol_svd, maxd, prec);
        const double nmhv = tnorm(*hv[0]);
        KV_REQUIRE(std::isfinite(nmhv), KV_ENONFINITE, "global Krylov: non-finite vector norm");
        err *= nmhv;
        if (err < tol_exp || nmhv > 1.0) break;
        hv[0] = tscale(*hv[0], 1.0 / nmhv);
        Vm.push_back(std::move(hv));
        ++k;
    }
    // c = exp(-i Hm) e0 for the Hermitian tridiagonal matrix of joins
    // (diagonal <V_i|Hc|V_i>, upper <V_i|Hc|V_i+1>), on the device
    const int ld = (int)Vm.size();
    KrylovState h{};
    for (int i = 0; i < ld; ++i) {
        const cplx d = join(Vm[i], Hc, Vm[i]);
        h.alpha[i] = make_double2(d.real(), d.imag());
        if (i < ld - 1) {
            const cplx u = join(Vm[i], Hc, Vm[i + 1]);
            h.beta[i] = make_double2(u.real(), u.imag());
        }
    }
    h.iters = ld;
    DevBuf st(sizeof(KrylovState));
    upload_bytes(st.p, &h, sizeof(h));
    tridiag_exp(st.as<KrylovState>(), 0);
    KV_CUDA(cudaMemcpyAsync(&h, st.p, sizeof(h), cudaMemcpyDeviceToHost, ctx().stream));
    KV_CUDA(cudaStreamSynchronize(ctx().stream));
    State sum = scaled_first(Vm[0], cplx(h.coef[0].x, h.coef[0].y));
    for (int i = 1; i < ld; ++i) {
        sum = state_add(sum, scaled_first(Vm[i], cplx(h.coef[i].x, h.coef[i].y)));
        sum = op_canonicalize(sum, tol_svd, maxd, prec);
    }
    mps = sum;
}

TensorP op_scale(const DTensor &t, cplx s) {
    auto out = DTensor::make(t.meta, false);
    if (t.meta.nelem > 0) {
        k_scale_c<<<grid(t.meta.nelem), GT, 0, ctx().stream>>>(t.data(), out->data(), t.meta.nelem, s.real(),
                                                               s.imag());
        check_launch();
    }
    return out;
}

TensorP op_mix(const DTensor &t, const DTensor &W, int lead) {
    KV_REQUIRE(lead >= 0 && lead + 2 <= t.meta.rank && W.meta.rank == 4, KV_EINVAL, "internal: bad MPO mix");
    MixPlanFull M = plan_mix(t.meta, W.meta, lead);
    M.mix.upload();
    auto out = DTensor::make(M.out, false);
    launch_mix(M.mix, t.data(), W.data(), out->data(), nullptr);
    return out;
}

}  // namespace kv
