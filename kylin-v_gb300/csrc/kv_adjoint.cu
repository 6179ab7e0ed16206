// Adjoints (vector-Jacobian products) of the effective-Hamiltonian apply and
// of the environment update.  The reference has no derivative code; these
// are the reverse-mode rules of its two multilinear maps,
//   y  = H_eff(L, W1[, W2], R) psi          (holstein/product.h:478-486, 540-553)
//   L' = sum conj(A) L W A                   (holstein/product.h:488-503)
// with the cotangent convention of a real loss l: xbar = dl/dRe x + i dl/dIm x,
// so that dl = Re <ybar, dy> and, for y linear in x, xbar = (dy/dx)^H ybar.
// Every cotangent is itself a contraction of the same network with one
// tensor replaced by ybar and the others conjugated; each is built here from
// the engine's block-sparse products, MPO mixing and permutations, so the
// block-charge bookkeeping (matching sectors, leg directions) is the
// forward path's.  Dense forms (indices: a bond of L, s physical, w/u/v MPO):
//   1-site  y[a',s',b'] = L[a',w,a] W[s',w,s,v] psi[a,s,b] R[b',v,b]
//   2-site  y[a',s1',s2',b'] = L[a',w,a] W1[s1',w,s1,u] W2[s2',u,s2,v] psi[a,s1,s2,b] R[b',v,b]
//   0-site  y[a',b'] = L[a',w,a] C[a,b] R[b',w,b]
#include <vector>

#include "kv_engine.h"

namespace kv {

namespace {

__global__ void k_conj_scale(const double2 *__restrict__ in, double2 *__restrict__ out, int64_t n, double s,
                             int conj) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 v = in[i];
        out[i] = make_double2(s * v.x, conj ? -s * v.y : s * v.y);
    }
}

int grid(int64_t n) {
    const int64_t g = (n + 255) / 256;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)ctx().num_sms * 8));
}

constexpr int kN = KV_OP_N, kT = KV_OP_T, kC = KV_OP_C;

// s * t or s * conj(t) (directions flipped with the conjugate)
TensorP conj_scale(const DTensor &t, double s, bool conj) {
    Meta m = t.meta;
    if (conj)
        for (int i = 0; i < m.rank; ++i) m.dirs[i] = -m.dirs[i];
    auto out = DTensor::make(m, false);
    if (m.nelem > 0) {
        k_conj_scale<<<grid(m.nelem), 256, 0, ctx().stream>>>(t.data(), out->data(), m.nelem, s, conj ? 1 : 0);
        counted();
        KV_CUDA(cudaGetLastError());
    }
    return out;
}
TensorP cj(const DTensor &t) { return conj_scale(t, 1.0, true); }

// a + b over the union of their blocks
TensorP add(const DTensor &a, const DTensor &b) { return op_add_scaled(a, b, cplx(1.0, 0.0)); }

TensorP mix(const DTensor &t, const DTensor &W, int lead) { return op_mix(t, W, lead); }

TensorP perm(const DTensor &t, std::vector<int> ax) { return op_permute(t, ax); }

struct Net {  // one H_eff network: L, psi, W1, W2, R (W1/W2 null as nsite asks)
    int nsite;
    TensorP L, psi, W1, W2, R;
};

TensorP left_part(const Net &n, int prec) {
    TensorP o = op_product(*n.L, *n.psi, 1, kN, kN, prec);
    if (n.nsite >= 1) o = mix(*o, *n.W1, 1);
    if (n.nsite == 2) o = mix(*o, *n.W2, 2);
    return o;
}

TensorP apply(const Net &n, int prec) { return op_product(*left_part(n, prec), *n.R, 2, kN, kT, prec); }

std::vector<int> reversed(int rank) {
    std::vector<int> r(rank);
    for (int i = 0; i < rank; ++i) r[i] = rank - 1 - i;
    return r;
}

// The same network read right to left: R becomes the left environment, the
// bond and physical legs of psi and ybar reverse, each W swaps its bond legs.
Net reverse(const Net &n, const DTensor &ybar, TensorP *ybar_r) {
    auto wt = [](const TensorP &w) { return w ? perm(*w, {0, 3, 2, 1}) : nullptr; };
    Net r{n.nsite, n.R, perm(*n.psi, reversed(n.psi->meta.rank)), nullptr, nullptr, n.L};
    if (n.nsite == 2) {
        r.W1 = wt(n.W2);
        r.W2 = wt(n.W1);
    } else {
        r.W1 = wt(n.W1);
    }
    *ybar_r = perm(ybar, reversed(ybar.meta.rank));
    return r;
}

// R cotangent: conj(Rbar)[b', v, b] = sum conj(ybar)[a', s'.., b'] left[a', s'.., v, b]
TensorP grad_R(const Net &n, const DTensor &ybar, int prec) {
    return cj(*op_product(ybar, *left_part(n, prec), n.nsite + 1, kC, kN, prec));
}

// W1 cotangent (1- and 2-site)
TensorP grad_W1(const Net &n, const DTensor &ybar, int prec) {
    if (n.nsite == 1) {
        TensorP t = op_product(*op_product(*n.L, *n.psi, 1, kN, kN, prec), *n.R, 1, kN, kT, prec);  // [a',w,s,b',v]
        TensorP tp = perm(*t, {0, 3, 1, 2, 4});                                                   // [a',b',w,s,v]
        TensorP y = perm(ybar, {0, 2, 1});                                                        // [a',b',s']
        return cj(*op_product(*y, *tp, 2, kC, kN, prec));                                         // [s',w,s,v]
    }
    TensorP p1 = op_product(*n.psi, *n.R, 1, kN, kT, prec);          // [a, s1, s2, b', v]
    TensorP p2 = perm(*p1, {0, 1, 3, 4, 2});                         // [a, s1, b', v, s2]
    TensorP m = mix(*p2, *perm(*n.W2, {0, 3, 2, 1}), 3);             // [a, s1, b', s2', u]
    TensorP q = op_product(*n.L, *m, 1, kN, kN, prec);               // [a', w, s1, b', s2', u]
    TensorP qp = perm(*q, {0, 4, 3, 1, 2, 5});                       // [a', s2', b', w, s1, u]
    TensorP y = perm(ybar, {0, 2, 3, 1});                            // [a', s2', b', s1']
    return cj(*op_product(*y, *qp, 3, kC, kN, prec));                // [s1', w, s1, u]
}

}  // namespace

HeffGrads op_adjoint_heff(int nsite, const TensorP &L, const TensorP &psi, const TensorP &W1, const TensorP &W2,
                          const TensorP &R, double scale, const DTensor &ybar_in, int precision, unsigned want) {
    KV_REQUIRE(nsite >= 0 && nsite <= 2, KV_EINVAL, "nsite must be 0, 1 or 2");
    KV_REQUIRE(L && psi && R && (nsite < 1 || W1) && (nsite < 2 || W2), KV_EINVAL, "missing H_eff operand");
    KV_REQUIRE(L->meta.rank == 3 && R->meta.rank == 3 && psi->meta.rank == nsite + 2 &&
                   ybar_in.meta.rank == nsite + 2,
               KV_EINVAL, "H_eff operand ranks do not match nsite");
    // y = scale * H psi: every cotangent carries the (real) scale once
    TensorP ybar = conj_scale(ybar_in, scale, false);
    Net n{nsite, L, psi, nsite >= 1 ? W1 : nullptr, nsite == 2 ? W2 : nullptr, R};
    HeffGrads g;
    if (want & kGradPsi) {
        // psi cotangent: conj(H(L^T, conj(ybar), W^T.., R^T)), the transposes
        // exchanging the bra and ket legs of L, R and the physical legs of W
        auto wT = [](const TensorP &w) { return w ? perm(*w, {2, 1, 0, 3}) : nullptr; };
        Net t{nsite, perm(*L, {2, 1, 0}), cj(*ybar), wT(n.W1), wT(n.W2), perm(*R, {2, 1, 0})};
        g.psi = cj(*apply(t, precision));
    }
    if (want & kGradR) g.R = grad_R(n, *ybar, precision);
    if ((want & kGradL) || ((want & kGradW2) && nsite == 2)) {
        TensorP yr;
        Net r = reverse(n, *ybar, &yr);
        if (want & kGradL) g.L = grad_R(r, *yr, precision);
        if ((want & kGradW2) && nsite == 2) g.W2 = perm(*grad_W1(r, *yr, precision), {0, 3, 2, 1});
    }
    if ((want & kGradW1) && nsite >= 1) g.W1 = grad_W1(n, *ybar, precision);
    return g;
}

EnvGrads op_adjoint_env(bool l2r, const TensorP &env, const TensorP &A_in, const TensorP &W_in,
                        const DTensor &ebar, int precision, unsigned want) {
    KV_REQUIRE(env && A_in && W_in && env->meta.rank == 3 && A_in->meta.rank == 3 && W_in->meta.rank == 4 &&
                   ebar.meta.rank == 3,
               KV_EINVAL, "environment operands must be rank 3 (env, A) and 4 (W)");
    // right-to-left is left-to-right on A {2,1,0}, W {0,3,2,1} (holstein/product.h:488-503)
    TensorP A = l2r ? A_in : perm(*A_in, {2, 1, 0});
    TensorP W = l2r ? W_in : perm(*W_in, {0, 3, 2, 1});
    TensorP ce = cj(ebar);  // conj(ebar) has the directions of a right environment
    EnvGrads g;
    if (want & kGradEnv) {
        // conj(envbar) = the right-to-left update of conj(ebar) with A, W
        g.env = cj(*op_env(false, *ce, *A, *W, nullptr, precision, nullptr));
    }
    if (want & kGradA) {
        // A enters as ket (a2) and, conjugated, as bra (a1)
        Net ket{1, env, A, W, nullptr, ce};
        TensorP a2 = apply(ket, precision);
        Net bra{1, perm(*env, {2, 1, 0}), cj(*A), perm(*W, {2, 1, 0, 3}), nullptr, perm(*ce, {2, 1, 0})};
        TensorP a1 = cj(*apply(bra, precision));
        g.A = add(*a1, *a2);
        if (!l2r) g.A = perm(*g.A, {2, 1, 0});
    }
    if (want & kGradW) {
        Net n{1, env, A, W, nullptr, ce};
        g.W = grad_W1(n, *A, precision);
        if (!l2r) g.W = perm(*g.W, {0, 3, 2, 1});
    }
    return g;
}

}  // namespace kv
