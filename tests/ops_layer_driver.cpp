// A program written against the reference's tensor-level headers
// (holstein/tensor.h, product.h, exponential.h, svd.h) and its State /
// Operator classes, compiled against include/holstein/ and linked with
// -lkvgpu.  It runs the hot-path primitives on one site of a golden case,
// canonicalises the case's MPS and evaluates <psi|H|psi>, and writes every
// result as a .kvt file (or in its one JSON line) for tests/test_ops_layer.py
// to compare with the reference's dumps and the oracle.
//
//   ops_layer_driver <case dir> <ops dir> <out dir> <site> <max D>
#include <cstdio>
#include <fstream>
#include <string>

#include "holstein/exponential.h"
#include "holstein/product.h"
#include "holstein/svd.h"
#include "holstein/tensor.h"

using namespace KylinVib;
using namespace KylinVib::Holstein;

namespace {

constexpr int kKvtMagic = 0x3154564B;

template <INT R>
Tensor<R> read_kvt(const string &path) {
    ifstream f(path, ios::binary);
    if (!f) detail::fail("cannot open " + path);
    int magic = 0, rank = 0, nb = 0;
    f.read(reinterpret_cast<char *>(&magic), 4);
    f.read(reinterpret_cast<char *>(&rank), 4);
    if (magic != kKvtMagic || rank != R) detail::fail(path + ": not a rank-" + to_string(R) + " KVT file");
    array<INT, R> dirs{};
    f.read(reinterpret_cast<char *>(dirs.data()), 4 * R);
    f.read(reinterpret_cast<char *>(&nb), 4);
    Tensor<R> t(dirs);
    for (int b = 0; b < nb; ++b) {
        array<INT, R> sh{}, qn{};
        f.read(reinterpret_cast<char *>(sh.data()), 4 * R);
        f.read(reinterpret_cast<char *>(qn.data()), 4 * R);
        Block<R> blk(sh, qn);
        f.read(reinterpret_cast<char *>(blk.ptr()), sizeof(Complex) * blk.size());
        t.push_back(blk);
    }
    t.check_legs();
    return t;
}

template <INT R>
void write_kvt(const string &path, const Tensor<R> &t) {
    ofstream f(path, ios::binary);
    const int magic = kKvtMagic, rank = R, nb = t.num_blocks();
    f.write(reinterpret_cast<const char *>(&magic), 4);
    f.write(reinterpret_cast<const char *>(&rank), 4);
    f.write(reinterpret_cast<const char *>(t.dirs().data()), 4 * R);
    f.write(reinterpret_cast<const char *>(&nb), 4);
    for (INT b = 0; b < nb; ++b) {
        const Block<R> &blk = t.at(b);
        f.write(reinterpret_cast<const char *>(blk.shape().data()), 4 * R);
        f.write(reinterpret_cast<const char *>(blk.qn().data()), 4 * R);
        f.write(reinterpret_cast<const char *>(blk.cptr()), sizeof(Complex) * blk.size());
    }
}

}  // namespace

int main(int argc, char **argv) {
    if (argc != 6) {
        cout << "usage: ops_layer_driver <case dir> <ops dir> <out dir> <site> <max D>" << endl;
        return 2;
    }
    const string cs = argv[1], ops = argv[2], out = string(argv[3]) + "/";
    const INT i = atoi(argv[4]), maxD = atoi(argv[5]);
    ifstream fm(cs + "/in.mps", ios::binary), fo(cs + "/H.mpo", ios::binary);
    State mps = State::load(fm);
    Operator mpo = Operator::load(fo);
    const Tensor<3> A = to_tensor(mps.at(i)), B = to_tensor(mps.at(i + 1));
    const Tensor<4> W = to_tensor(mpo.at(i)), W2 = to_tensor(mpo.at(i + 1));
    const Tensor<3> L = read_kvt<3>(ops + "/envL.kvt"), R = read_kvt<3>(ops + "/envR.kvt"),
                    R2 = read_kvt<3>(ops + "/envR2.kvt");

    // contractions (holstein/product.h)
    write_kvt(out + "h1.kvt", apply_single(L, A, W, R));
    write_kvt(out + "envR_prev.kvt", env_sweep(R, A, W, false));
    Tensor<4> mm = product<3, 3, 1>(A, B, CblasNoTrans, CblasNoTrans);
    write_kvt(out + "mm.kvt", mm);
    write_kvt(out + "h2.kvt", apply_double(L, mm, W, W2, R2));
    const Tensor<3> U21 = read_kvt<3>(ops + "/svd21_U.kvt");
    const Tensor<2> V21 = read_kvt<2>(ops + "/svd21_V.kvt");
    const Tensor<3> Ln = env_sweep(L, U21, W, true);
    write_kvt(out + "envL_next.kvt", Ln);
    write_kvt(out + "h0.kvt", apply_zero(read_kvt<3>(ops + "/envL_next.kvt"), V21, R));

    // block SVDs (holstein/svd.h), the two-site ones writing the SVS record
    SVDConfig cfg;
    cfg.SVDThres = 1e-8;
    cfg.MaxDim = maxD;
    {
        Tensor<3> a = A;
        cfg.Left2Right = true;
        auto [u, v] = svd_impl<2, 1>(a, cfg, -1);
        write_kvt(out + "svd21_U.kvt", u);
        write_kvt(out + "svd21_V.kvt", v);
        cfg.Left2Right = false;
        auto [u2, v2] = svd_impl<1, 2>(a, cfg, -1);
        write_kvt(out + "svd12_U.kvt", u2);
        write_kvt(out + "svd12_V.kvt", v2);
        cfg.Left2Right = true;
        auto [u3, v3] = svd_impl<2, 2>(mm, cfg, -1, true, true);
        write_kvt(out + "svd22l_U.kvt", u3);
        write_kvt(out + "svd22l_V.kvt", v3);
        cfg.Left2Right = false;
        auto [u4, v4] = svd_impl<2, 2>(mm, cfg, -1, true, true);
        write_kvt(out + "svd22r_U.kvt", u4);
        write_kvt(out + "svd22r_V.kvt", v4);
    }

    // Krylov exponentials (holstein/exponential.h)
    KrylovConfig kc;
    kc.KrylovThres = 1e-8;
    kc.MaxIter = 11;
    kc.TimeStep = 0.05;
    Tensor<3> p1 = A;
    const KrylovExit e1 = local_krylov<3>(L, p1, W, W, R, kc);
    write_kvt(out + "k1.kvt", p1);
    Tensor<4> p2 = read_kvt<4>(ops + "/mm.kvt");
    const KrylovExit e2 = local_krylov<4>(L, p2, W, W2, R2, kc);
    write_kvt(out + "k2.kvt", p2);
    Tensor<2> p0 = V21;
    const KrylovExit e0 = local_krylov<2>(read_kvt<3>(ops + "/envL_next.kvt"), p0, W, W, R, kc, true);
    write_kvt(out + "k0.kvt", p0);

    // host-side tensor operations (holstein/tensor.h)
    write_kvt(out + "A_t210.kvt", transpose<3>(A, {2, 1, 0}));
    Tensor<3> a3 = A * Complex(0.0, 2.0);
    a3 += A;
    a3 *= 0.5;
    write_kvt(out + "A_combo.kvt", a3);
    const Complex ov = overlap(A, a3);
    // the two-leg bra/ket environment env_sweep (holstein/product.h:523-538)
    // (the identity on the left-bond sector of A's first block)
    Tensor<2> e2l({1, -1});
    {
        const INT d = A.at(0).shape()[0], q = A.at(0).qn()[0];
        Block<2> one({d, d}, {q, q});
        for (INT k = 0; k < d; ++k) one({k, k}) = 1.0;
        e2l.push_back(one);
    }
    write_kvt(out + "env2_l2r.kvt", env_sweep(e2l, A, a3, true));

    // State / Operator level (holstein/state.h, holstein/operator.h)
    const Complex j0 = mpo.join(mps, mps);
    State c = mps;
    c.canonicalize();
    const Complex j1 = mpo.join(c, c);
    Operator half = mpo;
    half *= 0.5;
    const Complex j2 = half.join(c * 2.0, c);  // 0.5 * 2 <c|H|c>
    for (INT k = 0; k < c.nsite(); ++k) write_kvt(out + "canon_" + to_string(k) + ".kvt", to_tensor(c.at(k)));
    // direct sums: H + 2H represents 3H, psi + psi represents 2 psi
    Operator h3 = mpo, two = mpo;
    two *= 2.0;
    h3 += two;
    const Complex j3 = h3.join(mps, mps);
    State s2 = mps;
    s2 += mps;
    const Complex j4 = mpo.join(s2, s2);
    write_kvt(out + "sum_state_1.kvt", to_tensor(s2.at(1)));
    write_kvt(out + "sum_mpo_1.kvt", to_tensor(h3.at(1)));
    Tensor<3> x = to_tensor(mps.at(1));
    stack<3>(x, to_tensor(mps.at(1)), {0, 2});
    write_kvt(out + "stack_1.kvt", x);

    printf("{\"k1_iters\": %d, \"k2_iters\": %d, \"k0_iters\": %d, \"k1_loss\": %.17g, \"k1_maxitr\": %d, "
           "\"norm_A\": %.17g, \"overlap_re\": %.17g, \"overlap_im\": %.17g, \"join\": [%.17g, %.17g, %.17g, "
           "%.17g, %.17g, %.17g, %.17g, %.17g, %.17g, %.17g]}\n",
           e1.RealIter, e2.RealIter, e0.RealIter, e1.LossNorm,
           e1.reason == KrylovExitReason::AchMaxItr ? 1 : 0, norm(A), ov.real(), ov.imag(), j0.real(), j0.imag(),
           j1.real(), j1.imag(), j2.real(), j2.imag(), j3.real(), j3.imag(), j4.real(), j4.imag());
    return 0;
}
