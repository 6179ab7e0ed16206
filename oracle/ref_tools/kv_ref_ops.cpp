/*
 * Golden block-level tool (test infrastructure; compiled against the
 * reference headers in place, see oracle/Makefile).
 *
 * Given an MPS, an MPO and a site index i, it builds the environments the way
 * TDVP::total_start does (boundaries holstein/tdvp.h:303-311, right stack
 * holstein/tdvp.h:313-316; the left environment of site i by L->R env_sweep over
 * sites 0..i-1) and dumps the outputs of each hot-path primitive on those
 * exact inputs:
 *   envL, envR, envR2    environments of site i (and of the bond i,i+1)
 *   h1   apply_single(L, A_i, W_i, R)                   holstein/product.h:547-553
 *   h2   apply_double(L, A_i A_i+1, W_i, W_i+1, R2)      holstein/product.h:478-486
 *   h0   apply_zero(L', C, R)                            holstein/product.h:540-545
 *   envL_next  env_sweep(L, U, W_i, true)                holstein/product.h:488-496
 *   envR_prev  env_sweep(R, A_i, W_i, false)             holstein/product.h:497-502
 *   mm   product<3,3,1>(A_i, A_i+1)                      holstein/product.h:61-201
 *   svd21_*, svd12_*, svd22l_*, svd22r_*  svd_impl U / V factors and singular values
 *   k1, k2, k0  local_krylov<3|4|2> results              holstein/exponential.h:92-190
 *
 * usage: kv_ref_ops -w mps -o mpo -i site -v dt -k maxIter -e tolExp
 *                   -t tolSVD -D maxD -O outdir
 */
#include <getopt.h>
#include <unistd.h>
#include "holstein/tdvp.h"
#include "kvt_io.h"

using namespace KylinVib;
using namespace KylinVib::Holstein;

template <int R>
static void dump(const std::string &dir, const char *name, const Tensor<R> &t) {
    kvt::write_tensor<Tensor<R>, R>(dir + "/" + name + ".kvt", t);
}

int main(int argc, char **argv) {
    std::string mps_file, mpo_file, outdir = ".";
    int site = 0, max_iter = 11, max_d = 1000;
    double dt = 0.05, tol_exp = 1e-8, tol_svd = 1e-8;
    int ch;
    while ((ch = getopt(argc, argv, "w:o:i:v:k:e:t:D:O:")) != -1) {
        switch (ch) {
            case 'w': mps_file = optarg; break;
            case 'o': mpo_file = optarg; break;
            case 'i': site = std::stoi(optarg); break;
            case 'v': dt = std::stod(optarg); break;
            case 'k': max_iter = std::stoi(optarg); break;
            case 'e': tol_exp = std::stod(optarg); break;
            case 't': tol_svd = std::stod(optarg); break;
            case 'D': max_d = std::stoi(optarg); break;
            case 'O': outdir = optarg; break;
            default: return 2;
        }
    }
    std::ifstream ifss(mps_file), ifso(mpo_file);
    State mps = State::load(ifss);
    Operator mpo = Operator::load(ifso);
    const int ns = mps.nsite();
    if (site < 0 || site + 1 >= ns) { std::fprintf(stderr, "site must be in [0, ns-2]\n"); return 2; }

    // boundaries exactly as holstein/tdvp.h:303-311
    Tensor<3> envl({1, -1, -1});
    Block<3> ri({1, 1, 1}, {0, 0, 0});
    ri({0, 0, 0}) = 1.0;
    envl.push_back(ri);
    envl.check_legs();
    INT tot = mps.at(ns - 1).at(0).qn()[2];
    Tensor<3> envr({-1, 1, 1});
    Block<3> rf({1, 1, 1}, {tot, 0, tot});
    rf({0, 0, 0}) = 1.0;
    envr.push_back(rf);
    envr.check_legs();

    std::vector<Tensor<3>> rstack = {envr};
    for (int i = ns - 1; i > site; --i) rstack.push_back(env_sweep(rstack.back(), mps.at(i), mpo.at(i), false));
    Tensor<3> R = rstack.back();                  // environment right of site
    Tensor<3> R2 = rstack[rstack.size() - 2];     // environment right of site+1
    Tensor<3> L = envl;
    for (int i = 0; i < site; ++i) L = env_sweep(L, mps.at(i), mpo.at(i), true);

    dump<3>(outdir, "envL", L);
    dump<3>(outdir, "envR", R);
    dump<3>(outdir, "envR2", R2);

    // one-site H_eff, env updates
    dump<3>(outdir, "h1", apply_single(L, mps.at(site), mpo.at(site), R));
    dump<3>(outdir, "envR_prev", env_sweep(R, mps.at(site), mpo.at(site), false));

    // SVDs of the one-site tensor (both directions)
    SVDConfig cfg;
    cfg.SVDThres = tol_svd;
    cfg.MaxDim = max_d;
    Tensor<3> a = mps.at(site);
    cfg.Left2Right = true;
    auto [u21, v21] = svd_impl<2, 1>(a, cfg, -1);
    dump<3>(outdir, "svd21_U", u21);
    dump<2>(outdir, "svd21_V", v21);
    cfg.Left2Right = false;
    auto [u12, v12] = svd_impl<1, 2>(a, cfg, -1);
    dump<2>(outdir, "svd12_U", u12);
    dump<3>(outdir, "svd12_V", v12);

    Tensor<3> Lnext = env_sweep(L, u21, mpo.at(site), true);
    dump<3>(outdir, "envL_next", Lnext);
    dump<2>(outdir, "h0", apply_zero(Lnext, v21, R));

    // two-site
    Tensor<4> mm = product<3, 3, 1>(mps.at(site), mps.at(site + 1), CblasNoTrans, CblasNoTrans);
    dump<4>(outdir, "mm", mm);
    dump<4>(outdir, "h2", apply_double(L, mm, mpo.at(site), mpo.at(site + 1), R2));
    cfg.Left2Right = true;
    auto [u22l, v22l] = svd_impl<2, 2>(mm, cfg, -1);
    dump<3>(outdir, "svd22l_U", u22l);
    dump<3>(outdir, "svd22l_V", v22l);
    cfg.Left2Right = false;
    auto [u22r, v22r] = svd_impl<2, 2>(mm, cfg, -1);
    dump<3>(outdir, "svd22r_U", u22r);
    dump<3>(outdir, "svd22r_V", v22r);

    // Krylov exponentials
    KrylovConfig kc;
    kc.KrylovThres = tol_exp;
    kc.MaxIter = max_iter;
    kc.TimeStep = dt;
    Tensor<4> dummy;
    Tensor<3> k1 = mps.at(site);
    local_krylov<3>(L, k1, mpo.at(site), dummy, R, kc);
    dump<3>(outdir, "k1", k1);
    Tensor<4> k2 = mm;
    local_krylov<4>(L, k2, mpo.at(site), mpo.at(site + 1), R2, kc);
    dump<4>(outdir, "k2", k2);
    Tensor<2> k0 = v21;
    local_krylov<2>(Lnext, k0, dummy, dummy, R, kc, true);
    dump<2>(outdir, "k0", k0);
    return 0;
}
