/*
 * Golden-trajectory tool (test infrastructure; compiled against the reference
 * headers in place, see oracle/Makefile).
 *
 * Runs the reference's own TDVP driver, holstein/tdvp.h:60-76 (ctor) and
 * holstein/tdvp.h:297-385 (total_start), exactly as src/kln-tdvp.cpp:73-78 does,
 * except that the Krylov maxIter / tolExp that kln-tdvp hard-codes
 * (src/kln-tdvp.cpp:28) are command-line options here.  After the run it reads
 * back the per-sweep checkpoints State/T-k.mps (holstein/tdvp.h:374-383) and
 * prints, per sweep, <psi|psi> (holstein/state.h:206-227), <psi|H|psi> and
 * <psi|D_j|psi> (Operator::join, holstein/operator.h:178-198).
 *
 * usage: kv_ref_tdvp -w mps -o mpo -s [nK,n2,nSA,n1] -v dt -D maxD -t tolSVD
 *                    -k maxIter -e tolExp [-d dens1,dens2,...] > trajectory.txt
 * Must run in a directory that has a State/ sub-directory.
 */
#include <getopt.h>
#include <unistd.h>
#include "holstein/tdvp.h"

using namespace KylinVib;

static std::vector<std::string> split_commas(const std::string &s) {
    std::vector<std::string> out;
    std::string cur;
    for (char c : s) {
        if (c == ',') { if (!cur.empty()) out.push_back(cur); cur.clear(); }
        else cur.push_back(c);
    }
    if (!cur.empty()) out.push_back(cur);
    return out;
}

int main(int argc, char **argv) {
    std::string mps_file, mpo_file, stage = "[0,0,0,1]", dens;
    double dt = 0.05, tol_svd = 1e-8, tol_exp = 1e-8;
    int max_d = 1000, max_iter = 15;
    int ch;
    while ((ch = getopt(argc, argv, "w:o:s:v:D:t:k:e:d:")) != -1) {
        switch (ch) {
            case 'w': mps_file = optarg; break;
            case 'o': mpo_file = optarg; break;
            case 's': stage = optarg; break;
            case 'v': dt = std::stod(optarg); break;
            case 'D': max_d = std::stoi(optarg); break;
            case 't': tol_svd = std::stod(optarg); break;
            case 'k': max_iter = std::stoi(optarg); break;
            case 'e': tol_exp = std::stod(optarg); break;
            case 'd': dens = optarg; break;
            default: return 2;
        }
    }
    std::vector<std::string> dens_files = split_commas(dens);
    std::array<INT, 4> stg = Holstein::parse_stage(stage);
    int nsweeps = stg[0] + stg[1] + stg[2] + stg[3];
    {
        std::ifstream ifss(mps_file), ifso(mpo_file);
        Holstein::State mps0 = Holstein::State::load(ifss);
        Holstein::Operator mpo = Holstein::Operator::load(ifso);
        // redirect the reference's progress output away from the trajectory
        std::streambuf *old = std::cout.rdbuf();
        std::ofstream sink("tdvp_ref.log");
        std::cout.rdbuf(sink.rdbuf());
        Holstein::TDVP drive(mps0, mpo, tol_svd, tol_exp, max_d, max_iter, dt);
        drive.total_start(stg);
        std::cout.rdbuf(old);
    }
    std::ifstream ifso(mpo_file);
    Holstein::Operator ham = Holstein::Operator::load(ifso);
    std::vector<Holstein::Operator> dops;
    for (auto &f : dens_files) { std::ifstream ifs(f); dops.push_back(Holstein::Operator::load(ifs)); }
    std::printf("# sweep norm2 energy pops...\n");
    for (int k = 0; k < nsweeps; ++k) {
        std::string fn = "State/T-" + std::to_string(k) + ".mps";
        std::ifstream ifs(fn);
        Holstein::State s = Holstein::State::load(ifs);
        double n2 = std::real(Holstein::overlap(s, s));
        double e = std::real(ham.join(s, s));
        std::printf("%d %.17e %.17e", k, n2, e);
        for (auto &d : dops) std::printf(" %.17e", std::real(d.join(s, s)));
        int maxb = 0;
        for (INT i = 0; i < s.nsite() - 1; ++i) {
            int b = 0;
            for (auto &kv : s.at(i).cleg(2)) b += kv.second;
            maxb = std::max(maxb, b);
        }
        std::printf(" %d\n", maxb);
    }
    return 0;
}
