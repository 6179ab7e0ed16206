// Host-side engine declarations: plans, operations, TDVP driver.
#pragma once
#include <chrono>
#include <random>

#include "kv_internal.h"

namespace kv {

// precision mode -> which parts run in mixed precision
inline bool gemm_mixed(int precision) { return precision == KV_MIXED_TF32 || precision == KV_MIXED_GEMM; }
inline bool svd_mixed(int precision) { return precision == KV_MIXED_TF32 || precision == KV_MIXED_SVD; }
// Output tile shape of the grouped GEMM for a precision mode.
inline int kTileM(int precision) { return gemm_mixed(precision) ? kMixedTileM : 32; }
inline int kTileN(int precision) { return gemm_mixed(precision) ? kMixedTileN : 32; }

// reference flop count split by who executes it here: the grouped GEMM
// (product<> pairs) or the MPO mixing kernel (env_mps_mpo zgemms)
struct Flops {
    double gemm = 0.0, mix = 0.0;
};

struct ProductPlan {
    Meta out;
    GemmPlan gemm;
    // segments grouped by output block: block b owns segs[out_start[b] .. out_start[b+1])
    std::vector<GemmSeg> segs;
    std::vector<std::pair<int, int>> pairs;  // (A block, B block) of each segment
    std::vector<int> out_start;
    std::vector<std::pair<int, int>> mn;     // (M, N) per output block
};

struct MixPlanFull {
    Meta out;                  // merged output structure (what is computed)
    std::vector<double> mult;  // reference blocks (matched pairs) merged into each output block
    MixPlan mix;
    double ref_flops = 0.0;
    std::vector<int> term_in;        // input block of each term (aligned with mix.terms)
    std::vector<double> term_coef;   // its reference flops per matched input block
};

struct HeffPlan {
    int nsite = 1;
    Meta klayout;  // Krylov layout (closure of psi's blocks under H_eff)
    ProductPlan p1, p2;
    MixPlanFull m1, m2;
    std::vector<Flops> iter_flops;  // reference flops of the apply at Lanczos iteration k
    // elements of the layout prefix holding the blocks reached within j
    // applications (j = 0 .. napply; later iterations keep the last)
    std::vector<int64_t> prefix;
    int napply = 1;
};

struct SvdOut {
    TensorP U, V;
    int n_kept = 0, n_total = 0;
    std::vector<double> kept_s;
};

// keys_only: the output structure (and reference flops) without segment lists
ProductPlan plan_product(const Meta &A, const Meta &B, int nc, int opA, int opB, bool keys_only = false);
void build_tiles(ProductPlan &P, const std::vector<int64_t> &target_off, int tile_m, int tile_n);
MixPlanFull plan_mix(const Meta &lm, const Meta &W, int lead, const std::vector<double> *mult_in = nullptr,
                     bool keys_only = false);
double ref_product_flops(const Meta &A, const Meta &B, int nc, int opA, int opB, const std::vector<double> *multA,
                         const std::vector<double> *multB);
HeffPlan plan_heff(int nsite, const Meta &L, const Meta &psi, const Meta *W1, const Meta *W2, const Meta &R,
                   int precision, int max_iter);

void clear_plan_cache();
// H_eff plans built (cache misses) and host ms spent building them since kv_init
void plan_stats(long long *built, double *ms);
TensorP op_product(const DTensor &A, const DTensor &B, int nc, int opA, int opB, int precision,
                   Flops *fl = nullptr);
TensorP op_heff(int nsite, const DTensor &L, const DTensor &psi, const DTensor *W1, const DTensor *W2,
                const DTensor &R, double scale, int precision);
TensorP op_lanczos(int nsite, const DTensor &L, const DTensor &psi, const DTensor *W1, const DTensor *W2,
                   const DTensor &R, double dt, int max_iter, double tol, bool reverse, int precision,
                   KrylovState *st_dev, std::vector<Flops> *per_iter, int *iters_out = nullptr);
// The SA-1TDVP split (sa_svd_impl, holstein/svd.h:443-614): every sector's
// full SVD is kept and the bond is extended by synthetic states (FP64 SVD in
// every precision mode).  seeds: the seed stream every random draw's
// generator is seeded from, in the reference's order of draws.
struct SaParams {
    double beta = 1.0;              // width of the quasi-Gaussian draws (betaSet[bond])
    std::mt19937 *seeds = nullptr;
    int added = 0;                  // out: states added to the bond
};
SvdOut op_svd(const DTensor &A, int r1, bool l2r, double thres, int max_dim, int precision, SaParams *sa = nullptr);
TensorP op_env(bool l2r, const DTensor &env, const DTensor &A, const DTensor &W, const DTensor *Wt, int precision,
               Flops *fl);
TensorP op_permute(const DTensor &t, const std::vector<int> &ax);
// out[k, s', wr, rest] = sum_{wl, s} W[s', wl, s, wr] t[k, wl, s, rest] (k = legs [0, lead)),
// equal output blocks merged
TensorP op_mix(const DTensor &t, const DTensor &W, int lead);
TensorP boundary_env(int dir0, int q);
TensorP op_scale(const DTensor &t, cplx s);  // s * t
// t + v s over the union of the blocks (equal keys merged, t's blocks first)
TensorP op_add_scaled(const DTensor &t, const DTensor &s, cplx v);
// global_main (holstein/krylov.h:199-283) on the MPO Hc (already scaled by dt)
void global_main(const std::vector<TensorP> &Hc, std::vector<TensorP> &mps, int max_iter, double tol_exp,
                 double tol_svd, int maxd, int precision);
std::vector<TensorP> op_canonicalize(const std::vector<TensorP> &in, double tol, int max_dim, int precision);
cplx op_expectation(const std::vector<DTensor *> &a, const std::vector<DTensor *> &w, const std::vector<DTensor *> &b);
// <psi|O_k|psi> for operators that are the identity except on site op_site[k]
// (its MPO tensor op[k]); ident: the identity MPO's tensors
std::vector<cplx> op_local_expectations(const std::vector<DTensor *> &mps, const std::vector<DTensor *> &ident,
                                        const std::vector<int> &op_site, const std::vector<DTensor *> &op);
// the same value with all device scratch in a fixed static array (kv_noalloc.cu)
cplx expectation_noalloc(const std::vector<DTensor *> &bra, const std::vector<DTensor *> &w,
                         const std::vector<DTensor *> &ket);

// Adjoints of the H_eff apply and the environment update (kv_adjoint.cu):
// the cotangents selected by `want` (a mask of the kGrad* bits)
enum : unsigned { kGradPsi = 1, kGradL = 2, kGradW1 = 4, kGradW2 = 8, kGradR = 16 };
enum : unsigned { kGradEnv = 1, kGradA = 2, kGradW = 4 };
struct HeffGrads {
    TensorP psi, L, W1, W2, R;
};
struct EnvGrads {
    TensorP env, A, W;
};
HeffGrads op_adjoint_heff(int nsite, const TensorP &L, const TensorP &psi, const TensorP &W1, const TensorP &W2,
                          const TensorP &R, double scale, const DTensor &ybar, int precision, unsigned want);
EnvGrads op_adjoint_env(bool l2r, const TensorP &env, const TensorP &A, const TensorP &W, const DTensor &ebar,
                        int precision, unsigned want);

enum Module { MOD_EVL0 = 0, MOD_EVL1, MOD_EVL2, MOD_SVD, MOD_UPDATE, MOD_SWEEP, MOD_COUNT };

class Tdvp {
  public:
    Tdvp(const std::vector<TensorP> &mps, const std::vector<TensorP> &mpo, double tol_svd, double tol_exp,
         int max_dim, int max_iter, double dt, int precision);
    ~Tdvp();
    void one_site();
    void two_site();
    // TDVP::sa_site (holstein/tdvp.h:230-294) with the widths and seed of set_sa
    void sa_site();
    void set_sa(const double *beta, int nbeta, unsigned long long seed);
    std::vector<double> sa_beta;  // one width per bond (betaSet)
    std::mt19937 sa_seeds;        // seed stream of the SA draws
    long long sa_added = 0;       // states the SA splits added in the last sweep
    // the kept singular values (descending) of every two-site split since they
    // were last read: the record svd_impl appends to the SVS file
    // (holstein/svd.h:390-402) for the SA stage's fit; kept once svs_on is set
    // (the first kv_tdvp_svs call on the handle)
    std::vector<std::vector<double>> svs;
    bool svs_on = false;
    // n timed local updates of the two-site left-to-right pass from site i0
    // (the pass advanced there first, untimed)
    void window(int i0, int n);
    int window_at = -1;  // site the two-site pass has reached in window mode (-1: none)
    // one step of total_start's global-Krylov stage, then the environments
    // rebuilt from the new state
    void global_krylov();
    std::vector<TensorP> mps, mpo, mpo_t;
    std::vector<TensorP> envL, envR;
    double tol_svd, tol_exp;
    int max_dim, max_iter;
    double dt;
    int precision;
    double module_ms[MOD_COUNT] = {};
    double sweep_ms = 0.0;
    double module_host_ms[MOD_COUNT] = {};  // host wall-clock of the last sweep
    double sweep_host_ms = 0.0;
    long long plans_built = 0;               // H_eff plan-cache misses in the last sweep
    double plan_ms = 0.0;                    // host ms spent building them
    double last_ref_flops = 0.0;   // all reference zgemm flops of the last sweep
    double last_gemm_flops = 0.0;  // of which in product<> pairs (grouped GEMM)

  private:
    void two_site_lr(int i);
    static constexpr int kStateSlots = 8192;
    static constexpr int kMaxEvents = 16384;
    TensorP krylov(int nsite, const DTensor &L, const DTensor &psi, const DTensor *W1, const DTensor *W2,
                   const DTensor &R, bool reverse, int module);
    void mark(int module, bool start);
    void init_envs();
    KrylovState *next_state();
    void begin_sweep();
    void end_sweep();
    DevBuf kstate;
    std::vector<cudaEvent_t> events;
    int mark_module[kMaxEvents] = {};
    std::chrono::steady_clock::time_point host_t0, sweep_t0;
    long long plans0 = 0;
    double plan_ms0 = 0.0;
    int n_marks = 0, n_krylov = 0;
    std::vector<std::pair<KrylovState *, std::vector<Flops>>> krylov_flops;
    Flops other;
    cudaEvent_t sweep_ev[2] = {};
};

}  // namespace kv
