// C ABI of libkvgpu (include/kvgpu.h).  Every entry point converts C++
// exceptions into status codes; nothing here exits the process.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "kv_engine.h"

struct kv_tensor_s {
    kv::TensorP t;
};
struct kv_tdvp_s {
    std::unique_ptr<kv::Tdvp> s;
};

namespace {
thread_local std::string g_err;

// A call that fails part-way can leave the device error word of the
// tensor-core GEMM set (an Inf/NaN operand seen before the failure was
// raised); it belongs to the failed call, so it is cleared, not reported by
// the next one.
void drop_pending_status() noexcept {
    try {
        if (kv::ctx().device >= 0) kv::mixed_gemm_status();
    } catch (...) {
    }
}

template <class F>
int guard(F &&f) {
    try {
        f();
        return KV_OK;
    } catch (const kv::Error &e) {
        g_err = e.what();
        if (e.code != KV_ECUDA) drop_pending_status();
        return e.code;
    } catch (const std::bad_alloc &) {
        g_err = "host allocation failed";
        return KV_ENOMEM;
    } catch (const std::exception &e) {
        g_err = e.what();
        return KV_EINVAL;
    }
}

kv::DTensor *T(kv_tensor h) {
    KV_REQUIRE(h && h->t, KV_EINVAL, "null tensor handle");
    return h->t.get();
}
kv::DTensor *Topt(kv_tensor h) { return (h && h->t) ? h->t.get() : nullptr; }

kv_tensor wrap(kv::TensorP t) {
    auto *h = new kv_tensor_s;
    h->t = std::move(t);
    return h;
}

void sync() {
    KV_CUDA(cudaStreamSynchronize(kv::ctx().stream));
    const int st = kv::mixed_gemm_status();
    KV_REQUIRE(st == KV_OK, st, st == KV_ETIMEOUT ? "a tensor-core GEMM wait timed out"
                                                  : "a tensor-core GEMM operand holds Inf or NaN");
}

// CUDA events owned by one call, destroyed on every exit path.
struct Events {
    std::vector<cudaEvent_t> ev;
    cudaEvent_t make(unsigned flags) {
        cudaEvent_t e;
        KV_CUDA(cudaEventCreateWithFlags(&e, flags));
        ev.push_back(e);
        return e;
    }
    ~Events() {
        for (auto e : ev) cudaEventDestroy(e);
    }
};

// Worker contexts of kv_sweep_batched, kept between calls so their plan
// caches stay warm; closed by kv_shutdown.
std::vector<std::unique_ptr<kv::Context>> g_workers;
constexpr int kDefaultBatchStreams = 8;

void close_workers() {
    for (auto &w : g_workers) kv::context_close(*w);
    g_workers.clear();
}
}  // namespace

namespace kv {
void context_open(Context &c, int device) {
    KV_CUDA(cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, device));
    KV_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    KV_CUDA(cudaHostAlloc((void **)&c.ring, (size_t)Context::kRingChunks * Context::kRingChunk, cudaHostAllocDefault));
    for (auto &e : c.ring_ev) KV_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    KV_CUDA(cudaHostAlloc((void **)&c.stop_host, sizeof(int), cudaHostAllocMapped));
    *c.stop_host = 0;
    KV_CUDA(cudaHostGetDevicePointer((void **)&c.stop_dev, c.stop_host, 0));
    for (auto &e : c.iter_ev) KV_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    c.device = device;
}

void context_close(Context &c) {
    if (c.device < 0) return;
    KV_CUDA(cudaStreamSynchronize(c.stream));
    Context *prev = &ctx();
    bind_thread_context(&c);  // plans free their buffers on their own stream
    clear_plan_cache();
    bind_thread_context(prev == &main_ctx() ? nullptr : prev);
    for (auto &e : c.ring_ev) cudaEventDestroy(e);
    cudaFreeHost(c.ring);
    c.ring = nullptr;
    for (auto &e : c.iter_ev) cudaEventDestroy(e);
    cudaFreeHost(c.stop_host);
    c.stop_host = c.stop_dev = nullptr;
    for (auto &e : c.ev_free) cudaEventDestroy(e);
    c.ev_free.clear();
    KV_CUDA(cudaStreamSynchronize(c.stream));
    KV_CUDA(cudaStreamDestroy(c.stream));
    c.stream = nullptr;
    c.device = -1;
}
}  // namespace kv

extern "C" {

int kv_version(void) { return 1; }

const char *kv_last_error(void) { return g_err.c_str(); }

int kv_init(int device) {
    return guard([&] {
        auto &c = kv::main_ctx();
        if (c.device == device && c.stream) return;
        KV_REQUIRE(c.device < 0, KV_EINVAL, "kv_init already called for another device");
        int n = 0;
        KV_CUDA(cudaGetDeviceCount(&n));
        KV_REQUIRE(device >= 0 && device < n, KV_EINVAL, "no such CUDA device");
        KV_CUDA(cudaSetDevice(device));
        cudaMemPool_t pool;
        KV_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
        uint64_t thr = ~0ull;  // keep freed blocks cached in the pool
        KV_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
        kv::context_open(c, device);
    });
}

int kv_shutdown(void) {
    return guard([&] {
        auto &c = kv::main_ctx();
        if (c.device < 0) return;
        close_workers();
        kv::context_close(c);
    });
}

int kv_tensor_create(int rank, const int *dirs, int nblocks, const int *shapes, const int *qns, const double *data,
                     kv_tensor *out) {
    return guard([&] {
        kv::require_init();
        KV_REQUIRE(out && dirs && (nblocks == 0 || (shapes && qns)), KV_EINVAL, "null argument");
        *out = wrap(kv::upload_tensor(rank, dirs, nblocks, shapes, qns, data));
        sync();
    });
}

int kv_tensor_info(kv_tensor t, int *rank, int *nblocks, long long *nelem) {
    return guard([&] {
        kv::DTensor *x = T(t);
        if (rank) *rank = x->meta.rank;
        if (nblocks) *nblocks = (int)x->meta.blocks.size();
        if (nelem) *nelem = x->meta.nelem;
    });
}

int kv_tensor_download(kv_tensor t, int *dirs, int *shapes, int *qns, double *data) {
    return guard([&] {
        kv::require_init();
        kv::download_tensor(*T(t), dirs, shapes, qns, data);
    });
}

int kv_tensor_free(kv_tensor t) {
    return guard([&] { delete t; });
}

int kv_product(kv_tensor A, kv_tensor B, int nc, int opA, int opB, int precision, kv_tensor *out) {
    return guard([&] {
        kv::require_init();
        *out = wrap(kv::op_product(*T(A), *T(B), nc, opA, opB, precision));
        sync();
    });
}

int kv_heff_apply(int nsite, kv_tensor L, kv_tensor psi, kv_tensor W1, kv_tensor W2, kv_tensor R, double scale,
                  int precision, kv_tensor *out) {
    return guard([&] {
        kv::require_init();
        KV_REQUIRE(nsite >= 0 && nsite <= 2, KV_EINVAL, "nsite must be 0, 1 or 2");
        KV_REQUIRE(nsite < 1 || Topt(W1), KV_EINVAL, "W1 required");
        KV_REQUIRE(nsite < 2 || Topt(W2), KV_EINVAL, "W2 required");
        *out = wrap(kv::op_heff(nsite, *T(L), *T(psi), Topt(W1), Topt(W2), *T(R), scale, precision));
        sync();
    });
}

int kv_env_update(int l2r, kv_tensor env, kv_tensor A, kv_tensor W, int precision, kv_tensor *out) {
    return guard([&] {
        kv::require_init();
        *out = wrap(kv::op_env(l2r != 0, *T(env), *T(A), *T(W), nullptr, precision, nullptr));
        sync();
    });
}

int kv_adjoint_heff(int nsite, kv_tensor L, kv_tensor psi, kv_tensor W1, kv_tensor W2, kv_tensor R, double scale,
                    kv_tensor ybar, int precision, kv_tensor *psi_bar, kv_tensor *L_bar, kv_tensor *W1_bar,
                    kv_tensor *W2_bar, kv_tensor *R_bar) {
    return guard([&] {
        kv::require_init();
        KV_REQUIRE(nsite >= 0 && nsite <= 2, KV_EINVAL, "nsite must be 0, 1 or 2");
        KV_REQUIRE(nsite < 1 || Topt(W1), KV_EINVAL, "W1 required");
        KV_REQUIRE(nsite < 2 || Topt(W2), KV_EINVAL, "W2 required");
        KV_REQUIRE(nsite >= 1 || !W1_bar, KV_EINVAL, "no W1 in the zero-site H_eff");
        KV_REQUIRE(nsite == 2 || !W2_bar, KV_EINVAL, "W2 is only in the two-site H_eff");
        unsigned want = (psi_bar ? kv::kGradPsi : 0u) | (L_bar ? kv::kGradL : 0u) | (W1_bar ? kv::kGradW1 : 0u) |
                        (W2_bar ? kv::kGradW2 : 0u) | (R_bar ? kv::kGradR : 0u);
        T(L);
        T(psi);
        T(R);
        kv::HeffGrads g = kv::op_adjoint_heff(nsite, L->t, psi->t, nsite >= 1 ? W1->t : nullptr,
                                              nsite == 2 ? W2->t : nullptr, R->t, scale, *T(ybar), precision, want);
        sync();
        if (psi_bar) *psi_bar = wrap(g.psi);
        if (L_bar) *L_bar = wrap(g.L);
        if (W1_bar) *W1_bar = wrap(g.W1);
        if (W2_bar) *W2_bar = wrap(g.W2);
        if (R_bar) *R_bar = wrap(g.R);
    });
}

int kv_adjoint_env(int l2r, kv_tensor env, kv_tensor A, kv_tensor W, kv_tensor env_out_bar, int precision,
                   kv_tensor *env_bar, kv_tensor *A_bar, kv_tensor *W_bar) {
    return guard([&] {
        kv::require_init();
        unsigned want = (env_bar ? kv::kGradEnv : 0u) | (A_bar ? kv::kGradA : 0u) | (W_bar ? kv::kGradW : 0u);
        T(env);
        T(A);
        T(W);
        kv::EnvGrads g = kv::op_adjoint_env(l2r != 0, env->t, A->t, W->t, *T(env_out_bar), precision, want);
        sync();
        if (env_bar) *env_bar = wrap(g.env);
        if (A_bar) *A_bar = wrap(g.A);
        if (W_bar) *W_bar = wrap(g.W);
    });
}

int kv_lanczos_expm(int nsite, kv_tensor L, kv_tensor psi, kv_tensor W1, kv_tensor W2, kv_tensor R, double dt,
                    int max_iter, double tol, int reverse, int precision, kv_tensor *out, int *iters) {
    return guard([&] {
        kv::require_init();
        KV_REQUIRE(nsite >= 0 && nsite <= 2, KV_EINVAL, "nsite must be 0, 1 or 2");
        KV_REQUIRE(nsite < 1 || Topt(W1), KV_EINVAL, "W1 required");
        KV_REQUIRE(nsite < 2 || Topt(W2), KV_EINVAL, "W2 required");
        kv::DevBuf st(sizeof(kv::KrylovState));
        kv::TensorP r = kv::op_lanczos(nsite, *T(L), *T(psi), Topt(W1), Topt(W2), *T(R), dt, max_iter, tol,
                                       reverse != 0, precision, st.as<kv::KrylovState>(), nullptr);
        kv::KrylovState h;
        KV_CUDA(cudaMemcpyAsync(&h, st.p, sizeof(h), cudaMemcpyDeviceToHost, kv::ctx().stream));
        sync();
        KV_REQUIRE(h.status == KV_OK, h.status, "non-finite norm in the Lanczos recurrence");
        if (iters) *iters = h.iters;
        *out = wrap(r);
    });
}

int kv_svd_truncate(kv_tensor A, int r1, int l2r, double tol, int max_dim, int precision, kv_tensor *U, kv_tensor *V,
                    int *n_kept, int *n_total) {
    return guard([&] {
        kv::require_init();
        KV_REQUIRE(precision >= KV_FP64 && precision <= KV_MIXED_SVD, KV_EINVAL, "unknown precision mode");
        kv::SvdOut r = kv::op_svd(*T(A), r1, l2r != 0, tol, max_dim, precision);
        sync();
        *U = wrap(r.U);
        *V = wrap(r.V);
        if (n_kept) *n_kept = r.n_kept;
        if (n_total) *n_total = r.n_total;
    });
}

int kv_tdvp_create(int nsites, const kv_tensor *mps, const kv_tensor *mpo, double tol_svd, double tol_exp,
                   int max_dim, int max_iter, double dt, int precision, kv_tdvp *out) {
    return guard([&] {
        kv::require_init();
        KV_REQUIRE(nsites >= 2 && mps && mpo, KV_EINVAL, "need >= 2 sites");
        std::vector<kv::TensorP> a, w;
        for (int i = 0; i < nsites; ++i) {
            T(mps[i]);
            T(mpo[i]);
            a.push_back(mps[i]->t);
            w.push_back(mpo[i]->t);
        }
        auto *h = new kv_tdvp_s;
        try {
            h->s.reset(new kv::Tdvp(a, w, tol_svd, tol_exp, max_dim, max_iter, dt, precision));
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

int kv_tdvp_sweep(kv_tdvp s, int mode) {
    return guard([&] {
        kv::require_init();
        KV_REQUIRE(s && s->s, KV_EINVAL, "null TDVP handle");
        if (mode == 1) s->s->one_site();
        else if (mode == 2) s->s->two_site();
        else if (mode == 0) s->s->global_krylov();
        else if (mode == 3) s->s->sa_site();
        else throw kv::Error(KV_EINVAL, "mode must be 0, 1, 2 or 3");
    });
}

int kv_tdvp_svs(kv_tdvp s, int *n_records, long long *n_values, int *counts, double *values) {
    return guard([&] {
        kv::require_init();
        KV_REQUIRE(s && s->s, KV_EINVAL, "null TDVP handle");
        s->s->svs_on = true;
        auto &v = s->s->svs;
        long long nv = 0;
        for (auto &r : v) nv += (long long)r.size();
        if (n_records) *n_records = (int)v.size();
        if (n_values) *n_values = nv;
        if (!values) return;
        KV_REQUIRE(counts, KV_EINVAL, "null count array");
        long long k = 0;
        for (size_t i = 0; i < v.size(); ++i) {
            counts[i] = (int)v[i].size();
            for (double x : v[i]) values[k++] = x;
        }
        v.clear();
    });
}

int kv_tdvp_set_sa(kv_tdvp s, const double *beta, int nbeta, unsigned long long seed, long long *added_last) {
    return guard([&] {
        kv::require_init();
        KV_REQUIRE(s && s->s, KV_EINVAL, "null TDVP handle");
        if (added_last) *added_last = s->s->sa_added;
        if (beta) s->s->set_sa(beta, nbeta, seed);
    });
}

int kv_sweep_batched(int n_chains, const kv_tdvp *chains, int mode, int steps, int max_streams, double *device_ms) {
    return guard([&] {
        kv::require_init();
        KV_REQUIRE(n_chains >= 0 && (n_chains == 0 || chains), KV_EINVAL, "null chain array");
        KV_REQUIRE(mode >= 0 && mode <= 3, KV_EINVAL, "mode must be 0, 1, 2 or 3");
        KV_REQUIRE(steps >= 0, KV_EINVAL, "steps must be >= 0");
        std::set<const kv_tdvp_s *> seen;
        for (int i = 0; i < n_chains; ++i) {
            KV_REQUIRE(chains[i] && chains[i]->s, KV_EINVAL, "null TDVP handle");
            KV_REQUIRE(seen.insert(chains[i]).second, KV_EINVAL, "a chain appears twice");
        }
        if (device_ms) *device_ms = 0.0;
        if (n_chains == 0 || steps == 0) return;
        auto &m = kv::main_ctx();
        KV_REQUIRE(&kv::ctx() == &m, KV_EINVAL, "kv_sweep_batched called from a worker");
        const int nw = std::min(n_chains, max_streams > 0 ? max_streams : kDefaultBatchStreams);
        while ((int)g_workers.size() < nw) {
            auto w = std::make_unique<kv::Context>();
            kv::context_open(*w, m.device);
            g_workers.push_back(std::move(w));
        }
        // Longest first, each chain to the least-loaded worker, by an estimate
        // of its work (sum over sites of |A|^1.5); deterministic, so a chain
        // returns to the same worker and finds its H_eff plans cached there.
        std::vector<double> cost(n_chains, 0.0);
        for (int i = 0; i < n_chains; ++i)
            for (auto &a : chains[i]->s->mps) cost[i] += std::pow((double)a->meta.nelem, 1.5);
        std::vector<int> order(n_chains);
        for (int i = 0; i < n_chains; ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
        std::vector<std::vector<int>> assign(nw);
        std::vector<double> load(nw, 0.0);
        for (int i : order) {
            const int w = (int)(std::min_element(load.begin(), load.end()) - load.begin());
            assign[w].push_back(i);
            load[w] += cost[i];
        }
        // every worker stream starts after everything on the main stream
        Events ev;
        cudaEvent_t t0 = ev.make(cudaEventDefault), t1 = ev.make(cudaEventDefault);
        KV_CUDA(cudaEventRecord(t0, m.stream));
        std::vector<cudaEvent_t> done(nw);
        for (auto &e : done) e = ev.make(cudaEventDisableTiming);
        std::vector<int> code(n_chains, KV_OK), wcode(nw, KV_OK);
        std::vector<std::string> msg(n_chains), wmsg(nw);
        std::vector<std::thread> th;
        auto join_all = [&] {
            for (auto &x : th)
                if (x.joinable()) x.join();
        };
        auto body = [&](int w) {
            kv::Context *c = g_workers[w].get();
            wcode[w] = guard([&] {
                KV_CUDA(cudaSetDevice(c->device));
                KV_CUDA(cudaStreamWaitEvent(c->stream, t0, 0));
            });
            if (wcode[w] != KV_OK) {
                wmsg[w] = g_err;
                return;
            }
            kv::bind_thread_context(c);
            for (int i : assign[w]) {
                kv::Tdvp &t = *chains[i]->s;
                code[i] = guard([&] {
                    for (int s = 0; s < steps; ++s) {
                        if (mode == 0) t.global_krylov();
                        else if (mode == 1) t.one_site();
                        else if (mode == 3) t.sa_site();
                        else t.two_site();
                    }
                });
                if (code[i] != KV_OK) msg[i] = g_err;
            }
            wcode[w] = guard([&] {
                KV_CUDA(cudaEventRecord(done[w], c->stream));
                KV_CUDA(cudaStreamSynchronize(c->stream));
            });
            if (wcode[w] != KV_OK) wmsg[w] = g_err;
            kv::bind_thread_context(nullptr);
        };
        try {
            for (int w = 0; w < nw; ++w) th.emplace_back(body, w);
        } catch (...) {  // a thread could not be started: wait for the others, then report
            join_all();
            throw;
        }
        join_all();
        for (int w = 0; w < nw; ++w) {
            m.launches += g_workers[w]->launches;
            g_workers[w]->launches = 0;
            if (wcode[w] == KV_OK) KV_CUDA(cudaStreamWaitEvent(m.stream, done[w], 0));
        }
        KV_CUDA(cudaEventRecord(t1, m.stream));
        sync();
        float ms = 0.0f;
        KV_CUDA(cudaEventElapsedTime(&ms, t0, t1));
        if (device_ms) *device_ms = ms;
        for (int w = 0; w < nw; ++w)
            KV_REQUIRE(wcode[w] == KV_OK, wcode[w], "batched sweep, stream " + std::to_string(w) + ": " + wmsg[w]);
        for (int i = 0; i < n_chains; ++i)
            KV_REQUIRE(code[i] == KV_OK, code[i], "batched sweep, chain " + std::to_string(i) + ": " + msg[i]);
    });
}

int kv_tdvp_window(kv_tdvp s, int i0, int n) {
    return guard([&] {
        kv::require_init();
        KV_REQUIRE(s && s->s, KV_EINVAL, "null TDVP handle");
        s->s->window(i0, n);
    });
}

int kv_tdvp_site(kv_tdvp s, int i, kv_tensor *out) {
    return guard([&] {
        KV_REQUIRE(s && s->s && i >= 0 && i < (int)s->s->mps.size(), KV_EINVAL, "bad site index");
        *out = wrap(kv::clone(*s->s->mps[i]));
        sync();
    });
}

int kv_tdvp_stats(kv_tdvp s, double *module_ms, double *sweep_ms, double *ref_flops, double *gemm_ref_flops) {
    return guard([&] {
        KV_REQUIRE(s && s->s, KV_EINVAL, "null TDVP handle");
        if (module_ms)
            for (int i = 0; i < kv::MOD_COUNT; ++i) module_ms[i] = s->s->module_ms[i];
        if (sweep_ms) *sweep_ms = s->s->sweep_ms;
        if (ref_flops) *ref_flops = s->s->last_ref_flops;
        if (gemm_ref_flops) *gemm_ref_flops = s->s->last_gemm_flops;
    });
}

int kv_tdvp_host_stats(kv_tdvp s, double *module_host_ms, double *sweep_host_ms, long long *plans_built,
                       double *plan_ms) {
    return guard([&] {
        KV_REQUIRE(s && s->s, KV_EINVAL, "null TDVP handle");
        if (module_host_ms)
            for (int i = 0; i < kv::MOD_COUNT; ++i) module_host_ms[i] = s->s->module_host_ms[i];
        if (sweep_host_ms) *sweep_host_ms = s->s->sweep_host_ms;
        if (plans_built) *plans_built = s->s->plans_built;
        if (plan_ms) *plan_ms = s->s->plan_ms;
    });
}

int kv_profile(int enable) {
    return guard([&] {
        kv::require_init();
        kv::ctx().prof = enable != 0;
    });
}

static int profile_read_bytes(int kind, double *ms, double *bytes, long long *launches) {
    return guard([&] {
        kv::require_init();
        auto &c = kv::ctx();
        if (ms) *ms = c.bw_ms[kind];
        if (bytes) *bytes = c.bw_bytes[kind];
        if (launches) *launches = c.bw_launches[kind];
        c.bw_ms[kind] = c.bw_bytes[kind] = 0.0;
        c.bw_launches[kind] = 0;
    });
}

int kv_profile_read_lanczos(double *ms, double *bytes, long long *launches) {
    return profile_read_bytes(kv::kProfLanczos, ms, bytes, launches);
}

int kv_profile_read_mix(double *ms, double *bytes, long long *launches) {
    return profile_read_bytes(kv::kProfMix, ms, bytes, launches);
}

int kv_profile_read(double *gemm_ms, double *gemm_ref_flops, long long *gemm_launches) {
    return guard([&] {
        kv::require_init();
        kv::prof_resolve(nullptr, nullptr);
        auto &c = kv::ctx();
        if (gemm_ms) *gemm_ms = c.prof_ms;
        if (gemm_ref_flops) *gemm_ref_flops = c.prof_flops;
        if (gemm_launches) *gemm_launches = c.prof_launches;
        c.prof_ms = c.prof_flops = 0.0;
        c.prof_launches = 0;
    });
}

int kv_debug_gemm_stall(int on) {
    return guard([&] {
        kv::require_init();
        KV_CUDA(cudaStreamSynchronize(kv::ctx().stream));
        kv::set_gemm_stall_test(on);
    });
}

int kv_svd_stats(int reset, long long *sectors, long long *columns, long long *rank, long long *sweeps,
                 int *max_sweeps) {
    return guard([&] {
        kv::require_init();
        auto &v = kv::ctx().svd;
        if (sectors) *sectors = v.sectors;
        if (columns) *columns = v.columns;
        if (rank) *rank = v.rank;
        if (sweeps) *sweeps = v.sweeps;
        if (max_sweeps) *max_sweeps = v.max_sweeps;
        if (reset) v = kv::Context::SvdStats{};
    });
}

int kv_krylov_stats(int reset, long long *calls, long long *issued, long long *used) {
    return guard([&] {
        kv::require_init();
        auto &c = kv::ctx();
        if (calls) *calls = c.krylov_calls;
        if (issued) *issued = c.krylov_issued;
        if (used) *used = c.krylov_used;
        if (reset) c.krylov_calls = c.krylov_issued = c.krylov_used = 0;
    });
}

int kv_debug_pool_usage(int reset_high, long long *used_current, long long *used_high) {
    return guard([&] {
        kv::require_init();
        KV_CUDA(cudaStreamSynchronize(kv::ctx().stream));
        cudaMemPool_t pool;
        KV_CUDA(cudaDeviceGetDefaultMemPool(&pool, kv::ctx().device));
        unsigned long long cur = 0, high = 0;
        if (reset_high) {
            unsigned long long zero = 0;  // resets the high-water mark to the current use
            KV_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &zero));
        }
        KV_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &cur));
        KV_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &high));
        if (used_current) *used_current = (long long)cur;
        if (used_high) *used_high = (long long)high;
    });
}

int kv_counters(long long *launches) {
    return guard([&] {
        if (launches) *launches = kv::ctx().launches;
    });
}

int kv_tdvp_free(kv_tdvp s) {
    return guard([&] { delete s; });
}

int kv_canonicalize(int nsites, const kv_tensor *mps, double tol_svd, int max_dim, int precision, kv_tensor *out) {
    return guard([&] {
        kv::require_init();
        KV_REQUIRE(nsites >= 1 && mps && out, KV_EINVAL, "null argument");
        std::vector<kv::TensorP> in;
        for (int i = 0; i < nsites; ++i) in.push_back(kv::clone(*T(mps[i])));
        std::vector<kv::TensorP> r = kv::op_canonicalize(in, tol_svd, max_dim, precision);
        sync();
        for (int i = 0; i < nsites; ++i) out[i] = wrap(r[i]);
    });
}

int kv_expectation(int nsites, const kv_tensor *bra, const kv_tensor *mpo, const kv_tensor *ket, double *re,
                   double *im) {
    return guard([&] {
        kv::require_init();
        std::vector<kv::DTensor *> a, w, b;
        for (int i = 0; i < nsites; ++i) {
            a.push_back(T(bra[i]));
            w.push_back(T(mpo[i]));
            b.push_back(T(ket[i]));
        }
        kv::cplx r = kv::op_expectation(a, w, b);
        *re = r.real();
        *im = r.imag();
    });
}

int kv_local_expectations(int nsites, const kv_tensor *mps, const kv_tensor *ident_mpo, int nops, const int *op_site,
                          const kv_tensor *op_tensor, double *re, double *im) {
    return guard([&] {
        kv::require_init();
        KV_REQUIRE(nsites >= 1 && nops >= 0 && mps && ident_mpo && (nops == 0 || (op_site && op_tensor && re && im)),
                   KV_EINVAL, "null argument");
        std::vector<kv::DTensor *> a, w, o;
        for (int i = 0; i < nsites; ++i) {
            a.push_back(T(mps[i]));
            w.push_back(T(ident_mpo[i]));
        }
        std::vector<int> sites(op_site, op_site + nops);
        for (int k = 0; k < nops; ++k) o.push_back(T(op_tensor[k]));
        std::vector<kv::cplx> r = kv::op_local_expectations(a, w, sites, o);
        for (int k = 0; k < nops; ++k) {
            re[k] = r[k].real();
            im[k] = r[k].imag();
        }
    });
}

int kv_expectation_noalloc(int nsites, const kv_tensor *bra, const kv_tensor *mpo, const kv_tensor *ket, double *re,
                           double *im) {
    return guard([&] {
        kv::require_init();
        KV_REQUIRE(nsites >= 1 && bra && mpo && ket && re && im, KV_EINVAL, "null argument");
        std::vector<kv::DTensor *> a, w, b;
        for (int i = 0; i < nsites; ++i) {
            a.push_back(T(bra[i]));
            w.push_back(T(mpo[i]));
            b.push_back(T(ket[i]));
        }
        kv::cplx r = kv::expectation_noalloc(a, w, b);
        *re = r.real();
        *im = r.imag();
    });
}

}  // extern "C"
