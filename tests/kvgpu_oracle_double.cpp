// Test double of libkvgpu's C ABI for host-side tests of the C++ layer
// (include/holstein/: kv_ops.h and the TDVP driver layer of kv_holstein.h):
// the entry points that layer calls, with the same signatures and argument
// meaning as include/kvgpu.h, answered by the CPU oracle
// (oracle/_build/libkvoracle.so) instead of the GPU.  The sweep timings it
// reports are zeros and it keeps no singular-value record.  Built by the
// tests (kvtest_util.build_abi_double) into a temporary libkvgpu.so; it never
// ships and is never loaded by the product path.
#include <cstring>
#include <string>
#include <vector>

#include "kvgpu.h"

extern "C" {
const char *kvo_last_error();
int kvo_tensor_new(int rank, const int *dirs, int nblocks, const int *shapes, const int *qns, const double *data,
                   void **out);
int kvo_tensor_info(void *h, int *rank, int *nblocks, long long *nelem);
int kvo_tensor_get(void *h, int *dirs, int *shapes, int *qns, double *data);
void kvo_tensor_free(void *h);
int kvo_product(void *a, void *b, int nc, int ta, int tb, void **out);
int kvo_apply(int nsite, void *L, void *psi, void *W1, void *W2, void *R, void **out);
int kvo_env_sweep(void *env, void *A, void *W, int l2r, void **out);
int kvo_local_krylov(int nsite, void *L, void *psi, void *W1, void *W2, void *R, double dt, int max_iter, double tol,
                     int reverse, int *iters, void **out);
int kvo_svd(void *A, int r1, int l2r, double tol, int max_dim, void **U, void **V, double *svals, int *nkept,
            int *ntotal);
int kvo_join(int ns, void **a, void **w, void **b, double *re, double *im);
int kvo_tdvp_new(int ns, void **mps, void **mpo, double tol_svd, double tol_exp, int max_dim, int max_iter,
                 double dt, void **out);
int kvo_tdvp_sweep(void *h, int mode);
int kvo_tdvp_set_sa(void *h, const double *beta, int nbeta, unsigned long long seed);
int kvo_tdvp_site(void *h, int i, void **out);
void kvo_tdvp_free(void *h);
}

namespace {

std::string g_err;
long long g_calls = 0;  // operations answered (tensor I/O excluded)

void *H(kv_tensor t) { return static_cast<void *>(t); }
kv_tensor T(void *p) { return static_cast<kv_tensor>(p); }

int status(int rc) {
    if (rc == 0) return KV_OK;
    g_err = kvo_last_error();
    return KV_EINVAL;
}

}  // namespace

extern "C" {

int kv_init(int) { return KV_OK; }
int kv_shutdown(void) { return KV_OK; }
const char *kv_last_error(void) { return g_err.c_str(); }
long long kv_double_calls(void) { return g_calls; }

int kv_tensor_create(int rank, const int *dirs, int nblocks, const int *shapes, const int *qns, const double *data,
                     kv_tensor *out) {
    std::vector<double> zeros;
    if (!data) {
        long long n = 0;
        for (int b = 0; b < nblocks; ++b) {
            long long s = 1;
            for (int i = 0; i < rank; ++i) s *= shapes[b * rank + i];
            n += s;
        }
        zeros.assign(2 * (size_t)n + 2, 0.0);
        data = zeros.data();
    }
    void *h = nullptr;
    const int rc = kvo_tensor_new(rank, dirs, nblocks, shapes, qns, data, &h);
    *out = T(h);
    return status(rc);
}

int kv_tensor_info(kv_tensor t, int *rank, int *nblocks, long long *nelem) {
    return status(kvo_tensor_info(H(t), rank, nblocks, nelem));
}

int kv_tensor_download(kv_tensor t, int *dirs, int *shapes, int *qns, double *data) {
    return status(kvo_tensor_get(H(t), dirs, shapes, qns, data));
}

int kv_tensor_free(kv_tensor t) {
    kvo_tensor_free(H(t));
    return KV_OK;
}

int kv_product(kv_tensor A, kv_tensor B, int nc, int opA, int opB, int, kv_tensor *out) {
    ++g_calls;
    void *h = nullptr;
    const int rc = kvo_product(H(A), H(B), nc, opA, opB, &h);
    *out = T(h);
    return status(rc);
}

int kv_heff_apply(int nsite, kv_tensor L, kv_tensor psi, kv_tensor W1, kv_tensor W2, kv_tensor R, double scale, int,
                  kv_tensor *out) {
    ++g_calls;
    void *h = nullptr;
    int rc = kvo_apply(nsite, H(L), H(psi), H(W1), H(W2), H(R), &h);
    if (rc == 0 && scale != 1.0) {  // the oracle applies H_eff unscaled
        int rank = 0, nb = 0;
        long long ne = 0;
        kvo_tensor_info(h, &rank, &nb, &ne);
        std::vector<int> dirs(rank), sh((size_t)nb * rank), qn((size_t)nb * rank);
        std::vector<double> d(2 * (size_t)ne + 2);
        kvo_tensor_get(h, dirs.data(), sh.data(), qn.data(), d.data());
        for (auto &x : d) x *= scale;
        kvo_tensor_free(h);
        rc = kvo_tensor_new(rank, dirs.data(), nb, sh.data(), qn.data(), d.data(), &h);
    }
    *out = T(h);
    return status(rc);
}

int kv_env_update(int l2r, kv_tensor env, kv_tensor A, kv_tensor W, int, kv_tensor *out) {
    ++g_calls;
    void *h = nullptr;
    const int rc = kvo_env_sweep(H(env), H(A), H(W), l2r, &h);
    *out = T(h);
    return status(rc);
}

int kv_lanczos_expm(int nsite, kv_tensor L, kv_tensor psi, kv_tensor W1, kv_tensor W2, kv_tensor R, double dt,
                    int max_iter, double tol, int reverse, int, kv_tensor *out, int *iters) {
    ++g_calls;
    void *h = nullptr;
    int it = 0;
    const int rc = kvo_local_krylov(nsite, H(L), H(psi), H(W1), H(W2), H(R), dt, max_iter, tol, reverse, &it, &h);
    *out = T(h);
    if (iters) *iters = it;
    return status(rc);
}

int kv_svd_truncate(kv_tensor A, int r1, int l2r, double tol, int max_dim, int, kv_tensor *U, kv_tensor *V,
                    int *n_kept, int *n_total) {
    ++g_calls;
    void *u = nullptr, *v = nullptr;
    int nk = 0, nt = 0;
    const int rc = kvo_svd(H(A), r1, l2r, tol, max_dim, &u, &v, nullptr, &nk, &nt);
    *U = T(u);
    *V = T(v);
    if (n_kept) *n_kept = nk;
    if (n_total) *n_total = nt;
    return status(rc);
}

// State::canonicalize by the reference's sequence of SVDs and products
// (holstein/state.h:166-185) on the oracle's primitives
int kv_canonicalize(int nsites, const kv_tensor *mps, double tol_svd, int max_dim, int, kv_tensor *out) {
    ++g_calls;
    std::vector<void *> t(nsites);
    auto copy = [](void *h) {  // a fresh oracle tensor equal to h
        int rank = 0, nb = 0;
        long long ne = 0;
        kvo_tensor_info(h, &rank, &nb, &ne);
        std::vector<int> dirs(rank), sh((size_t)nb * rank), qn((size_t)nb * rank);
        std::vector<double> d(2 * (size_t)ne + 2);
        kvo_tensor_get(h, dirs.data(), sh.data(), qn.data(), d.data());
        void *c = nullptr;
        kvo_tensor_new(rank, dirs.data(), nb, sh.data(), qn.data(), d.data(), &c);
        return c;
    };
    for (int i = 0; i < nsites; ++i) t[i] = copy(H(mps[i]));
    int rc = 0;
    for (int i = 0; i + 1 < nsites && rc == 0; ++i) {
        void *u = nullptr, *v = nullptr, *nx = nullptr;
        int nk = 0, nt = 0;
        rc = kvo_svd(t[i], 2, 1, tol_svd, max_dim, &u, &v, nullptr, &nk, &nt);
        if (rc == 0) rc = kvo_product(v, t[i + 1], 1, KV_OP_N, KV_OP_N, &nx);
        if (rc != 0) break;
        kvo_tensor_free(t[i]);
        kvo_tensor_free(t[i + 1]);
        kvo_tensor_free(v);
        t[i] = u;
        t[i + 1] = nx;
    }
    for (int i = nsites - 1; i > 0 && rc == 0; --i) {
        void *u = nullptr, *v = nullptr, *pv = nullptr;
        int nk = 0, nt = 0;
        rc = kvo_svd(t[i], 1, 0, tol_svd, max_dim, &u, &v, nullptr, &nk, &nt);
        if (rc == 0) rc = kvo_product(t[i - 1], u, 1, KV_OP_N, KV_OP_N, &pv);
        if (rc != 0) break;
        kvo_tensor_free(t[i]);
        kvo_tensor_free(t[i - 1]);
        kvo_tensor_free(u);
        t[i] = v;
        t[i - 1] = pv;
    }
    for (int i = 0; i < nsites; ++i) out[i] = T(t[i]);
    return status(rc);
}

int kv_expectation(int nsites, const kv_tensor *bra, const kv_tensor *mpo, const kv_tensor *ket, double *re,
                   double *im) {
    ++g_calls;
    std::vector<void *> a(bra, bra + nsites), w(mpo, mpo + nsites), b(ket, ket + nsites);
    return status(kvo_join(nsites, a.data(), w.data(), b.data(), re, im));
}

int kv_tdvp_create(int nsites, const kv_tensor *mps, const kv_tensor *mpo, double tol_svd, double tol_exp,
                   int max_dim, int max_iter, double dt, int, kv_tdvp *out) {
    std::vector<void *> m(mps, mps + nsites), w(mpo, mpo + nsites);
    void *h = nullptr;
    const int rc = kvo_tdvp_new(nsites, m.data(), w.data(), tol_svd, tol_exp, max_dim, max_iter, dt, &h);
    *out = static_cast<kv_tdvp>(h);
    return status(rc);
}

int kv_tdvp_sweep(kv_tdvp s, int mode) {
    ++g_calls;
    return status(kvo_tdvp_sweep(static_cast<void *>(s), mode));
}

int kv_tdvp_set_sa(kv_tdvp s, const double *beta, int nbeta, unsigned long long seed, long long *added_last) {
    if (added_last) *added_last = 0;
    return status(kvo_tdvp_set_sa(static_cast<void *>(s), beta, nbeta, seed));
}

int kv_tdvp_svs(kv_tdvp, int *n_records, long long *n_values, int *, double *) {
    if (n_records) *n_records = 0;
    if (n_values) *n_values = 0;
    return KV_OK;
}

int kv_tdvp_site(kv_tdvp s, int i, kv_tensor *out) {
    void *h = nullptr;
    const int rc = kvo_tdvp_site(static_cast<void *>(s), i, &h);
    *out = T(h);
    return status(rc);
}

int kv_tdvp_stats(kv_tdvp, double *module_ms, double *sweep_ms, double *ref_flops, double *gemm_ref_flops) {
    if (module_ms)
        for (int i = 0; i < 6; ++i) module_ms[i] = 0.0;
    if (sweep_ms) *sweep_ms = 0.0;
    if (ref_flops) *ref_flops = 0.0;
    if (gemm_ref_flops) *gemm_ref_flops = 0.0;
    return KV_OK;
}

int kv_tdvp_free(kv_tdvp s) {
    kvo_tdvp_free(static_cast<void *>(s));
    return KV_OK;
}

}  // extern "C"
