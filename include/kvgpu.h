/*
 * kvgpu.h -- C ABI of the GB300-native Holstein TDVP library (libkvgpu.so).
 *
 * The reference (Kylin-V) has no FFI: its operator surface is the C++
 * template API of the holstein/ headers, called by src/kln-tdvp.cpp:73-78.  Each entry
 * point below replaces one function of that surface; the citation on each
 * declaration names the reference function (file:line) whose arguments,
 * results and error behaviour it mirrors.
 *
 * Conventions
 *  - Tensors are U(1) block-sparse, complex128 at the boundary.  A tensor is
 *    passed as (rank, dirs[rank], nblocks, shapes[nblocks*rank],
 *    qns[nblocks*rank], data): the reference's Tensor<Rank>/Block<Rank>
 *    (holstein/tensor.h:16-209, holstein/block.h:23-166) -- leg directions,
 *    then per block its shape and per-leg charges, block data row-major and
 *    blocks concatenated in order (the same order as the .mps/.mpo files,
 *    holstein/state.h:107-128).  `data` is interleaved (re, im) doubles.
 *  - Device-resident tensors are opaque kv_tensor handles owned by the caller
 *    (kv_tensor_free).  Nothing in the ABI exposes torch or CUDA types.
 *  - Every function returns KV_OK (0) or a negative KV_E* code; it never
 *    exits the process (the reference prints and calls exit(1)).
 *    kv_last_error() returns a message for the calling thread's last error.
 *  - All work is issued on the library's CUDA stream of the current device;
 *    calls are synchronous with respect to the host unless stated otherwise.
 */
#ifndef KVGPU_H
#define KVGPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------- status codes */
#define KV_OK          0
#define KV_EINVAL     -1  /* bad argument (rank, shapes, directions, mode)   */
#define KV_ECUDA      -2  /* CUDA runtime error                             */
#define KV_ENOMEM     -3  /* device allocation failed                       */
#define KV_ENONFINITE -4  /* NaN/Inf in an operand, a norm or a singular value */
#define KV_ETIMEOUT   -5  /* a bounded device wait gave up                  */
#define KV_ENOTINIT   -6  /* kv_init not called                            */
#define KV_EMISMATCH  -7  /* contracted legs' directions mismatch           */

/* ------------------------------------------------------- arithmetic modes */
/* KV_FP64: every contraction in complex128 on the CUDA cores.
 * KV_MIXED_3M_DIGITS (the mixed-precision path): block contractions as 3M
 *   (Gauss) real products on the tcgen05 tensor cores.  Each operand is
 *   rounded to 38-bit fixed point against a per-row (A) or per-column (B)
 *   power of two and split into five balanced 8-bit digits, held exactly in
 *   FP16; the digit products of orders 0-4 accumulate exactly in FP32 tensor
 *   memory and are combined in int64, so a product carries about 1e-10
 *   relative error, far below a TF32 or BF16x3 split.  Lanczos,
 *   norms, the tridiagonal exponential and MPO mixing stay FP64; the SVD
 *   picks the kept subspace in FP32 and rebuilds the kept factors in FP64
 *   (Cholesky-QR, exact projection).
 * KV_MIXED_TF32, KV_MIXED_3M_TF32 and KV_MIXED_3M_BF16X3 are other names of
 *   the same mode, kept so code written against the mixed-precision names
 *   of the survey compiles: no TF32 or BF16 split is implemented, because
 *   the digit products are more accurate than either at the same tensor
 *   pipe cost per exact product. */
#define KV_FP64             0
#define KV_MIXED_3M_DIGITS  1
#define KV_MIXED_TF32       KV_MIXED_3M_DIGITS
#define KV_MIXED_3M_TF32    KV_MIXED_3M_DIGITS
#define KV_MIXED_3M_BF16X3  KV_MIXED_3M_DIGITS
/* one part mixed, the other FP64 (to attribute mixed-precision error):
 * KV_MIXED_GEMM = tensor-core contractions + FP64 SVD,
 * KV_MIXED_SVD  = FP64 contractions + mixed SVD */
#define KV_MIXED_GEMM  2
#define KV_MIXED_SVD   3

/* contraction operand modes (numerically the CBLAS ones the reference uses) */
#define KV_OP_N 111
#define KV_OP_T 112
#define KV_OP_C 113

typedef struct kv_tensor_s *kv_tensor;
typedef struct kv_tdvp_s *kv_tdvp;

/* Library lifetime: select the device and create the stream / pools. */
int kv_init(int device);
int kv_shutdown(void);
const char *kv_last_error(void);
int kv_version(void);

/* -------------------------------------------------------------- tensors */
/* Upload a block tensor to the device.  data may be NULL (zero blocks).
 * Replaces constructing Tensor<Rank> from Blocks (holstein/tensor.h:55-77,
 * holstein/state.h:130-157 for the file order). */
int kv_tensor_create(int rank, const int *dirs, int nblocks, const int *shapes, const int *qns,
                     const double *data, kv_tensor *out);
/* rank, block count and total complex elements */
int kv_tensor_info(kv_tensor t, int *rank, int *nblocks, long long *nelem);
/* Download: dirs[rank], shapes/qns[nblocks*rank], data[2*nelem]. */
int kv_tensor_download(kv_tensor t, int *dirs, int *shapes, int *qns, double *data);
int kv_tensor_free(kv_tensor t);

/* -------------------------------------------------------- primitives */
/* product<N1,N2,nc>(A, B, opA, opB): contract the last nc legs of op(A) with
 * the first nc legs of op(B); opA in {N, C}, opB in {N, T}.
 * holstein/product.h:61-201 */
int kv_product(kv_tensor A, kv_tensor B, int nc, int opA, int opB, int precision, kv_tensor *out);

/* H_eff . psi for nsite = 0 (apply_zero, holstein/product.h:540-545; W1, W2
 * unused), 1 (apply_single, holstein/product.h:547-553; W2 unused) or 2
 * (apply_double, holstein/product.h:478-486).  Result scaled by `scale`. */
int kv_heff_apply(int nsite, kv_tensor L, kv_tensor psi, kv_tensor W1, kv_tensor W2, kv_tensor R,
                  double scale, int precision, kv_tensor *out);

/* Environment update env_sweep(env, A, W, l2r) (holstein/product.h:488-503). */
int kv_env_update(int l2r, kv_tensor env, kv_tensor A, kv_tensor W, int precision, kv_tensor *out);
/* Adjoints (vector-Jacobian products).  No reference counterpart: the
 * reference has no derivative code.  For a real loss l, a cotangent is
 * xbar = dl/dRe(x) + i dl/dIm(x) (so dl = Re<ybar, dy>, and for y linear in x,
 * xbar = (dy/dx)^H ybar).  kv_adjoint_heff: given ybar for
 * y = kv_heff_apply(nsite, L, psi, W1, W2, R, scale), returns the cotangents
 * of psi, L, W1, W2 (two-site only) and R; pass NULL for any not wanted.
 * kv_adjoint_env: given the cotangent of out = kv_env_update(l2r, env, A, W),
 * returns those of env, A (through both its bra and ket use) and W.  Each
 * cotangent tensor holds every charge block the contraction reaches, which
 * can be more blocks than the primal tensor has; only the primal's blocks
 * pair with a perturbation of it.  The contractions run in `precision`. */
int kv_adjoint_heff(int nsite, kv_tensor L, kv_tensor psi, kv_tensor W1, kv_tensor W2, kv_tensor R, double scale,
                    kv_tensor ybar, int precision, kv_tensor *psi_bar, kv_tensor *L_bar, kv_tensor *W1_bar,
                    kv_tensor *W2_bar, kv_tensor *R_bar);
int kv_adjoint_env(int l2r, kv_tensor env, kv_tensor A, kv_tensor W, kv_tensor out_bar, int precision,
                   kv_tensor *env_bar, kv_tensor *A_bar, kv_tensor *W_bar);

/* local_krylov<Rank> (holstein/exponential.h:92-190): psi <- exp(-+i H_eff dt/2) psi
 * (normalised first), Lanczos while k < max_iter-1 and the product of Lanczos
 * norms exceeds tol; reverse selects exp(+i ...).  psi is replaced by a new
 * device tensor (the old handle stays valid and unchanged).  iters receives
 * the Krylov dimension used. */
int kv_lanczos_expm(int nsite, kv_tensor L, kv_tensor psi, kv_tensor W1, kv_tensor W2, kv_tensor R,
                    double dt, int max_iter, double tol, int reverse, int precision, kv_tensor *out,
                    int *iters);

/* svd_impl<R1,R2>(A, cfg, -1) (holstein/svd.h:296-440): block SVD per charge
 * sector with the reference's global truncation (keep while index < max_dim
 * and s > tol, never fewer than one).  l2r folds S into V (S.Vt), else into U.
 * n_kept / n_total receive the kept and total singular-value counts.
 * KV_FP64: FP64 one-sided Jacobi.  KV_MIXED_TF32: FP32 one-sided Jacobi
 * chooses the kept subspace and the truncation, then the kept factor is made
 * orthonormal in FP64 (Cholesky-QR) and the other factor is the exact FP64
 * projection of the sector matrix onto it. */
int kv_svd_truncate(kv_tensor A, int r1, int l2r, double tol, int max_dim, int precision, kv_tensor *U,
                    kv_tensor *V, int *n_kept, int *n_total);

/* ---------------------------------------------------- sweep driver */
/* TDVP(State, Operator, tolSVD, tolExp, maxDim, maxIter, dt) followed by the
 * environment set-up of total_start (holstein/tdvp.h:60-76, 303-316).
 * mps/mpo are arrays of nsites tensor handles (copied). */
int kv_tdvp_create(int nsites, const kv_tensor *mps, const kv_tensor *mpo, double tol_svd, double tol_exp,
                   int max_dim, int max_iter, double dt, int precision, kv_tdvp *out);
/* One time step: mode 1 = TDVP::one_site (holstein/tdvp.h:78-141),
 * mode 2 = TDVP::two_site (holstein/tdvp.h:144-227), mode 0 = one step of
 * total_start's global-Krylov stage (holstein/tdvp.h:318-327, global_main in
 * holstein/krylov.h:199-283: a Krylov basis of whole MPSs, the MPO scaled by
 * dt, tolExp / maxIter / tolSVD / maxDim as given); after it the sweep
 * environments are rebuilt from the new state (the reference keeps the ones
 * built before that stage, so its next sweep mixes two states).  The global
 * step's contractions run in `precision`, its SVDs in FP64.  mode 3 = one
 * SA-1TDVP sweep, TDVP::sa_site (holstein/tdvp.h:230-294) with the widths
 * and seed of kv_tdvp_set_sa: one_site with sa_svd_impl's split
 * (holstein/svd.h:443-614; FP64 SVD in every precision mode). */
int kv_tdvp_sweep(kv_tdvp s, int mode);
/* SA-1TDVP settings: beta[i] is bond i's width (betaSet[i] of
 * holstein/tdvp.h:343-358, i.e. 1 / the fitted value bin/nls.py writes),
 * nbeta >= nsites - 1; seed starts the seed stream.  The reference seeds a
 * fresh mt19937 from std::random_device before each group of draws (one
 * synthetic singular value; one new vector); here each group's mt19937 is
 * seeded by the next 32-bit value of an mt19937 stream started at `seed`, so a
 * run repeats.  beta == NULL leaves the settings unchanged.  added_last (may
 * be NULL) receives the states the SA splits of the last sweep added. */
int kv_tdvp_set_sa(kv_tdvp s, const double *beta, int nbeta, unsigned long long seed, long long *added_last);
/* The kept singular values (descending) of every two-site split since the
 * last read, the record svd_impl appends to its SVS file for the SA stage's
 * fit (holstein/svd.h:356-402, holstein/tdvp.h:166, 202).  values == NULL:
 * only the number of records and of values; else counts[n_records] and
 * values[n_values] (sized by a previous query) are filled, in order, and the
 * records are cleared.  Records are kept from the first call on a handle. */
int kv_tdvp_svs(kv_tdvp s, int *n_records, long long *n_values, int *counts, double *values);
/* A window of TDVP::two_site's left-to-right pass (holstein/tdvp.h:150-185):
 * the pass is advanced to site i0 (untimed; n = 0 does only that), then the
 * n local updates at sites (i0, i0+1) ... (i0+n-1, i0+n) run and
 * kv_tdvp_stats reports them as the last sweep.  For chains too long to sweep
 * in a benchmark run; afterwards the handle is inside the pass and takes only
 * further windows at later sites (kv_tdvp_sweep fails with KV_EINVAL). */
int kv_tdvp_window(kv_tdvp s, int i0, int n);
/* New handle with a copy of the current site tensor i. */
int kv_tdvp_site(kv_tdvp s, int i, kv_tensor *out);
/* Timings of the last one- or two-site sweep (a global-Krylov step leaves
 * them as they were): per-module device time in ms in the order
 * Evl-0, Evl-1, Evl-2, SVD, Update, Sweep (the reference's Timer modules,
 * util/timer.h:19-66, holstein/tdvp.h:85-106), the whole sweep's device
 * time, the algorithmic flop count (8*M*N*K summed over every zgemm the
 * reference issues for the same sweep, Lanczos iterations as actually run)
 * and the part of it in product<> block pairs (the grouped GEMM kernel). */
int kv_tdvp_stats(kv_tdvp s, double *module_ms, double *sweep_ms, double *ref_flops, double *gemm_ref_flops);
/* Host side of the last sweep: wall-clock ms per module (same order; the
 * reference's Timer table measures wall-clock, util/timer.h:19-66), the
 * sweep's wall-clock ms, and the H_eff plans built (plan-cache misses) with
 * the host ms spent building them.  No other reference counterpart. */
int kv_tdvp_host_stats(kv_tdvp s, double *module_host_ms, double *sweep_host_ms, long long *plans_built,
                       double *plan_ms);
int kv_tdvp_free(kv_tdvp s);
/* Advances n_chains independent chains (kv_tdvp handles, each created with
 * kv_tdvp_create) by `steps` time steps of `mode` (as kv_tdvp_sweep).  No
 * reference counterpart: the reference runs one chain per process
 * (src/kln-tdvp.cpp:73-78).  It replaces a loop of kv_tdvp_sweep
 * calls over the chains and leaves the same site tensors, bit for bit.  The
 * chains are spread over up to max_streams worker threads (<= 0: 8), each
 * with its own CUDA stream, staging ring and H_eff plan cache, so kernels of
 * different chains run concurrently on the GPU; chains go to workers longest
 * first by an estimate of their work, so the same set of chains is split the
 * same way on every call and finds its plans cached.  Returns when all chains
 * are done; device_ms (may be NULL) receives the device time from the first
 * launch to the last.  A failing chain does not stop the others: the first
 * failure's status is returned, kv_last_error names the chain, and that
 * chain's state is undefined.  Call from the thread that called kv_init;
 * the handles must not be used by another call meanwhile. */
int kv_sweep_batched(int n_chains, const kv_tdvp *chains, int mode, int steps, int max_streams, double *device_ms);

/* ------------------------------------------------------ instrumentation */
/* No reference counterpart (the reference only has its Timer table).
 * kv_profile(1) brackets every grouped-GEMM launch with CUDA events;
 * kv_profile_read returns (and resets) their summed device time, the
 * reference flops of the block pairs they multiplied and the launch count.
 * kv_counters returns the number of kernels launched since kv_init. */
int kv_profile(int enable);
int kv_profile_read(double *gemm_ms, double *gemm_ref_flops, long long *gemm_launches);
/* With profiling on: the Lanczos steps (one per iteration after the H_eff
 * apply) that ran since the last read, resolved at the end of each sweep:
 * their device ms, their algorithmic bytes (16 B per complex element moved:
 * 4 per element of v_{k-1}'s support, 4 per element of v_k's, 3 per element
 * of v_{k+1}'s, for the two overlaps, the two subtractions, the norm and the
 * normalisation) and their number; the counters are cleared.  No reference
 * counterpart. */
int kv_profile_read_lanczos(double *ms, double *bytes, long long *launches);
/* The same for the MPO mixings of the sweep (inside the H_eff applies and
 * the environment updates): algorithmic bytes = per output element 16 B
 * written plus 16 B read per contracted index of every active term. */
int kv_profile_read_mix(double *ms, double *bytes, long long *launches);
int kv_counters(long long *launches);
/* Charge sectors factorised by the block SVD on the calling thread's stream
 * since kv_init (or the last reset): their count, summed column counts, summed
 * ranks the mixed path's QR reduction kept (min(rows, columns) where none
 * ran), summed Jacobi sweeps and the largest sweep count of one sector.
 * reset != 0 clears the counters after reading them.  No reference
 * counterpart. */
int kv_svd_stats(int reset, long long *sectors, long long *columns, long long *rank, long long *sweeps,
                 int *max_sweeps);
/* local_krylov calls on the calling thread's stream since kv_init (or the
 * last reset), the Lanczos iterations issued for them, and the Krylov
 * dimensions they reached.  The host stops issuing iterations two behind the
 * device's stop test, so issued - used stays at most 2 per call.  reset != 0
 * clears the counters after reading them.  No reference counterpart. */
int kv_krylov_stats(int reset, long long *calls, long long *issued, long long *used);
/* Test hook for the failure path of the tensor-core GEMM; no reference
 * counterpart.  kv_debug_gemm_stall(1): until called with 0, every
 * tensor-core GEMM issues no operand copies and gives up each wait after a
 * short limit, so its first wait runs out with nothing in flight; the kernel
 * then frees its tensor memory and returns, and the call reports KV_ETIMEOUT.
 * Calls after kv_debug_gemm_stall(0) run normally. */
int kv_debug_gemm_stall(int on);
/* Test hook; no reference counterpart.  Bytes of the device's default memory
 * pool (where the library's stream-ordered allocations live) in use now and
 * at the high-water mark; reset_high != 0 first resets the mark to the
 * current use.  A call that allocates nothing leaves the mark unchanged. */
int kv_debug_pool_usage(int reset_high, long long *used_current, long long *used_high);

/* State::canonicalize (holstein/state.h:166-185): an L->R SVD sweep then an
 * R->L one with truncation tol_svd / max_dim (the reference's defaults are 0
 * and 1000), leaving the orthogonality centre on site 0.  out receives nsites
 * new handles; the inputs are not modified. */
int kv_canonicalize(int nsites, const kv_tensor *mps, double tol_svd, int max_dim, int precision, kv_tensor *out);

/* <a|W|b> (Operator::join, holstein/operator.h:178-198) over nsites. */
int kv_expectation(int nsites, const kv_tensor *bra, const kv_tensor *mpo, const kv_tensor *ket, double *re,
                   double *im);

/* <psi|O_k|psi> for nops operators that are the identity except on one site
 * each: Operator::join (holstein/operator.h:178-198) with the MPO that has
 * op_tensor[k] (a bond-dimension-1 MPO tensor, e.g. the site's exciton
 * density of Op/Density_j) on site op_site[k] and ident_mpo elsewhere (the
 * identity MPO's tensors, one per site).  The identity environments are built
 * once from each end, then each operator costs one environment update: all
 * site populations of a chain in about three passes.  The reference runs one
 * kln-join process per observable and step. */
int kv_local_expectations(int nsites, const kv_tensor *mps, const kv_tensor *ident_mpo, int nops, const int *op_site,
                          const kv_tensor *op_tensor, double *re, double *im);

/* The same value as kv_expectation without allocating any GPU memory; it has
 * no counterpart in the reference.  For callers that cannot let a library
 * call cudaMalloc: applications that own all device memory through their own
 * allocator or budget, and latency-critical loops that must not stall on an
 * allocation.  Every intermediate (environments, MPO-mixing buffers, GEMM
 * task lists) lives in one static 64 MiB device array that each GPU loading
 * this library reserves until the process exits; a call whose scratch would
 * exceed 64 MiB fails with KV_ENOMEM.  The scratch is set by the largest
 * site, not by the number of sites (after each site only the new environment
 * is kept): at most about 16*D^2*w*(2d+2) bytes for bond dimension D, MPO
 * bond dimension w and local dimension d (charge blocks make it smaller),
 * plus the task lists -- a D = 128, w = 7, d = 16 chain fits.  The first call
 * on a device looks up the array's address (cudaGetSymbolAddress, under a
 * lock, so first calls from several threads are safe) and must come before
 * any stream capture.  All calls share the array: calls that overlap on the
 * GPU race.  The inputs are device
 * tensors the caller already holds; re/im are host doubles.  kv_init must
 * have been called. */
int kv_expectation_noalloc(int nsites, const kv_tensor *bra, const kv_tensor *mpo, const kv_tensor *ket,
                           double *re, double *im);

#ifdef __cplusplus
}
#endif
#endif /* KVGPU_H */
