// Block SVD plan structures shared by the host planner (kv_engine.cu) and the
// device kernels (kv_svd.cu).
#pragma once
#include "kv_internal.h"

namespace kv {

struct SvdSector {
    int64_t t_off;  // T (p x q, column-major) and its sorted U copy
    int64_t v_off;  // V (q x q, column-major) and its sorted copy
    int64_t s_off;  // q singular values
    int p, q;       // FP64 path: tall orientation, p >= q; mixed path: see op_svd
    int transposed; // 0: T = A (m = p, n = q); 1: T = A^H (m = q, n = p)
    int m, n;       // sector matrix of A (rows x cols)
};

struct SvdGather {  // one block of A into its sector matrix
    int64_t blk_off;
    int sector, row_off, col_off, nrows, ncols;
};

struct SvdScatter {  // one output block of U (side 0) or S.V^H / V^H (side 1)
    int64_t out_off;
    int sector, side, pos, len, kept, scale_s;
    int ld;  // side 0: the block's row length (>= kept; larger where SA-1TDVP adds columns)
};

// SA-1TDVP bond extension of one sector (holstein/svd.h:562-600): the kept
// vectors of the extended side as a dense row-major basis B (n x kept;
// side 0: U's columns, side 1: V^H's rows as vectors) and the new vectors X
// (n x ext, row-major)
struct SaSector {
    int64_t b_off, x_off;
    int sector, side, n, kept, ext;
};
// one output block's share of the new vectors: side 0 columns kept.. of a U
// block (rows pos.. of the sector), side 1 rows kept.. of a V^H block
struct SaOut {
    int64_t out_off, x_off;
    int side, pos, len, kept, ext;
};

struct SvdPlan {
    std::vector<SvdSector> secs;
    std::vector<SvdGather> gathers;
    int64_t t_elems = 0, v_elems = 0, s_elems = 0;
    int max_q = 0;
    DevBuf d_secs, d_gathers;
    void upload() { d_secs = upload_vec(secs); d_gathers = upload_vec(gathers); }
};

// FP64 polish of the kept factor of one sector (mixed mode): W (the FP32
// singular vectors of the other side, divided by their singular values) at
// w_off, the factor X (rows x k, row-major with row stride ldx >= k) at
// x_off, its Gram / Cholesky factor (k x k) at g_off
struct SvdPolish {
    int64_t x_off, g_off, w_off;
    int sector, rows, k, ldx;
};
// one output block copied from a dense row-major factor M (ld columns);
// ctrans: the block is taken from M^H
struct SvdDense {
    int64_t out_off, m_off;
    int side, pos, len, kept, ld, ctrans;
};

void svd_gather(const SvdPlan &p, const double2 *A, double2 *T);
// largest number of columns the mixed-mode Jacobi handles in one sector
constexpr int kJacobiMaxQ = 2048;
// mixed mode: FP32 one-sided Jacobi of T without accumulated rotations
// (T oriented so the wanted singular vectors are its columns), sorted
// normalised columns and singular values, and the first k columns in FP64
void svd_jacobi_f32(const SvdPlan &p, const double2 *T64, float2 *T, int *status, int max_sweeps, float tol);
// (T64 == nullptr: T already holds the FP32 matrix)
// mixed mode, sectors beyond shared memory: the QR reduction to numerical rank
// (rows below qr_floor ||T||_F dropped) on an L2-resident workspace; T32 =
// the rank-r factor, column-major, zero beyond column r; ranks[sector] = r
void svd_qr_global(const SvdPlan &p, const double2 *T64, float2 *T32, int *ranks, float qr_floor);
void svd_finalize_f32(const SvdPlan &p, const float2 *T, float2 *Us, double *S);
// mixed mode, every sector in shared memory: pivoted Householder on T's rows
// truncated where the remaining rows fall below qr_floor ||T||_F, one-sided
// Jacobi on the rank-r factor, sorted normalised columns and singular values
// (zero beyond r; ranks[sector] = r).  Returns false, launching nothing, when
// a sector does not fit shared memory.
bool svd_qrjacobi_f32(const SvdPlan &p, const double2 *T64, float2 *Us, double *S, int *status, int *ranks,
                      int max_sweeps, float tol, float qr_floor);
void svd_extract(const DevBuf &pol, int npol, const SvdPlan &p, const float2 *Us, const double *S, double2 *W);
// rows of X per triangular-solve CTA (one warp per row)
constexpr int kTrsmRows = 8;
// squared column norms of each polish factor X into G[g_off + j].x
void svd_col_norm2(const DevBuf &pol, int npol, const double2 *X, double2 *G);
void svd_chol(const DevBuf &pol, int npol, double2 *G, int *status, double *diagv, double shift);
void svd_trsm(const DevBuf &pol, const std::vector<int> &item_pol, const std::vector<int> &item_row0,
              const double2 *G, double2 *X, int kmax);
void svd_scatter_dense(const std::vector<SvdDense> &d, const double2 *M, double2 *out);
void svd_jacobi(const SvdPlan &p, double2 *T, double2 *V, int *status, int max_sweeps, double tol);
void svd_finalize(const SvdPlan &p, const double2 *T, const double2 *V, double2 *Us, double2 *Vs, double *S);
void svd_scatter(const std::vector<SvdScatter> &sc, const SvdPlan &p, const double2 *Us, const double2 *Vs,
                 const double *S, double2 *out);
// FP64 path: the kept vectors of each SA sector into B (after svd_finalize)
void sa_basis(const std::vector<SaSector> &v, const SvdPlan &p, const double2 *Us, const double2 *Vs, double2 *B);
// x -= y over n elements
void sa_subtract(double2 *x, const double2 *y, int64_t n);
void sa_scatter(const std::vector<SaOut> &v, const double2 *X, double2 *out);

}  // namespace kv
