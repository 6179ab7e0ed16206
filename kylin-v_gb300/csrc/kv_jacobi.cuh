// Complex Jacobi rotations shared by the device SVD / eigensolver kernels and
// the host-side unit test (compiled with g++ as well as nvcc).
//
// For a Hermitian 2x2 [[a, c], [conj(c), b]] (a, b real) the unitary
//     J = [[cs, s], [-conj(s), cs]],  s = sn * c/|c|
// with t = sign(z)/(|z| + sqrt(1 + z^2)), z = (b - a) / (2|c|),
// cs = 1/sqrt(1 + t^2), sn = t*cs, makes J^H [[a,c],[c*,b]] J diagonal.
// Applied to two columns x, y:  x' = cs x - conj(s) y,  y' = s x + cs y.
// This is the textbook (Hestenes / Rutishauser) Jacobi step; one-sided SVD
// applies it to column pairs with a = |x|^2, b = |y|^2, c = x^H y.
#pragma once

#if defined(__CUDACC__)
#define KV_HD __host__ __device__ __forceinline__
#else
#define KV_HD inline
#include <cmath>
#endif

namespace kvj {

template <class T>
struct Rot {
    T cs;
    T s_re, s_im;  // s = sn * exp(i phi)
};

// Returns false (no rotation needed) when |c| <= tol * sqrt(a b) or |c| == 0.
template <class T>
KV_HD bool make_rotation(T a, T b, T c_re, T c_im, T tol, Rot<T> &r) {
    T ac = sqrt(c_re * c_re + c_im * c_im);
    if (!(ac > tol * sqrt(a * b)) || ac == T(0)) return false;
    T z = (b - a) / (T(2) * ac);
    T t = (z >= T(0) ? T(1) : T(-1)) / (fabs(z) + sqrt(T(1) + z * z));
    T cs = T(1) / sqrt(T(1) + t * t);
    T sn = t * cs;
    r.cs = cs;
    r.s_re = sn * c_re / ac;
    r.s_im = sn * c_im / ac;
    return true;
}

// (x, y) <- (cs x - conj(s) y, s x + cs y) for one complex element pair.
template <class T>
KV_HD void rotate_pair(const Rot<T> &r, T &xr, T &xi, T &yr, T &yi) {
    T nxr = r.cs * xr - (r.s_re * yr + r.s_im * yi);
    T nxi = r.cs * xi - (r.s_re * yi - r.s_im * yr);
    T nyr = (r.s_re * xr - r.s_im * xi) + r.cs * yr;
    T nyi = (r.s_re * xi + r.s_im * xr) + r.cs * yi;
    xr = nxr; xi = nxi; yr = nyr; yi = nyi;
}

// Cyclic two-sided Jacobi for an n x n complex Hermitian matrix stored
// row-major as (re, im) pairs in H (overwritten: diagonal -> eigenvalues) with
// eigenvectors accumulated into Z (columns).  Serial; for the tiny Lanczos
// tridiagonal (n <= 32).  Returns the number of sweeps used.
template <class T>
KV_HD int hermitian_jacobi(int n, T *H, T *Z, int max_sweeps) {
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            Z[2 * (i * n + j)] = (i == j) ? T(1) : T(0);
            Z[2 * (i * n + j) + 1] = T(0);
        }
    for (int i = 0; i < n; ++i) H[2 * (i * n + i) + 1] = T(0);
    int sweep = 0;
    for (; sweep < max_sweeps; ++sweep) {
        bool rotated = false;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                T a = H[2 * (p * n + p)], b = H[2 * (q * n + q)];
                T cr = H[2 * (p * n + q)], ci = H[2 * (p * n + q) + 1];
                Rot<T> r;
                // scale-aware threshold on the off-diagonal
                T scale = fabs(a) + fabs(b);
                T ac = sqrt(cr * cr + ci * ci);
                if (!(ac > T(1e-300)) || ac <= T(1e-17) * scale) continue;
                T z = (b - a) / (T(2) * ac);
                T t = (z >= T(0) ? T(1) : T(-1)) / (fabs(z) + sqrt(T(1) + z * z));
                r.cs = T(1) / sqrt(T(1) + t * t);
                T sn = t * r.cs;
                r.s_re = sn * cr / ac;
                r.s_im = sn * ci / ac;
                rotated = true;
                // columns p, q of H  (H <- H J)
                for (int k = 0; k < n; ++k)
                    rotate_pair(r, H[2 * (k * n + p)], H[2 * (k * n + p) + 1], H[2 * (k * n + q)],
                                H[2 * (k * n + q) + 1]);
                // rows p, q of H  (H <- J^H H): conjugate of the column rule
                for (int k = 0; k < n; ++k) {
                    T xr = H[2 * (p * n + k)], xi = -H[2 * (p * n + k) + 1];
                    T yr = H[2 * (q * n + k)], yi = -H[2 * (q * n + k) + 1];
                    rotate_pair(r, xr, xi, yr, yi);
                    H[2 * (p * n + k)] = xr; H[2 * (p * n + k) + 1] = -xi;
                    H[2 * (q * n + k)] = yr; H[2 * (q * n + k) + 1] = -yi;
                }
                H[2 * (p * n + q)] = H[2 * (p * n + q) + 1] = T(0);
                H[2 * (q * n + p)] = H[2 * (q * n + p) + 1] = T(0);
                H[2 * (p * n + p) + 1] = H[2 * (q * n + q) + 1] = T(0);
                for (int k = 0; k < n; ++k)
                    rotate_pair(r, Z[2 * (k * n + p)], Z[2 * (k * n + p) + 1], Z[2 * (k * n + q)],
                                Z[2 * (k * n + q) + 1]);
            }
        if (!rotated) break;
    }
    return sweep;
}

// Round-robin (tournament) pairing for parallel one-sided Jacobi: in round r
// (0 <= r < m-1) of an even count m, slot i (0 <= i < m/2) pairs columns
// (first, second).  Every unordered pair appears exactly once per m-1 rounds.
KV_HD void tournament_pair(int m, int r, int i, int &first, int &second) {
    // fixed element 0; the others rotate through positions 1..m-1
    auto pos = [&](int p) { return p == 0 ? 0 : 1 + ((p - 1 + r) % (m - 1)); };
    first = pos(i);
    second = pos(m - 1 - i);
    if (first > second) { int t = first; first = second; second = t; }
}

}  // namespace kvj
