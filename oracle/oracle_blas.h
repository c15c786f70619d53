/*
 * oracle_blas.h — TEST INFRASTRUCTURE ONLY (the oracle's tile math).
 *
 * The reference's task bodies call CBLAS/LAPACKE (cblas_dgemm, cblas_dsyrk,
 * cblas_dtrsm, LAPACKE_dpotrf; miniapp/dense_cholesky/2d_cholesky.cpp:319,
 * 404-405, 490-494 and miniapp/gemm/2d_gemm.cpp:157).  The BLAS the reference
 * links is a site install (MKL or OpenBLAS, unpinned).  Here the same calls go
 * to the OpenBLAS that ships inside the scipy wheel when its path is given in
 * TTG_ORACLE_BLAS (resolved with dlopen, since there are no cblas headers),
 * else to the plain loops below (column-major, same argument meaning).
 *
 * Only the tests, the smoke check and bench.py's CPU baseline may use this.
 */
#ifndef TTG_ORACLE_BLAS_H
#define TTG_ORACLE_BLAS_H

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <dlfcn.h>
#include <string>

namespace orc {

enum { ColMajor = 102, NoTrans = 111, Trans = 112, Upper = 121, Lower = 122, NonUnit = 131, Unit = 132, Left = 141, Right = 142 };

typedef void (*dgemm_t)(int, int, int, int, int, int, double, const double*, int, const double*, int, double, double*, int);
typedef void (*dsyrk_t)(int, int, int, int, int, double, const double*, int, double, double*, int);
typedef void (*dtrsm_t)(int, int, int, int, int, int, int, double, const double*, int, double*, int);
typedef int (*dpotrf_t)(int, char, int, double*, int);
typedef void (*setthreads_t)(int);

struct Blas {
    dgemm_t gemm = nullptr;
    dsyrk_t syrk = nullptr;
    dtrsm_t trsm = nullptr;
    dpotrf_t potrf = nullptr;
    std::string name = "loops";
};

inline void* find_sym(void* h, const char* const* names) {
    for (int i = 0; names[i]; ++i) {
        void* p = dlsym(h, names[i]);
        if (p) return p;
    }
    return nullptr;
}

/* Resolve the BLAS once.  32-bit-integer OpenBLAS builds only. */
inline Blas& blas() {
    static Blas b = [] {
        Blas r;
        const char* path = getenv("TTG_ORACLE_BLAS");
        if (!path || !*path) return r;
        void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
        if (!h) return r;
        static const char* g[] = {"scipy_cblas_dgemm", "cblas_dgemm", nullptr};
        static const char* s[] = {"scipy_cblas_dsyrk", "cblas_dsyrk", nullptr};
        static const char* t[] = {"scipy_cblas_dtrsm", "cblas_dtrsm", nullptr};
        static const char* p[] = {"scipy_LAPACKE_dpotrf", "LAPACKE_dpotrf", nullptr};
        static const char* n[] = {"scipy_openblas_set_num_threads", "openblas_set_num_threads", nullptr};
        r.gemm = (dgemm_t)find_sym(h, g);
        r.syrk = (dsyrk_t)find_sym(h, s);
        r.trsm = (dtrsm_t)find_sym(h, t);
        r.potrf = (dpotrf_t)find_sym(h, p);
        setthreads_t st = (setthreads_t)find_sym(h, n);
        if (!r.gemm || !r.syrk || !r.trsm || !r.potrf) return Blas();
        if (st) st(1); /* one BLAS thread per task, as the reference runs it */
        r.name = std::string("openblas:") + path;
        return r;
    }();
    return b;
}

/* C[m×n] = alpha·op(A)·op(B) + beta·C, column-major. */
inline void dgemm(int ta, int tb, int m, int n, int k, double alpha, const double* A, int lda, const double* B, int ldb,
                  double beta, double* C, int ldc) {
    Blas& b = blas();
    if (b.gemm) { b.gemm(ColMajor, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc); return; }
    for (int j = 0; j < n; ++j) {
        for (int i = 0; i < m; ++i) C[i + (size_t)j * ldc] = (beta == 0.0) ? 0.0 : beta * C[i + (size_t)j * ldc];
        for (int l = 0; l < k; ++l) {
            double bv = (tb == NoTrans) ? B[l + (size_t)j * ldb] : B[j + (size_t)l * ldb];
            bv *= alpha;
            if (ta == NoTrans) {
                const double* a = A + (size_t)l * lda;
                double* c = C + (size_t)j * ldc;
                for (int i = 0; i < m; ++i) c[i] += a[i] * bv;
            } else {
                double* c = C + (size_t)j * ldc;
                for (int i = 0; i < m; ++i) c[i] += A[l + (size_t)i * lda] * bv;
            }
        }
    }
}

/* Lower triangle of C[n×n] = alpha·A·Aᵀ + beta·C, A is n×k (NoTrans). */
inline void dsyrk_ln(int n, int k, double alpha, const double* A, int lda, double beta, double* C, int ldc) {
    Blas& b = blas();
    if (b.syrk) { b.syrk(ColMajor, Lower, NoTrans, n, k, alpha, A, lda, beta, C, ldc); return; }
    for (int j = 0; j < n; ++j) {
        for (int i = j; i < n; ++i) C[i + (size_t)j * ldc] = (beta == 0.0) ? 0.0 : beta * C[i + (size_t)j * ldc];
        for (int l = 0; l < k; ++l) {
            double bv = alpha * A[j + (size_t)l * lda];
            const double* a = A + (size_t)l * lda;
            double* c = C + (size_t)j * ldc;
            for (int i = j; i < n; ++i) c[i] += a[i] * bv;
        }
    }
}

/* B[m×n] ← alpha·B·L⁻ᵀ with L n×n lower, non-unit (Right, Lower, Trans). */
inline void dtrsm_rltn(int m, int n, double alpha, const double* L, int ldl, double* B, int ldb) {
    Blas& b = blas();
    if (b.trsm) { b.trsm(ColMajor, Right, Lower, Trans, NonUnit, m, n, alpha, L, ldl, B, ldb); return; }
    /* X Lᵀ = alpha B: column c of X depends on columns < c. */
    for (int c = 0; c < n; ++c) {
        double* x = B + (size_t)c * ldb;
        if (alpha != 1.0)
            for (int i = 0; i < m; ++i) x[i] *= alpha;
        for (int l = 0; l < c; ++l) {
            double f = L[c + (size_t)l * ldl];
            const double* xl = B + (size_t)l * ldb;
            for (int i = 0; i < m; ++i) x[i] -= xl[i] * f;
        }
        double d = L[c + (size_t)c * ldl];
        for (int i = 0; i < m; ++i) x[i] /= d;
    }
}

/* In-place lower Cholesky of A[n×n]; returns 0 or the 1-based failing column. */
inline int dpotrf_l(int n, double* A, int lda) {
    Blas& b = blas();
    if (b.potrf) return b.potrf(ColMajor, 'L', n, A, lda);
    for (int j = 0; j < n; ++j) {
        double d = A[j + (size_t)j * lda];
        for (int l = 0; l < j; ++l) d -= A[j + (size_t)l * lda] * A[j + (size_t)l * lda];
        if (!(d > 0.0)) return j + 1;
        d = std::sqrt(d);
        A[j + (size_t)j * lda] = d;
        for (int i = j + 1; i < n; ++i) {
            double s = A[i + (size_t)j * lda];
            for (int l = 0; l < j; ++l) s -= A[i + (size_t)l * lda] * A[j + (size_t)l * lda];
            A[i + (size_t)j * lda] = s / d;
        }
    }
    return 0;
}

}  // namespace orc

#endif
