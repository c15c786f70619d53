// ttor::gpu — tile operations recorded by task bodies.
//
// In the reference, task bodies call CBLAS/LAPACKE on host tiles
// (miniapp/dense_cholesky/2d_cholesky.cpp:319,404-405,490-494;
// miniapp/gemm/2d_gemm.cpp:157).  Here the same calls, with the same argument
// order and meaning, take DEVICE pointers and are recorded into the running
// task during the thread pool's capture; the persistent executor computes
// them on the GPU when join() runs the graph.  Only the argument combinations
// of those call sites are supported; anything else throws
// std::invalid_argument at capture time.
#ifndef TTOR_GB300_GPU_BLAS_HPP
#define TTOR_GB300_GPU_BLAS_HPP

#include <stdexcept>

#include "../../../include/ttg.h"
#include "threadpool_shared.hpp"

namespace ttor {
namespace gpu {

enum CBLAS_LAYOUT { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 };
enum CBLAS_DIAG { CblasNonUnit = 131, CblasUnit = 132 };
enum CBLAS_SIDE { CblasLeft = 141, CblasRight = 142 };
enum { LAPACK_ROW_MAJOR = 101, LAPACK_COL_MAJOR = 102 };

inline void record(const ttg_op& op) {
    detail::Capture* c = detail::current_capture();
    if (!c) throw std::logic_error("ttor::gpu: tile operation called outside a task body");
    c->record_op(op);
}

inline ttg_op make_op(int kind) {
    ttg_op op{};
    op.kind = kind;
    op.prec = TTG_PREC_F64;
    op.alpha = 1.0;
    op.beta = 0.0;
    return op;
}

// spin_for_seconds(t): the task keeps its block busy for t seconds — the body
// of the reference's scheduler micro-benchmarks (mini_benchmarks/common.hpp:21-28
// spins a host thread).  0 <= t <= 1.
inline void spin_for_seconds(double seconds) {
    if (!(seconds >= 0.0 && seconds <= 1.0)) throw std::invalid_argument("ttor::gpu::spin_for_seconds: 0 <= seconds <= 1");
    ttg_op op = make_op(TTG_OP_SPIN);
    op.alpha = seconds;
    record(op);
}

// LAPACKE_dpotrf(LAPACK_COL_MAJOR, 'L', n, A, lda): in-place lower Cholesky.
// Returns 0; a failing pivot is reported by the executor (TTG_ENOTPD with the
// column in ttg_report::info) after join().
inline int LAPACKE_dpotrf(int layout, char uplo, int n, double* A, int lda) {
    if (layout != LAPACK_COL_MAJOR || (uplo != 'L' && uplo != 'l'))
        throw std::invalid_argument("ttor::gpu::LAPACKE_dpotrf: only column-major 'L'");
    ttg_op op = make_op(TTG_OP_POTRF_L);
    op.n = n;
    op.m = n;
    op.c = A;
    op.ldc = lda;
    record(op);
    return 0;
}

// cblas_dtrsm(ColMajor, Right, Lower, Trans, NonUnit, m, n, alpha, L, ldl, B, ldb).
inline void cblas_dtrsm(int layout, int side, int uplo, int trans, int diag, int m, int n, double alpha, const double* L,
                        int ldl, double* B, int ldb) {
    if (layout != CblasColMajor || side != CblasRight || uplo != CblasLower || trans != CblasTrans || diag != CblasNonUnit)
        throw std::invalid_argument("ttor::gpu::cblas_dtrsm: only ColMajor, Right, Lower, Trans, NonUnit");
    ttg_op op = make_op(TTG_OP_TRSM_RLTN);
    op.m = m;
    op.n = n;
    op.alpha = alpha;
    op.a = L;
    op.lda = ldl;
    op.c = B;
    op.ldc = ldb;
    record(op);
}

// cblas_dsyrk(ColMajor, Lower, NoTrans, n, k, alpha, A, lda, beta, C, ldc).
inline void cblas_dsyrk(int layout, int uplo, int trans, int n, int k, double alpha, const double* A, int lda, double beta,
                        double* C, int ldc) {
    if (layout != CblasColMajor || uplo != CblasLower || trans != CblasNoTrans)
        throw std::invalid_argument("ttor::gpu::cblas_dsyrk: only ColMajor, Lower, NoTrans");
    ttg_op op = make_op(TTG_OP_SYRK_LN);
    op.m = n;
    op.n = n;
    op.k = k;
    op.alpha = alpha;
    op.beta = beta;
    op.a = A;
    op.lda = lda;
    op.c = C;
    op.ldc = ldc;
    record(op);
}

// cblas_dgemm(ColMajor, NoTrans, {Trans | NoTrans}, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc).
inline void cblas_dgemm(int layout, int transa, int transb, int m, int n, int k, double alpha, const double* A, int lda,
                        const double* B, int ldb, double beta, double* C, int ldc) {
    if (layout != CblasColMajor || transa != CblasNoTrans || (transb != CblasTrans && transb != CblasNoTrans))
        throw std::invalid_argument("ttor::gpu::cblas_dgemm: only ColMajor, NoTrans, {Trans, NoTrans}");
    ttg_op op = make_op(transb == CblasTrans ? TTG_OP_GEMM_NT : TTG_OP_GEMM_NN);
    op.m = m;
    op.n = n;
    op.k = k;
    op.alpha = alpha;
    op.beta = beta;
    op.a = A;
    op.lda = lda;
    op.b = B;
    op.ldb = ldb;
    op.c = C;
    op.ldc = ldc;
    record(op);
}

// C <- alpha·A + beta·C on an m×n tile (the Eigen `*blocks[ij] += *Atmp` of
// the accumulate flow, 2d_cholesky.cpp:570).
inline void geadd(int m, int n, double alpha, const double* A, int lda, double beta, double* C, int ldc) {
    ttg_op op = make_op(TTG_OP_GEADD);
    op.m = m;
    op.n = n;
    op.alpha = alpha;
    op.beta = beta;
    op.a = A;
    op.lda = lda;
    op.c = C;
    op.ldc = ldc;
    record(op);
}

// Record a fully specified operation (used by the mixed-precision path).
inline void record_op(const ttg_op& op) { record(op); }

}  // namespace gpu
}  // namespace ttor

#endif
