// tile_small.cuh — row-vector forms of the tile operations, for the block
// triangular solves of the batched path: the right-hand sides are kept as
// m × N row blocks (m = number of right-hand sides, m <= kSmallM), so the
// forward solve L y = b is y_iᵀ = (b_iᵀ − Σ_j y_jᵀ L_ijᵀ) L_ii⁻ᵀ and the
// backward solve Lᵀ x = y is x_iᵀ = (y_iᵀ − Σ_j x_jᵀ L_ji) L_ii⁻¹: GEMM_NT,
// TRSM_RLTN, GEMM_NN and TRSM_RLNN tasks with m rows.
//
// The 128×128-block kernels of tile_f64.cuh would spend a whole block row on
// each of these few rows; here every thread owns output columns and the
// block's threads share the k loop, so the work is the m·n·k the operation
// needs.  T is double (FP64 tasks) or float (FP32 tasks of the mixed path).
#pragma once
#include <cuda_runtime.h>

#include "tile_f64.cuh"

namespace ttg {

constexpr int kSmallM = 16;
constexpr int kSmallKC = 16;              // (layout of the TRSM's shared memory below)
constexpr int kSmallKA = 128;             // k rows of A staged per pass of gemm_small_cols
constexpr int kSmallU = 16;               // loads of B in flight per thread
constexpr int kSmallBPad = kThreads + 1;  // staged B row (conflict-free stores)
// Shared memory (elements of T) used by the small-m kernels: the staged A of
// gemm_small_cols, then the TRSM's panel of L and its inverse diagonal.
constexpr int kSmallSmem = kSmallKC * kSmallBPad + kSmallKC * kSmallM + kPanel * (kPanel + 1) + kPanel;
static_assert(kSmallKA * kSmallM <= kSmallKC * kSmallBPad + kSmallKC * kSmallM, "staged A below the TRSM panel");

// C[m×n] (columns [j0, j1)) <- alpha·A·op(B) + beta·C, m <= kSmallM; A is m×k
// (lda).  op(B)(kk, j) = B[j + kk·ldb] (NT) or B[kk + j·ldb] (NN).  Thread t
// owns columns j0 + t, j0 + t + kThreads, ... and reads its column of op(B)
// straight from L2, kSmallU values at a time (all loads issued before the
// FMAs, so a thread keeps kSmallU loads in flight; NT reads are coalesced
// across the warp, NN reads walk down a column); A is staged kSmallKA rows
// of k at a time through shared memory.  The product is HBM/L2-latency
// bound (m·n·k FMAs on n·k elements of B): the work is the m·n·k the
// operation needs and the reads are as many as there are elements of B.
// MQ: kSmallM, or 1 when m == 1 (one right-hand side: no predicated rows).
template <class T, bool B_NN, int MQ>
__device__ void gemm_small_cols_q(int m, int j0, int j1, int k, T alpha, const T* A, int lda, const T* B, int ldb, T beta, T* C,
                                  int ldc, T* smem) {
    T* sA = smem;  // [kSmallKA][MQ]: sA[kk·MQ + q] = A(q, k0 + kk)
    for (int c0 = j0; c0 < j1; c0 += kThreads) {
        const int j = c0 + threadIdx.x;
        const bool act = j < j1;
        T acc[MQ];
#pragma unroll
        for (int q = 0; q < MQ; ++q) acc[q] = T(0);
        for (int k0 = 0; k0 < k; k0 += kSmallKA) {
            const int kc = min(kSmallKA, k - k0);
            __syncthreads();
            for (int e = threadIdx.x; e < kSmallKA * MQ; e += kThreads) {
                const int q = e % MQ, kk = e / MQ;
                sA[e] = (q < m && kk < kc) ? ldcg(A + q + (size_t)(k0 + kk) * lda) : T(0);
            }
            __syncthreads();
            if (act) {
                for (int u0 = 0; u0 < kc; u0 += kSmallU) {
                    T b[kSmallU];
#pragma unroll
                    for (int u = 0; u < kSmallU; ++u) {
                        const int kk = k0 + u0 + u;
                        b[u] = u0 + u < kc ? ldcg(B_NN ? B + kk + (size_t)j * ldb : B + j + (size_t)kk * ldb) : T(0);
                    }
#pragma unroll
                    for (int u = 0; u < kSmallU; ++u) {
                        const T* a = sA + (u0 + u) * MQ;
#pragma unroll
                        for (int q = 0; q < MQ; ++q)
                            if (q < m) acc[q] = fma(a[q], b[u], acc[q]);
                    }
                }
            }
        }
        if (act) {
#pragma unroll
            for (int q = 0; q < MQ; ++q) {
                if (q >= m) break;
                T* p = C + q + (size_t)j * ldc;
                T v = alpha * acc[q];
                if (beta != T(0)) v = fma(beta, ldcg(p), v);
                *p = v;
            }
        }
    }
    __syncthreads();
}

// The NN form with B read down its columns: warp w takes columns j0 + w,
// j0 + w + 8, ..., its lanes split k (kSmallUN loads of 32 consecutive
// elements in flight per lane, coalesced), and the warp's partial sums are
// added by shuffles.  A (m×k) is staged whole when it fits, else read from
// L2.
template <class T, int MQ>
__device__ void gemm_small_cols_nn_warp(int m, int j0, int j1, int k, T alpha, const T* A, int lda, const T* B, int ldb, T beta,
                                        T* C, int ldc, T* smem) {
    constexpr int kSmallUN = 4;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T* sA = smem;  // [k][MQ] when staged
    const bool staged = k * MQ <= kSmallKA * kSmallM;
    if (staged) {
        for (int e = threadIdx.x; e < k * MQ; e += kThreads) {
            const int q = e % MQ, kk = e / MQ;
            sA[e] = q < m ? ldcg(A + q + (size_t)kk * lda) : T(0);
        }
        __syncthreads();
    }
    for (int j = j0 + warp; j < j1; j += kThreads / 32) {
        T acc[MQ];
#pragma unroll
        for (int q = 0; q < MQ; ++q) acc[q] = T(0);
        const T* bj = B + (size_t)j * ldb;
        for (int k0 = 0; k0 < k; k0 += 32 * kSmallUN) {
            T b[kSmallUN];
#pragma unroll
            for (int u = 0; u < kSmallUN; ++u) {
                const int kk = k0 + 32 * u + lane;
                b[u] = kk < k ? ldcg(bj + kk) : T(0);
            }
#pragma unroll
            for (int u = 0; u < kSmallUN; ++u) {
                const int kk = k0 + 32 * u + lane;
                if (kk < k) {
#pragma unroll
                    for (int q = 0; q < MQ; ++q)
                        if (q < m) acc[q] = fma(staged ? sA[kk * MQ + q] : ldcg(A + q + (size_t)kk * lda), b[u], acc[q]);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < MQ; ++q) {
            if (q >= m) break;
            T v = acc[q];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) {
                T* p = C + q + (size_t)j * ldc;
                T r = alpha * v;
                if (beta != T(0)) r = fma(beta, ldcg(p), r);
                *p = r;
            }
        }
    }
    __syncthreads();
}

// The NN form with one right-hand side (m = 1), k <= kSmallKA·kSmallM: the
// row of A staged whole; a warp takes kSmallCW columns at a time, its lanes
// split k (kSmallUN loads of 32 consecutive elements per column in flight
// per lane), shuffle reductions.  (Splitting k over thread groups for the NT
// form, with a shared-memory reduction, measured 2.7× slower per task than
// one thread per column.)
constexpr int kSmallCW = 4;
template <class T>
__device__ void gemm_small_nn_m1(int j0, int j1, int k, T alpha, const T* A, int lda, const T* B, int ldb, T beta, T* C, int ldc,
                                 T* smem) {
    constexpr int kSmallUN = 4;
    T* sA = smem;  // [k]
    for (int e = threadIdx.x; e < k; e += kThreads) sA[e] = ldcg(A + (size_t)e * lda);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int jb = j0 + kSmallCW * warp; jb < j1; jb += kSmallCW * (kThreads / 32)) {
        T acc[kSmallCW];
#pragma unroll
        for (int c = 0; c < kSmallCW; ++c) acc[c] = T(0);
        for (int k0 = 0; k0 < k; k0 += 32 * kSmallUN) {
            T b[kSmallCW][kSmallUN];
#pragma unroll
            for (int c = 0; c < kSmallCW; ++c)
#pragma unroll
                for (int u = 0; u < kSmallUN; ++u) {
                    const int kk = k0 + 32 * u + lane;
                    b[c][u] = (jb + c < j1 && kk < k) ? ldcg(B + kk + (size_t)(jb + c) * ldb) : T(0);
                }
#pragma unroll
            for (int c = 0; c < kSmallCW; ++c)
#pragma unroll
                for (int u = 0; u < kSmallUN; ++u) {
                    const int kk = k0 + 32 * u + lane;
                    if (kk < k) acc[c] = fma(sA[kk], b[c][u], acc[c]);
                }
        }
#pragma unroll
        for (int c = 0; c < kSmallCW; ++c) {
            T v = acc[c];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0 && jb + c < j1) {
                T* p = C + (size_t)(jb + c) * ldc;
                T r = alpha * v;
                if (beta != T(0)) r = fma(beta, ldcg(p), r);
                *p = r;
            }
        }
    }
    __syncthreads();
}

template <class T, bool B_NN>
__device__ inline void gemm_small_cols(int m, int j0, int j1, int k, T alpha, const T* A, int lda, const T* B, int ldb, T beta, T* C,
                                       int ldc, T* smem) {
    if (B_NN && m == 1 && k <= kSmallKA * kSmallM) {
        gemm_small_nn_m1<T>(j0, j1, k, alpha, A, lda, B, ldb, beta, C, ldc, smem);
        return;
    }
    if (B_NN) {
        if (m == 1) gemm_small_cols_nn_warp<T, 1>(m, j0, j1, k, alpha, A, lda, B, ldb, beta, C, ldc, smem);
        else gemm_small_cols_nn_warp<T, kSmallM>(m, j0, j1, k, alpha, A, lda, B, ldb, beta, C, ldc, smem);
        return;
    }
    if (m == 1) gemm_small_cols_q<T, false, 1>(m, j0, j1, k, alpha, A, lda, B, ldb, beta, C, ldc, smem);
    else gemm_small_cols_q<T, false, kSmallM>(m, j0, j1, k, alpha, A, lda, B, ldb, beta, C, ldc, smem);
}

// The part `part` of `parts` of a small-m GEMM: a contiguous range of columns.
template <class T, bool B_NN>
__device__ inline void gemm_small_m(int m, int n, int k, T alpha, const T* A, int lda, const T* B, int ldb, T beta, T* C, int ldc,
                                    T* smem, int part, int parts) {
    const int per = (n + parts - 1) / parts;
    const int j0 = min(n, part * per), j1 = min(n, j0 + per);
    gemm_small_cols<T, B_NN>(m, j0, j1, k, alpha, A, lda, B, ldb, beta, C, ldc, smem);
}

// B[m×n] <- alpha·B·L⁻ᵀ (TRANS, cblas_dtrsm R,L,T,N) or alpha·B·L⁻¹ (cblas_dtrsm
// R,L,N,N), L n×n lower non-unit, m <= kSmallM: forward (TRANS) or backward
// substitution over 32-column panels.  Panel solve: warp w takes rows
// w, w+8, ...; lane j is column j of the panel, and each solved column is
// passed to the lanes that still need it by a shuffle.  The rest of the row
// is then updated by a small-m GEMM with the solved panel.
template <class T, bool TRANS>
__device__ void trsm_small_m(int m, int n, T alpha, const T* L, int ldl, T* B, int ldb, T* smem) {
    T* Ls = smem + kSmallKC * kSmallBPad + kSmallKC * kSmallM;  // [kPanel][kPanel+1]: Ls[c][l] = L(p+c, p+l)
    T* invd = Ls + kPanel * (kPanel + 1);                      // 1 / L(p+c, p+c)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (alpha != T(1)) {
        for (int e = threadIdx.x; e < m * n; e += kThreads) {
            const int q = e % m, j = e / m;
            B[q + (size_t)j * ldb] = alpha * ldcg(B + q + (size_t)j * ldb);
        }
    }
    const int npan = (n + kPanel - 1) / kPanel;
    for (int pi = 0; pi < npan; ++pi) {
        const int p = (TRANS ? pi : npan - 1 - pi) * kPanel;
        const int nb = min(kPanel, n - p);
        __syncthreads();
        load_panel_block<T>(L + p + (size_t)p * ldl, ldl, nb, Ls);
        if (threadIdx.x < kPanel)
            invd[threadIdx.x] = (int)threadIdx.x < nb ? T(1) / ldcg(L + (size_t)(p + threadIdx.x) * (ldl + 1)) : T(0);
        __syncthreads();
        for (int q = warp; q < m; q += kThreads / 32) {
            T t = lane < nb ? ldcg(B + q + (size_t)(p + lane) * ldb) : T(0);
            if (TRANS) {
                for (int c = 0; c < nb; ++c) {
                    const T x = __shfl_sync(0xffffffffu, t, c) * invd[c];
                    if (lane == c) t = x;
                    else if (lane > c) t = fma(-Ls[lane * (kPanel + 1) + c], x, t);
                }
            } else {
                for (int c = nb - 1; c >= 0; --c) {
                    const T x = __shfl_sync(0xffffffffu, t, c) * invd[c];
                    if (lane == c) t = x;
                    else if (lane < c) t = fma(-Ls[c * (kPanel + 1) + lane], x, t);
                }
            }
            if (lane < nb) B[q + (size_t)(p + lane) * ldb] = t;
        }
        __syncthreads();
        if (TRANS) {
            // Columns right of the panel: B[:, p+nb:] -= X · L[p+nb:, p:p+nb]ᵀ.
            if (p + nb < n)
                gemm_small_cols<T, false>(m, 0, n - p - nb, nb, T(-1), B + (size_t)p * ldb, ldb, L + (p + nb) + (size_t)p * ldl,
                                          ldl, T(1), B + (size_t)(p + nb) * ldb, ldb, smem);
        } else {
            // Columns left of the panel: B[:, :p] -= X · L[p:p+nb, :p].
            if (p > 0) gemm_small_cols<T, true>(m, 0, p, nb, T(-1), B + (size_t)p * ldb, ldb, L + p, ldl, T(1), B, ldb, smem);
        }
    }
    __syncthreads();
}

// Rows [r0, r1) of part `part` of a TRSM, as successive groups of kSmallM
// rows (the row-vector kernel above; used for m <= kSmallM, and for
// TRSM_RLNN of any size).
template <class T, bool TRANS>
__device__ inline void trsm_rows_small(int m, int n, T alpha, const T* L, int ldl, T* B, int ldb, T* smem, int part, int parts) {
    const int per = (m + parts - 1) / parts;
    const int r0 = min(m, part * per), r1 = min(m, r0 + per);
    for (int q0 = r0; q0 < r1; q0 += kSmallM) trsm_small_m<T, TRANS>(min(kSmallM, r1 - q0), n, alpha, L, ldl, B + q0, ldb, smem);
}

// C[m×n] <- alpha·A + beta·C with A and C of either precision (TTG_OP_CONVERT:
// flags bit 0: A is float, bit 1: C is float); parts split the elements,
// each thread keeps kConvU elements' reads in flight.
constexpr int kConvU = 8;
__device__ inline void convert_tile(int m, int n, double alpha, const void* A, int lda, double beta, void* C, int ldc, int flags,
                                    int part, int parts) {
    const bool af = flags & 1, cf = flags & 2;
    const long total = (long)m * n, stride = (long)kThreads * parts;
    for (long e0 = threadIdx.x + (long)part * kThreads; e0 < total; e0 += stride * kConvU) {
        double a[kConvU], c[kConvU];
#pragma unroll
        for (int u = 0; u < kConvU; ++u) {
            const long e = e0 + u * stride;
            a[u] = c[u] = 0.0;
            if (e < total) {
                const int i = (int)(e % m), j = (int)(e / m);
                const size_t ia = i + (size_t)j * lda, ic = i + (size_t)j * ldc;
                a[u] = af ? (double)__ldcg((const float*)A + ia) : __ldcg((const double*)A + ia);
                if (beta != 0.0) c[u] = cf ? (double)__ldcg((const float*)C + ic) : __ldcg((const double*)C + ic);
            }
        }
#pragma unroll
        for (int u = 0; u < kConvU; ++u) {
            const long e = e0 + u * stride;
            if (e < total) {
                const int i = (int)(e % m), j = (int)(e / m);
                const size_t ic = i + (size_t)j * ldc;
                double v = alpha * a[u];
                if (beta != 0.0) v = fma(beta, c[u], v);
                if (cf) ((float*)C)[ic] = (float)v;
                else ((double*)C)[ic] = v;
            }
        }
    }
    __syncthreads();
}

}  // namespace ttg
