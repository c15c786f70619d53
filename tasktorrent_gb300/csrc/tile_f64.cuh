// tile_f64.cuh — FP64 tile kernels run by one block of the persistent executor.
//
// Each function is executed by all kThreads threads of a block on one tile task
// and replaces one BLAS/LAPACK call of the reference's task bodies:
//   potrf_l_f64   LAPACKE_dpotrf(COL_MAJOR,'L')      2d_cholesky.cpp:319
//   trsm_rltn_f64 cblas_dtrsm(Right,Lower,Trans,NonUnit) 2d_cholesky.cpp:404-405
//   gemm_f64<..., LOWER=true>  cblas_dsyrk(Lower,NoTrans) 2d_cholesky.cpp:490-491
//   gemm_f64<NT>  cblas_dgemm(NoTrans,Trans)         2d_cholesky.cpp:493-494
//   gemm_f64<NN>  cblas_dgemm(NoTrans,NoTrans)       2d_gemm.cpp:157
//
// The FP64 rate of a GB300 SM is a few DFMA per clock, so these kernels are
// built to keep the DFMA pipe busy (8×8 register blocking, 64 independent
// accumulators per thread) rather than to save bandwidth.  Tiles written by
// other blocks are read through L2 only (ld.global.cg): a persistent block can
// hold stale L1 lines of a tile another block has since updated.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ttg {

constexpr int kThreads = 256;
constexpr int kBM = 128, kBN = 128, kBK = 16;
constexpr int kBNP = kBN + 1;  // padded row of the B stage (conflict-free transposed store)
constexpr int kPanel = 32;     // POTRF / TRSM panel width
// Shared memory used by the FP64 kernels (doubles).
constexpr int kF64SmemDoubles = kBK * kBM + kBK * kBNP + kPanel * (kPanel + 1);

__device__ __forceinline__ double ldcg(const double* p) { return __ldcg(p); }
__device__ __forceinline__ float ldcg(const float* p) { return __ldcg(p); }

// C[m×n] = alpha·A·op(B) + beta·C on the block.  A is m×k (lda).  op(B)(kk,j)
// is B[j + kk·ldb] (B_NN = false: B is n×k, "NT") or B[kk + j·ldb] (B_NN =
// true: B is k×n, "NN").  LOWER restricts the update to i >= j (SYRK, m == n).
// beta == 0 never reads C, as in BLAS.  The 128×128 output blocks (the lower
// ones only for LOWER) are numbered column by column; part `part` of `parts`
// computes blocks part, part + parts, ...
// T is double (the FP64 path) or float (the FP32 updates of the mixed path).
template <class T, bool B_NN, bool LOWER>
__device__ void gemm_tile(int m, int n, int k, T alpha, const T* __restrict__ A, int lda, const T* __restrict__ B, int ldb,
                          T beta, T* C, int ldc, T* smem, int part = 0, int parts = 1) {
    T(*As)[kBM] = reinterpret_cast<T(*)[kBM]>(smem);
    T(*Bs)[kBNP] = reinterpret_cast<T(*)[kBNP]>(smem + kBK * kBM);
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int nbm = (m + kBM - 1) / kBM, nbn = (n + kBN - 1) / kBN;
    const int nblk = LOWER ? nbm * (nbm + 1) / 2 : nbm * nbn;
    for (int bidx = part; bidx < nblk; bidx += parts) {
        int bi, bj;
        if (LOWER) {
            int r = bidx;
            bj = 0;
            while (r >= nbm - bj) {
                r -= nbm - bj;
                ++bj;
            }
            bi = bj + r;
        } else {
            bi = bidx % nbm;
            bj = bidx / nbm;
        }
        const int m0 = bi * kBM, n0 = bj * kBN;
        {
            T acc[8][8];
#pragma unroll
            for (int r = 0; r < 8; ++r)
#pragma unroll
                for (int c = 0; c < 8; ++c) acc[r][c] = T(0);
            for (int k0 = 0; k0 < k; k0 += kBK) {
#pragma unroll
                for (int r = 0; r < (kBK * kBM) / kThreads; ++r) {
                    const int idx = tid + kThreads * r;
                    const int i = idx & (kBM - 1), kk = idx / kBM;
                    const int gi = m0 + i, gk = k0 + kk;
                    As[kk][i] = (gi < m && gk < k) ? ldcg(A + gi + (size_t)gk * lda) : T(0);
                }
#pragma unroll
                for (int r = 0; r < (kBK * kBN) / kThreads; ++r) {
                    const int idx = tid + kThreads * r;
                    int j, kk;
                    if (B_NN) { kk = idx & (kBK - 1); j = idx / kBK; }
                    else { j = idx & (kBN - 1); kk = idx / kBN; }
                    const int gj = n0 + j, gk = k0 + kk;
                    T v = T(0);
                    if (gj < n && gk < k) v = B_NN ? ldcg(B + gk + (size_t)gj * ldb) : ldcg(B + gj + (size_t)gk * ldb);
                    Bs[kk][j] = v;
                }
                __syncthreads();
#pragma unroll
                for (int kk = 0; kk < kBK; ++kk) {
                    T a[8], b[8];
#pragma unroll
                    for (int r = 0; r < 8; ++r) a[r] = As[kk][tx + 16 * r];
#pragma unroll
                    for (int c = 0; c < 8; ++c) b[c] = Bs[kk][ty + 16 * c];
#pragma unroll
                    for (int r = 0; r < 8; ++r)
#pragma unroll
                        for (int c = 0; c < 8; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
                }
                __syncthreads();
            }
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const int gj = n0 + ty + 16 * c;
#pragma unroll
                for (int r = 0; r < 8; ++r) {
                    const int gi = m0 + tx + 16 * r;
                    if (gi < m && gj < n && (!LOWER || gi >= gj)) {
                        T* p = C + gi + (size_t)gj * ldc;
                        T v = alpha * acc[r][c];
                        if (beta != T(0)) v = fma(beta, ldcg(p), v);
                        *p = v;
                    }
                }
            }
        }
    }
}

template <bool B_NN, bool LOWER>
__device__ __forceinline__ void gemm_f64(int m, int n, int k, double alpha, const double* A, int lda, const double* B, int ldb,
                                         double beta, double* C, int ldc, double* smem, int part = 0, int parts = 1) {
    gemm_tile<double, B_NN, LOWER>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, smem, part, parts);
}

// Unblocked lower Cholesky of the nb×nb (nb <= 32) diagonal block at A (lda)
// by one warp, lane = row.  Returns 0 or the 1-based failing column.
__device__ inline int potrf_diag32_warp(double* A, int lda, int nb) {
    const int lane = threadIdx.x & 31;
    double r[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) r[j] = (lane < nb && j < nb && j <= lane) ? ldcg(A + lane + (size_t)j * lda) : 0.0;
    int info = 0;
#pragma unroll
    for (int c = 0; c < 32; ++c) {
        if (c < nb && info == 0) {
            const double dcc = __shfl_sync(0xffffffffu, r[c], c);
            if (!(dcc > 0.0)) {
                info = c + 1;
            } else {
                const double d = sqrt(dcc);
                if (lane == c) r[c] = d;
                else if (lane > c) r[c] = r[c] / d;
#pragma unroll
                for (int j = c + 1; j < 32; ++j) {
                    const double ljc = __shfl_sync(0xffffffffu, r[c], j);
                    if (lane >= j) r[j] = fma(-r[c], ljc, r[j]);
                }
            }
        }
    }
    if (info == 0) {
#pragma unroll
        for (int j = 0; j < 32; ++j)
            if (lane < nb && j < nb && j <= lane) A[lane + (size_t)j * lda] = r[j];
    }
    return info;
}

// Rows [row0, m) of X[:, 0:nb] (ldx) <- X · Lᵀ⁻¹ with the nb×nb lower block
// Ls (shared, ld kPanel+1); one thread per row.
template <class T>
__device__ inline void trsm_rows_panel(T* X, int ldx, int row0, int m, int nb, const T* Ls, T alpha) {
    for (int i = row0 + threadIdx.x; i < m; i += kThreads) {
        T x[kPanel];
#pragma unroll
        for (int c = 0; c < kPanel; ++c) x[c] = (c < nb) ? alpha * ldcg(X + i + (size_t)c * ldx) : T(0);
#pragma unroll
        for (int c = 0; c < kPanel; ++c) {
            if (c < nb) {
                T s = x[c];
#pragma unroll
                for (int l = 0; l < c; ++l) s = fma(-x[l], Ls[c * (kPanel + 1) + l], s);
                x[c] = s / Ls[c * (kPanel + 1) + c];
            }
        }
#pragma unroll
        for (int c = 0; c < kPanel; ++c)
            if (c < nb) X[i + (size_t)c * ldx] = x[c];
    }
}

// Load the nb×nb lower block at L (ldl) into Ls (ld kPanel+1), zero above.
template <class T>
__device__ inline void load_panel_block(const T* L, int ldl, int nb, T* Ls) {
    for (int e = threadIdx.x; e < kPanel * kPanel; e += kThreads) {
        const int c = e / kPanel, l = e % kPanel;  // Ls[c][l] = L(c, l)
        Ls[c * (kPanel + 1) + l] = (c < nb && l < nb && l <= c) ? ldcg(L + c + (size_t)l * ldl) : T(0);
    }
}

// In-place lower Cholesky of A[n×n] (right-looking, 32-column panels).
// Returns 0 or the 1-based failing column (as LAPACK's info).
__device__ inline int potrf_l_f64(int n, double* A, int lda, double* smem) {
    __shared__ int s_info;
    double* Ls = smem + kBK * kBM + kBK * kBNP;
    for (int p = 0; p < n; p += kPanel) {
        const int nb = min(kPanel, n - p);
        double* Dpp = A + p + (size_t)p * lda;
        if (threadIdx.x < 32) {
            int info = potrf_diag32_warp(Dpp, lda, nb);
            if (threadIdx.x == 0) s_info = info ? p + info : 0;
        }
        __syncthreads();
        const int info = s_info;
        if (info) return info;
        load_panel_block<double>(Dpp, lda, nb, Ls);
        __syncthreads();
        const int rest = n - p - nb;
        if (rest > 0) {
            trsm_rows_panel<double>(A + (size_t)p * lda, lda, p + nb, n, nb, Ls, 1.0);
            __syncthreads();
            double* P = A + (p + nb) + (size_t)p * lda;
            gemm_f64<false, true>(rest, rest, nb, -1.0, P, lda, P, lda, 1.0, A + (p + nb) + (size_t)(p + nb) * lda, lda, smem);
        }
        __syncthreads();
    }
    return 0;
}

// B[m×n] <- alpha·B·L⁻ᵀ, L n×n lower non-unit (right-looking, 32-column panels).
// Rows are independent: part `part` of `parts` solves one slice of rows.
template <class T>
__device__ inline void trsm_rltn_tile(int m, int n, T alpha, const T* L, int ldl, T* B, int ldb, T* smem, int part = 0,
                                      int parts = 1) {
    T* Ls = smem + kBK * kBM + kBK * kBNP;
    {
        const int per = ((m + parts - 1) / parts + 15) / 16 * 16;
        const int r0 = min(m, part * per), r1 = min(m, r0 + per);
        B += r0;
        m = r1 - r0;
    }
    for (int p = 0; p < n; p += kPanel) {
        const int nb = min(kPanel, n - p);
        load_panel_block<T>(L + p + (size_t)p * ldl, ldl, nb, Ls);
        __syncthreads();
        // Columns right of p are scaled by alpha when their panel is solved;
        // the update below subtracts solved (already scaled) columns, so scale
        // the remaining columns once, before the first update touches them.
        if (p == 0 && alpha != T(1) && n > nb) {
            for (int e = threadIdx.x; e < m * (n - nb); e += kThreads) {
                const int i = e % m, j = nb + e / m;
                B[i + (size_t)j * ldb] = alpha * ldcg(B + i + (size_t)j * ldb);
            }
        }
        trsm_rows_panel<T>(B + (size_t)p * ldb, ldb, 0, m, nb, Ls, p == 0 ? alpha : T(1));
        __syncthreads();
        const int rest = n - p - nb;
        if (rest > 0)
            gemm_tile<T, false, false>(m, rest, nb, T(-1), B + (size_t)p * ldb, ldb, L + (p + nb) + (size_t)p * ldl, ldl, T(1),
                                       B + (size_t)(p + nb) * ldb, ldb, smem);
        __syncthreads();
    }
}

__device__ __forceinline__ void trsm_rltn_f64(int m, int n, double alpha, const double* L, int ldl, double* B, int ldb,
                                              double* smem, int part = 0, int parts = 1) {
    trsm_rltn_tile<double>(m, n, alpha, L, ldl, B, ldb, smem, part, parts);
}

// C[m×n] <- alpha·A + beta·C; part `part` of `parts` takes every parts-th element chunk.
template <class T>
__device__ inline void geadd_tile(int m, int n, T alpha, const T* A, int lda, T beta, T* C, int ldc, int part = 0,
                                  int parts = 1) {
    for (long e = threadIdx.x + (long)part * kThreads; e < (long)m * n; e += (long)kThreads * parts) {
        const int i = (int)(e % m), j = (int)(e / m);
        T v = alpha * ldcg(A + i + (size_t)j * lda);
        if (beta != T(0)) v = fma(beta, ldcg(C + i + (size_t)j * ldc), v);
        C[i + (size_t)j * ldc] = v;
    }
    __syncthreads();
}

__device__ __forceinline__ void geadd_f64(int m, int n, double alpha, const double* A, int lda, double beta, double* C,
                                          int ldc, int part = 0, int parts = 1) {
    geadd_tile<double>(m, n, alpha, A, lda, beta, C, ldc, part, parts);
}


// ------------------------------------------------------------------------
// Team POTRF: one diagonal tile factored by several blocks of the executor.
//
// The factorisation runs as a sequence of phases; for every 32-column panel:
// the 32×32 diagonal block (one warp), the panel rows below it (32-row
// items), and the lower 64×64 blocks of the trailing update.  Every block
// that holds a part of the task claims items of the current phase from a
// per-task counter and then waits until all items of the phase are done.  A
// block never waits for a part that has not started — whoever is present does
// the work — so the team cannot deadlock, and a single block alone factors
// the whole tile.  Waits are bounded by limit_ns.
//
// ctr: kTeamCounters ints per task, zero at launch: (claimed, done) per
// phase; ctr[kTeamCounters - 2] = phases completed; ctr[kTeamCounters - 1] =
// the first failing column.
constexpr int kTeamCounters = 256;
constexpr int kTeamPanelRows = 32;  // rows per panel item
constexpr int kTeamCopyRows = 128;  // rows per widen / narrow item

// Phases of potrf_l_f64_team on an n×n tile; the team form needs
// 2·phases + 2 <= kTeamCounters.
__host__ __device__ inline int team_phases(int n, bool widen) { return 3 * ((n + kPanel - 1) / kPanel) + (widen ? 2 : 0); }
__host__ __device__ inline bool team_fits(int n, bool widen) { return 2 * team_phases(n, widen) + 2 <= kTeamCounters; }

struct TeamCtx {
    int* ctr;
    long long limit_ns;
    int* err;  // executor status word (set to TTG_ETIMEOUT on a timeout)
};

__device__ __forceinline__ long long team_clock() {
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Claim the next item of phase ph (the same value on all threads).
__device__ __forceinline__ int team_claim(const TeamCtx& tc, int ph) {
    __shared__ int s_item;
    __syncthreads();
    if (threadIdx.x == 0) s_item = atomicAdd(tc.ctr + 2 * ph, 1);
    __syncthreads();
    return s_item;
}

// Publish one finished item of phase ph (of `items`); the block that finishes
// the last item advances the completed-phase marker.  Returns (on every
// thread) whether this item completed the phase.
__device__ __forceinline__ bool team_done(const TeamCtx& tc, int ph, int items) {
    __shared__ int s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const bool last = atomicAdd(tc.ctr + 2 * ph + 1, 1) == items - 1;
        if (last) atomicMax(tc.ctr + kTeamCounters - 2, ph + 1);
        s_last = last;
    }
    __syncthreads();
    return s_last != 0;
}

// Phases completed so far (the same value on all threads).
__device__ __forceinline__ int team_progress(const TeamCtx& tc) {
    __shared__ int s_prog;
    __syncthreads();
    if (threadIdx.x == 0) s_prog = *(const volatile int*)(tc.ctr + kTeamCounters - 2);
    __syncthreads();
    return s_prog;
}

// Wait until `items` items of phase ph are done; false on timeout.
__device__ __forceinline__ bool team_wait(const TeamCtx& tc, int ph, int items) {
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        int ok = 1;
        const volatile int* d = tc.ctr + 2 * ph + 1;
        if (*d < items) {
            const long long t0 = team_clock();
            for (unsigned it = 0; *d < items; ++it) {
                if ((it & 63) == 63 && team_clock() - t0 > tc.limit_ns) {
                    ok = 0;
                    atomicCAS(tc.err, 0, 3 /* TTG_ETIMEOUT */);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Shared-memory layout of the team POTRF (doubles): the 32×32 diagonal block
// L (ld 33), its inverse X (ld 33), 1/L_cc, and two 32×33 work panels.
constexpr int kTS = 0, kTX = 1056, kTInv = 2112, kTW1 = 2144, kTW2 = 3200, kTeamSmemDoubles = 4256;
static_assert(kTeamSmemDoubles <= kF64SmemDoubles, "team POTRF shared memory");

// Lower Cholesky of the nb×nb (nb <= 32) diagonal block at D (ld) in shared
// memory S (ld 33) by warps 0-3: column c's pivot is taken by warp c % 4
// (one rsqrt: l_cc = d·d^-1/2, the column scaled by d^-1/2, kept in inv[c]),
// then warp w updates the columns j > c with j % 4 == w (lane = row).  Every
// FP64 operation of a GB300 warp costs ~65 cycles whatever its active lanes,
// so the column updates are spread over the four sub-partitions.  Returns 0
// or the 1-based failing column; S and inv hold the factor.
__device__ inline int team_diag_factor(const double* D, int ld, int nb, double* S, double* inv) {
    __shared__ int s_info;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int e = threadIdx.x; e < 32 * 32; e += kThreads) {
        const int i = e & 31, j = e >> 5;
        S[i * 33 + j] = (i < nb && j < nb && i >= j) ? ldcg(D + i + (size_t)j * ld) : 0.0;
    }
    if (threadIdx.x == 0) s_info = 0;
    __syncthreads();
    for (int c = 0; c < nb; ++c) {
        if (warp == (c & 3)) {
            const double d = S[c * 33 + c];
            if (!(d > 0.0)) {
                if (lane == 0) s_info = c + 1;
            } else {
                const double y = rsqrt(d);
                if (lane == c) {
                    S[c * 33 + c] = d * y;
                    inv[c] = y;
                } else if (lane > c && lane < nb) {
                    S[lane * 33 + c] *= y;
                }
            }
        }
        __syncthreads();
        if (s_info) break;
        if (warp < 4)
            for (int j = c + 1 + ((warp - c - 1) & 3); j < nb; j += 4)
                if (lane >= j && lane < nb) S[lane * 33 + j] = fma(-S[lane * 33 + c], S[j * 33 + c], S[lane * 33 + j]);
        __syncthreads();
    }
    return s_info;
}

// X = L⁻¹ (lower, ld 33) from the factor S and inv (1/L_ii) by warps 0-3:
// row i of X is finished by warp i % 4, then warp w subtracts L_ji·X_i from
// its rows j > i (lane = column).
__device__ inline void team_diag_inverse(const double* S, const double* inv, int nb, double* X) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int e = threadIdx.x; e < 32 * 32; e += kThreads) {
        const int j = e >> 5, c = e & 31;
        X[j * 33 + c] = (j == c && j < nb) ? 1.0 : 0.0;
    }
    __syncthreads();
    for (int i = 0; i < nb; ++i) {
        if (warp == (i & 3) && lane <= i) X[i * 33 + lane] *= inv[i];
        __syncthreads();
        if (warp < 4)
            for (int j = i + 1 + ((warp - i - 1) & 3); j < nb; j += 4)
                if (lane <= i) X[j * 33 + lane] = fma(-S[j * 33 + i], X[i * 33 + lane], X[j * 33 + lane]);
        __syncthreads();
    }
}

// Rows [r0, r0 + rows) (rows <= 32) of the panel P (columns 0..nb-1, ld) <-
// P · L⁻ᵀ = P · Xᵀ: thread (r, g) computes columns g, g+8, g+16, g+24.
__device__ inline void team_panel_rows(double* P, int ld, int r0, int rows, int nb, const double* X, double* W) {
    for (int e = threadIdx.x; e < 32 * 32; e += kThreads) {
        const int r = e & 31, c = e >> 5;
        W[r * 33 + c] = (r < rows && c < nb) ? ldcg(P + r0 + r + (size_t)c * ld) : 0.0;
    }
    __syncthreads();
    const int r = threadIdx.x & 31, g = threadIdx.x >> 5;
    double acc[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int j = g + 8 * k;
        double a = 0.0;
        for (int c = 0; c <= j && c < nb; ++c) a = fma(W[r * 33 + c], X[j * 33 + c], a);
        acc[k] = a;
    }
    if (r < rows) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int j = g + 8 * k;
            if (j < nb) P[r0 + r + (size_t)j * ld] = acc[k];
        }
    }
    __syncthreads();
}

// Lower 32×32 block `item` (column by column over the lower triangle) of
// C[rest×rest] -= Q·Qᵀ, Q rest×nb (nb <= 32, ld).
__device__ inline void team_syrk_block32(int rest, int nb, const double* Q, int ld, double* C, int item, double* W1, double* W2) {
    const int mb = (rest + 31) / 32;
    int bj = 0, rr = item;
    while (rr >= mb - bj) {
        rr -= mb - bj;
        ++bj;
    }
    const int bi = bj + rr;
    const int m0 = bi * 32, n0 = bj * 32;
    for (int e = threadIdx.x; e < 32 * 32; e += kThreads) {
        const int r = e & 31, c = e >> 5;
        W1[r * 33 + c] = (m0 + r < rest && c < nb) ? ldcg(Q + m0 + r + (size_t)c * ld) : 0.0;
        W2[r * 33 + c] = (n0 + r < rest && c < nb) ? ldcg(Q + n0 + r + (size_t)c * ld) : 0.0;
    }
    __syncthreads();
    const int r = threadIdx.x & 31, g = threadIdx.x >> 5;
    const bool diag = bi == bj;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int j = g + 8 * k;
        const int gi = m0 + r, gj = n0 + j;
        if (gi < rest && gj < rest && (!diag || r >= j)) {
            double a = 0.0;
#pragma unroll 8
            for (int c = 0; c < kPanel; ++c) a = fma(W1[r * 33 + c], W2[j * 33 + c], a);
            double* q = C + gi + (size_t)gj * ld;
            *q = ldcg(q) - a;
        }
    }
    __syncthreads();
}

// Team lower Cholesky of the FP64 tile A[n×n] (lda); requires
// team_fits(n, W32 != nullptr).  With an FP32 source (W32 != nullptr) the
// team first widens the lower triangle of W32 (ldw) into A and at the end
// rounds the factor back into W32.  Per 32-column panel: the diagonal block
// (one block, team_diag_factor), the panel rows in 32-row items (each block
// that takes one first inverts the diagonal block for itself), the trailing
// lower 32×32 blocks.  Returns 0, the 1-based failing column, or -1 after a
// timeout.  *finisher (shared) is set to 1 in the one block that completed
// the factorisation (or found the failing column), else 0: that block
// releases the task's successors at once, whether or not the other parts of
// the team have run yet.  The result is the same for any number of blocks:
// every item computes the same arithmetic whoever runs it.
__device__ inline int potrf_l_f64_team(int n, double* A, int lda, double* smem, const TeamCtx& tc, float* W32, int ldw,
                                       int* finisher) {
    double* S = smem + kTS;
    double* X = smem + kTX;
    double* inv = smem + kTInv;
    double* W1 = smem + kTW1;
    double* W2 = smem + kTW2;
    // An empty tile has no phases: its parts complete as ordinary parts
    // (*finisher keeps the executor's -1).
    if (n <= 0) return 0;
    if (threadIdx.x == 0) *finisher = 0;
    int ph = 0;
    const int copy_items = (n + kTeamCopyRows - 1) / kTeamCopyRows;
    if (W32) {
        for (int it = team_claim(tc, ph); it < copy_items; it = team_claim(tc, ph)) {
            const int r0 = it * kTeamCopyRows, r1 = min(n, r0 + kTeamCopyRows), rows = r1 - r0;
            for (long e = threadIdx.x; e < (long)rows * n; e += kThreads) {
                const int i = r0 + (int)(e % rows), j = (int)(e / rows);
                A[i + (size_t)j * lda] = i >= j ? (double)__ldcg(W32 + i + (size_t)j * ldw) : 0.0;
            }
            team_done(tc, ph, copy_items);
        }
        if (!team_wait(tc, ph, copy_items)) return -1;
        ++ph;
    }
    for (int p = 0; p < n; p += kPanel, ph += 3) {
        // Panels that the team has already finished are skipped by late blocks.
        if (team_progress(tc) >= ph + 3) continue;
        const int nb = min(kPanel, n - p);
        double* Dpp = A + p + (size_t)p * lda;
        if (team_claim(tc, ph) == 0) {
            __shared__ int s_bad;
            const int info = team_diag_factor(Dpp, lda, nb, S, inv);
            if (info == 0) {
                for (int e = threadIdx.x; e < 32 * 32; e += kThreads) {
                    const int i = e & 31, j = e >> 5;
                    if (i < nb && j <= i) Dpp[i + (size_t)j * lda] = S[i * 33 + j];
                }
            }
            if (threadIdx.x == 0) {
                s_bad = info != 0;
                if (info) atomicExch(tc.ctr + kTeamCounters - 1, p + info);
            }
            team_done(tc, ph, 1);
            // The factorisation ends here after a failure, or after the last
            // panel when there is no FP32 copy to write.
            if (threadIdx.x == 0 && (s_bad || (p + nb >= n && !W32))) *finisher = 1;
        }
        if (!team_wait(tc, ph, 1)) return -1;
        {
            const int info = *(const volatile int*)(tc.ctr + kTeamCounters - 1);
            if (info) return info;
        }
        const int rest = n - p - nb;
        if (rest <= 0) continue;
        const int pitems = (rest + kTeamPanelRows - 1) / kTeamPanelRows;
        bool have_inverse = false;
        for (int it = team_claim(tc, ph + 1); it < pitems; it = team_claim(tc, ph + 1)) {
            if (!have_inverse) {
                // The factored diagonal block and 1/L_ii (this block may not
                // be the one that factored it), then its inverse.
                for (int e = threadIdx.x; e < 32 * 32; e += kThreads) {
                    const int i = e & 31, j = e >> 5;
                    S[i * 33 + j] = (i < nb && j < nb && i >= j) ? ldcg(Dpp + i + (size_t)j * lda) : 0.0;
                }
                __syncthreads();
                if (threadIdx.x < nb) inv[threadIdx.x] = 1.0 / S[threadIdx.x * 33 + threadIdx.x];
                __syncthreads();
                team_diag_inverse(S, inv, nb, X);
                have_inverse = true;
            }
            const int r0 = p + nb + it * kTeamPanelRows;
            team_panel_rows(A + (size_t)p * lda, lda, r0, min(kTeamPanelRows, n - r0), nb, X, W1);
            team_done(tc, ph + 1, pitems);
        }
        if (!team_wait(tc, ph + 1, pitems)) return -1;
        const int mb = (rest + 31) / 32;
        const int citems = mb * (mb + 1) / 2;
        const double* Q = A + (p + nb) + (size_t)p * lda;
        double* C = A + (p + nb) + (size_t)(p + nb) * lda;
        for (int it = team_claim(tc, ph + 2); it < citems; it = team_claim(tc, ph + 2)) {
            team_syrk_block32(rest, nb, Q, lda, C, it, W1, W2);
            team_done(tc, ph + 2, citems);
        }
        if (!team_wait(tc, ph + 2, citems)) return -1;
    }
    if (W32) {
        for (int it = team_claim(tc, ph); it < copy_items; it = team_claim(tc, ph)) {
            const int r0 = it * kTeamCopyRows, r1 = min(n, r0 + kTeamCopyRows), rows = r1 - r0;
            for (long e = threadIdx.x; e < (long)rows * n; e += kThreads) {
                const int i = r0 + (int)(e % rows), j = (int)(e / rows);
                if (i >= j) W32[i + (size_t)j * ldw] = (float)__ldcg(A + i + (size_t)j * lda);
            }
            if (team_done(tc, ph, copy_items) && threadIdx.x == 0) *finisher = 1;
        }
        if (!team_wait(tc, ph, copy_items)) return -1;
    }
    return 0;
}

}  // namespace ttg
