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
// beta == 0 never reads C, as in BLAS.  The BS×BS output blocks (the lower
// ones only for LOWER) are numbered column by column; part `part` of `parts`
// computes blocks part, part + parts, ...  BS = 128 (8×8 per thread) or 64
// (4×4 per thread: small tiles split into four times as many parts).
// T is double (the FP64 path) or float (the FP32 updates of the mixed path).
template <class T, bool B_NN, bool LOWER, int BS = 128>
__device__ void gemm_tile(int m, int n, int k, T alpha, const T* __restrict__ A, int lda, const T* __restrict__ B, int ldb,
                          T beta, T* C, int ldc, T* smem, int part = 0, int parts = 1) {
    static_assert(BS == 128 || BS == 64 || BS == 32, "output block edge");
    constexpr int R = BS / 16;  // outputs per thread and dimension
    T(*As)[BS] = reinterpret_cast<T(*)[BS]>(smem);
    T(*Bs)[BS + 1] = reinterpret_cast<T(*)[BS + 1]>(smem + kBK * BS);
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int nbm = (m + BS - 1) / BS, nbn = (n + BS - 1) / BS;
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
        const int m0 = bi * BS, n0 = bj * BS;
        {
            T acc[R][R];
#pragma unroll
            for (int r = 0; r < R; ++r)
#pragma unroll
                for (int c = 0; c < R; ++c) acc[r][c] = T(0);
            for (int k0 = 0; k0 < k; k0 += kBK) {
#pragma unroll
                for (int r = 0; r < (kBK * BS) / kThreads; ++r) {
                    const int idx = tid + kThreads * r;
                    const int i = idx & (BS - 1), kk = idx / BS;
                    const int gi = m0 + i, gk = k0 + kk;
                    As[kk][i] = (gi < m && gk < k) ? ldcg(A + gi + (size_t)gk * lda) : T(0);
                }
#pragma unroll
                for (int r = 0; r < (kBK * BS) / kThreads; ++r) {
                    const int idx = tid + kThreads * r;
                    int j, kk;
                    if (B_NN) { kk = idx & (kBK - 1); j = idx / kBK; }
                    else { j = idx & (BS - 1); kk = idx / BS; }
                    const int gj = n0 + j, gk = k0 + kk;
                    T v = T(0);
                    if (gj < n && gk < k) v = B_NN ? ldcg(B + gk + (size_t)gj * ldb) : ldcg(B + gj + (size_t)gk * ldb);
                    Bs[kk][j] = v;
                }
                __syncthreads();
#pragma unroll
                for (int kk = 0; kk < kBK; ++kk) {
                    T a[R], b[R];
#pragma unroll
                    for (int r = 0; r < R; ++r) a[r] = As[kk][tx + 16 * r];
#pragma unroll
                    for (int c = 0; c < R; ++c) b[c] = Bs[kk][ty + 16 * c];
#pragma unroll
                    for (int r = 0; r < R; ++r)
#pragma unroll
                        for (int c = 0; c < R; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
                }
                __syncthreads();
            }
            // Per column: the R reads of C first (in flight together), then
            // the R writes — with a short k the epilogue is otherwise a chain
            // of R² memory round trips.
#pragma unroll
            for (int c = 0; c < R; ++c) {
                const int gj = n0 + ty + 16 * c;
                T cv[R];
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int gi = m0 + tx + 16 * r;
                    const bool ok = gi < m && gj < n && (!LOWER || gi >= gj);
                    cv[r] = (ok && beta != T(0)) ? ldcg(C + gi + (size_t)gj * ldc) : T(0);
                }
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int gi = m0 + tx + 16 * r;
                    if (gi < m && gj < n && (!LOWER || gi >= gj)) {
                        T v = alpha * acc[r][c];
                        if (beta != T(0)) v = fma(beta, cv[r], v);
                        C[gi + (size_t)gj * ldc] = v;
                    }
                }
            }
        }
    }
}

// Output block edge of an FP64 tile update: 32 for tiles up to 128, 64 up
// to 256 (more parts, so that small tiles spread over more SMs: at this
// GPU's FP64 rate a 128×128×128 update takes ~0.5 ms on one block), else
// 128.  The edge never changes an output's summation order.  FP32 updates
// keep 128 (their 8×8 register blocks use the FMA pipe better).
__host__ __device__ constexpr int gemm_block_edge(int m, int n, bool f64 = true) {
    return (f64 && m <= 128 && n <= 128) ? 32 : (f64 && m <= 256 && n <= 256) ? 64 : 128;
}

// FP64 updates in 32-row blocks, out of line (the executor's register
// budget stays with the larger blocks).
template <bool B_NN, bool LOWER>
static __device__ __noinline__ void gemm_tile_f64_e32(int m, int n, int k, double alpha, const double* A, int lda, const double* B,
                                                      int ldb, double beta, double* C, int ldc, double* smem, int part, int parts) {
    gemm_tile<double, B_NN, LOWER, 32>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, smem, part, parts);
}

template <class T, bool B_NN, bool LOWER>
__device__ __forceinline__ void gemm_tile_auto(int m, int n, int k, T alpha, const T* A, int lda, const T* B, int ldb, T beta, T* C,
                                               int ldc, T* smem, int part = 0, int parts = 1) {
    if constexpr (sizeof(T) == 8) {
        if (gemm_block_edge(m, n, true) == 32) {
            gemm_tile_f64_e32<B_NN, LOWER>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, smem, part, parts);
            return;
        }
    }
    if (gemm_block_edge(m, n, sizeof(T) == 8) == 64)
        gemm_tile<T, B_NN, LOWER, 64>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, smem, part, parts);
    else
        gemm_tile<T, B_NN, LOWER, 128>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, smem, part, parts);
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
#pragma unroll
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

// The TRSM's column update for slices of at most 64 rows, in 64-row blocks;
// out of line, so that the executor's register budget stays with its tile
// kernels.
static __device__ __noinline__ void trsm_update_f64_small(int m, int n, int k, const double* A, int lda, const double* B, int ldb,
                                                          double* C, int ldc, double* smem) {
    gemm_tile<double, false, false, 64>(m, n, k, -1.0, A, lda, B, ldb, 1.0, C, ldc, smem);
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
        // The update of the columns right of the panel: FP64 slices of at
        // most 32 (64) rows in 32-row (64-row) blocks (a part of 32 rows in a
        // 128-row block ran four times the DFMAs it needs: 381 of a 527 µs
        // TRSM at tile 128).  The block edge does not change any output's
        // summation order.
        if constexpr (sizeof(T) == 8) {
            if (rest > 0 && m <= 32)
                gemm_tile_f64_e32<false, false>(m, rest, nb, -1.0, B + (size_t)p * ldb, ldb, L + (p + nb) + (size_t)p * ldl, ldl,
                                                1.0, B + (size_t)(p + nb) * ldb, ldb, smem, 0, 1);
            else if (rest > 0 && m <= 64)
                trsm_update_f64_small(m, rest, nb, B + (size_t)p * ldb, ldb, L + (p + nb) + (size_t)p * ldl, ldl,
                                      B + (size_t)(p + nb) * ldb, ldb, smem);
            else if (rest > 0)
                gemm_tile<T, false, false>(m, rest, nb, T(-1), B + (size_t)p * ldb, ldb, L + (p + nb) + (size_t)p * ldl, ldl, T(1),
                                           B + (size_t)(p + nb) * ldb, ldb, smem);
        } else if (rest > 0)
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
// The tile is cut into P×P blocks of 32×32 (P = ceil(n/32)), and the
// factorisation into items over the lower blocks:
//   F(j)       for j >= 1 first the panel block (j,j-1) <- A_j,j-1 · L_j-1,j-1⁻ᵀ
//              (published at once) and the last update of the diagonal block,
//              A_jj -= L_j,j-1 · L_j,j-1ᵀ; then factor (j,j) and invert it,
//   R(j, i)    panel block (i,j) <- A_ij · L_jj⁻ᵀ            (i >= j+2),
//   T(p, i, j) trailing update A_ij -= L_ip · L_jpᵀ           (i >= j > p, not i = j = p+1).
// F(j) holds the whole critical chain of a panel (one handoff per panel
// instead of three); its arithmetic is that of the separate D, R and T steps,
// in the same order.  One state byte per block counts what it has received:
// block (i,j) holds state p after the updates of panels 0..p-1, and j+1 once
// it is final.  Every item waits only for the blocks it reads and writes —
// F(j) for state(j-1,j-1) = j, state(j,j-1) = state(j,j) = j-1; R(j,i) for
// state(j,j) = j+1 and state(i,j) = j; T(p,i,j) for state(i,p) = state(j,p)
// = p+1 and state(i,j) = p — so the next panel starts as soon as its own
// blocks are ready (look-ahead) and the updates of every block are applied
// in panel order (deterministic result).
//
// Blocks of the team claim items from one counter in a fixed order, segment
// by segment: seg(j) = F(j), T(j-1,·,j), R(j,·), T(j-1,·,j+1), then the rest
// of panel j-1's trailing update T(j-1,·,>=j+2).  The next panel's critical
// items come before the bulk of the previous trailing update, and everything
// an item waits for is claimed before it by a block that is running, so the
// team cannot deadlock and a single block alone factors the whole tile.
// Waits are bounded by limit_ns.
//
// ctr: kTeamCounters ints per task, zero at launch: [0] items claimed, [1]
// items done, [2] first failing column (1-based), then the state bytes of
// the lower blocks ((i,j) at byte i(i+1)/2 + j).
constexpr int kTeamCounters = 256;
constexpr int kTeamHeader = 8;  // ints before the state bytes

__host__ __device__ inline int team_blocks(int n) { return (n + kPanel - 1) / kPanel; }
// The team form needs one state byte per lower block.
__host__ __device__ inline bool team_fits(int n) {
    const int P = team_blocks(n);
    return P * (P + 1) / 2 <= (kTeamCounters - kTeamHeader) * 4;
}

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

// One item of the order above: kind 0 F(p), 1 R(p, bi), 2 T(p, bi, bj); kind
// -1 past the last item.
struct TeamItem {
    int kind, p, bi, bj;
};

__host__ __device__ inline int team_segment_items(int P, int j) {
    const int m = P - 1 - j;
    return 1 + (m > 1 ? m - 1 : 0) + (j >= 1 ? 2 * m + m * (m - 1) / 2 : 0);
}

__host__ __device__ inline int team_total_items(int P) {
    int t = 0;
    for (int j = 0; j < P; ++j) t += team_segment_items(P, j);
    return t;
}

__host__ __device__ inline TeamItem team_item(int P, int idx) {
    for (int j = 0; j < P; ++j) {
        const int m = P - 1 - j;
        const int cnt = team_segment_items(P, j);
        if (idx >= cnt) {
            idx -= cnt;
            continue;
        }
        int k = idx;
        if (k < 1) return {0, j, j, j};  // F(j)
        k -= 1;
        if (j >= 1) {
            if (k < m) return {2, j - 1, j + 1 + k, j};  // panel j-1, column j
            k -= m;
        }
        const int nr = m > 1 ? m - 1 : 0;
        if (k < nr) return {1, j, j + 2 + k, j};  // R(j, i), i >= j+2
        k -= nr;
        if (k < m) return {2, j - 1, j + 1 + k, j + 1};  // panel j-1, column j+1 (j >= 1 here)
        k -= m;
        int bj = j + 2;
        while (k >= P - bj) {
            k -= P - bj;
            ++bj;
        }
        return {2, j - 1, bj + k, bj};  // rest of panel j-1
    }
    return {-1, 0, 0, 0};
}

__device__ __forceinline__ volatile unsigned char* team_state(const TeamCtx& tc, int bi, int bj) {
    return reinterpret_cast<volatile unsigned char*>(tc.ctr + kTeamHeader) + bi * (bi + 1) / 2 + bj;
}

// Thread 0 waits until every (state, value) pair holds (a null state is no
// condition); the outcome is returned on all threads: 0, the failing column
// after another block found the tile not positive definite, or -1 after a
// timeout.
__device__ inline int team_wait_states(const TeamCtx& tc, volatile unsigned char* s0, int v0, volatile unsigned char* s1,
                                       int v1, volatile unsigned char* s2, int v2) {
    __shared__ int s_res;
    if (threadIdx.x == 0) {
        auto ready = [&]() { return (!s0 || *s0 >= v0) && (!s1 || *s1 >= v1) && (!s2 || *s2 >= v2); };
        int res = 0;
        if (!ready()) {
            const long long t0 = team_clock();
            for (unsigned it = 0;; ++it) {
                if (ready()) break;
                if ((it & 63) == 63) {
                    const int bad = *(const volatile int*)(tc.ctr + 2);
                    if (bad) {
                        res = bad;
                        break;
                    }
                    if (team_clock() - t0 > tc.limit_ns) {
                        res = -1;
                        atomicCAS(tc.err, 0, 3 /* TTG_ETIMEOUT */);
                        break;
                    }
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        s_res = res;
    }
    __syncthreads();
    return s_res;
}

// Publish a block: its writes (all threads, before the call) are made
// visible, then its state is set.
__device__ __forceinline__ void team_publish(volatile unsigned char* st, int v) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        *st = (unsigned char)v;
    }
}

// Shared-memory layout of the team POTRF (doubles): a 32×32 block S (ld 33),
// the inverse X of a diagonal block (ld 33), 1/L_cc, and two 32×33 work
// blocks.
constexpr int kTS = 0, kTX = 1056, kTInv = 2112, kTW1 = 2144, kTW2 = 3200, kTeamSmemDoubles = 4256;
static_assert(kTeamSmemDoubles <= kF64SmemDoubles, "team POTRF shared memory");

// Lower Cholesky of the nb×nb (nb <= 32) block in S (ld 33) and, one column
// behind it, the inverse X = L⁻¹ (X starts as the identity).  Factor, warps
// 0-3: column c's pivot is taken by warp c % 4 (one rsqrt: l_cc = d·d^-1/2,
// the column scaled by d^-1/2, kept in inv[c]), then warp w updates the
// columns j > c with j % 4 == w (lane = row).  Inverse, warps 4-7, row i as
// soon as column i of L is final: row i of X is scaled by inv[i], then the
// rows j > i (j % 4 == w - 4) subtract L_ji·X_i (lane = column).  Every FP64
// operation of a GB300 warp costs ~65 cycles whatever its active lanes, so
// the work is spread over the four sub-partitions twice.  Returns 0 or the
// 1-based failing column.
__device__ inline int team_factor_invert(int nb, double* S, double* X, double* inv) {
    __shared__ int s_info;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) s_info = 0;
    __syncthreads();
    for (int c = 0; c <= nb; ++c) {
        const int i = c - 1;  // row of X finished in this step
        if (c < nb && warp == (c & 3)) {
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
        } else if (i >= 0 && warp == 4 + (i & 3) && lane <= i) {
            X[i * 33 + lane] *= inv[i];
        }
        __syncthreads();
        if (s_info) break;
        if (warp < 4) {
            if (c < nb)
                for (int j = c + 1 + ((warp - c - 1) & 3); j < nb; j += 4)
                    if (lane >= j && lane < nb) S[lane * 33 + j] = fma(-S[lane * 33 + c], S[j * 33 + c], S[lane * 33 + j]);
        } else if (i >= 0) {
            for (int j = i + 1 + ((warp - 4 - i - 1) & 3); j < nb; j += 4)
                if (lane <= i) X[j * 33 + lane] = fma(-S[j * 33 + i], X[i * 33 + lane], X[j * 33 + lane]);
        }
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

// Block of the tile (rows × cols at row r0, column c0) into W (ld 33), from
// the FP32 source when `wide` (the first touch of a block in the mixed path)
// else from A; lower_only keeps the lower triangle of a diagonal block.
__device__ inline void team_load_block(double* W, const double* A, int lda, const float* W32, int ldw, bool wide, int r0, int c0,
                                       int rows, int cols, bool lower_only) {
#pragma unroll
    for (int e = threadIdx.x; e < 32 * 32; e += kThreads) {
        const int r = e & 31, c = e >> 5;
        double v = 0.0;
        if (r < rows && c < cols && (!lower_only || r >= c))
            v = wide ? (double)__ldcg(W32 + (r0 + r) + (size_t)(c0 + c) * ldw) : ldcg(A + (r0 + r) + (size_t)(c0 + c) * lda);
        W[r * 33 + c] = v;
    }
}

// Block (rows × cols at r0, c0) from W (ld 33) into A and, when W32 is set,
// rounded into the FP32 tile (a final factor block of the mixed path).
__device__ inline void team_store_block(const double* W, double* A, int lda, float* W32, int ldw, int r0, int c0, int rows, int cols,
                                        bool lower_only) {
    for (int e = threadIdx.x; e < 32 * 32; e += kThreads) {
        const int r = e & 31, c = e >> 5;
        if (r < rows && c < cols && (!lower_only || r >= c)) {
            const double v = W[r * 33 + c];
            A[(r0 + r) + (size_t)(c0 + c) * lda] = v;
            if (W32) W32[(r0 + r) + (size_t)(c0 + c) * ldw] = (float)v;
        }
    }
}

// Where a diagonal block's inverse is kept for the R items of its panel: the
// strictly upper h×h corner of the FP64 scratch tile (rows 0..h-1, columns
// n-h..n-1, h = n/2), which the factorisation never touches.  Element k of the
// P inverses (32×32 each, ld 32) -> A offset; usable when h² >= P·1024.
__device__ __forceinline__ size_t team_xoff(int n, int lda, int k) {
    const int h = n / 2;
    return (size_t)(k % h) + (size_t)(n - h + k / h) * lda;
}

// W1 (32 rows × nb, ld 33) <- W1 · Xᵀ for the lower triangular X = L_pp⁻¹
// (ld 33): thread (row r, group g) forms columns g, 15-g, 16+g and 31-g
// (column j sums j+1 products: 66 per thread in every group).
__device__ __forceinline__ int team_apply_col(int g, int k) { return k == 0 ? g : (k == 1 ? 15 - g : (k == 2 ? 16 + g : 31 - g)); }
__device__ inline void team_apply_inverse(double* W1, const double* X, int nb) {
    const int r = threadIdx.x & 31, g = threadIdx.x >> 5;
    double acc[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int j = team_apply_col(g, k);
        double a = 0.0;
        for (int c = 0; c <= j && c < nb; ++c) a = fma(W1[r * 33 + c], X[j * 33 + c], a);
        acc[k] = a;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 4; ++k) W1[r * 33 + team_apply_col(g, k)] = acc[k];
}

// S = lower(C) − W1·W1ᵀ for the nb×nb diagonal block (C at (r0, r0) of A, or
// of the FP32 source when wide): the 528 lower entries packed over the
// block's threads (half the FP64 instructions of a full 32×32 product: on
// this GPU a warp's FP64 FMA holds its sub-partition's FP64 pipe for 64
// cycles whatever lanes are active), three independent sums per thread (32
// products each, in column order).  The upper part of S is zero.
__device__ inline void team_syrk_lower(double* S, const double* W1, const double* A, int lda, const float* W32, int ldw, bool wide,
                                       int r0, int nb) {
    int rr[3], jj[3];
    bool on[3];
    double cv[3], acc[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int e = threadIdx.x + q * kThreads;
        int r = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
        while (r > 0 && r * (r + 1) / 2 > e) --r;
        while ((r + 1) * (r + 2) / 2 <= e) ++r;
        rr[q] = r;
        jj[q] = e - r * (r + 1) / 2;
        on[q] = e < 528 && r < nb;
        const size_t o = (size_t)(r0 + r) + (size_t)(r0 + jj[q]) * (wide ? ldw : lda);
        cv[q] = !on[q] ? 0.0 : (wide ? (double)__ldcg(W32 + o) : ldcg(A + o));
        acc[q] = 0.0;
    }
#pragma unroll 8
    for (int c = 0; c < kPanel; ++c) {
#pragma unroll
        for (int q = 0; q < 3; ++q)
            if (on[q]) acc[q] = fma(W1[rr[q] * 33 + c], W1[jj[q] * 33 + c], acc[q]);
    }
#pragma unroll
    for (int q = 0; q < 3; ++q)
        if (threadIdx.x + q * kThreads < 528) {
            S[rr[q] * 33 + jj[q]] = on[q] ? cv[q] - acc[q] : 0.0;
            if (jj[q] != rr[q]) S[jj[q] * 33 + rr[q]] = 0.0;
        }
}

// Team lower Cholesky of the FP64 tile A[n×n] (lda); requires team_fits(n).
// With an FP32 source (W32 != nullptr, the mixed path) A is FP64 scratch:
// the first item that touches a block reads it from W32 (ldw), and every
// final block is also rounded back into W32.  Returns 0, the 1-based failing
// column, or -1 after a timeout.  *finisher (shared) is set to 1 in the one
// block that completed the last item (or found the failing column), else 0:
// that block releases the task's successors at once, whether or not the other
// parts of the team have run yet.  The result is the same for any number of
// blocks: every item computes the same arithmetic whoever runs it.
__device__ inline int potrf_l_f64_team(int n, double* A, int lda, double* smem, const TeamCtx& tc, float* W32, int ldw,
                                       int* finisher) {
    double* S = smem + kTS;
    double* X = smem + kTX;
    double* inv = smem + kTInv;
    double* W1 = smem + kTW1;
    double* W2 = smem + kTW2;
    __shared__ int s_item, s_xpanel;
    // An empty tile has no items: its parts complete as ordinary parts
    // (*finisher keeps the executor's -1).
    if (n <= 0) return 0;
    const int P = team_blocks(n);
    const int total = team_total_items(P);
    // The mixed path keeps each diagonal inverse for the panel's R items; the
    // FP64 path (A is the caller's tile) recomputes it in every block.
    const bool keep_x = W32 != nullptr && (long)(n / 2) * (n / 2) >= (long)P * 1024;
    if (threadIdx.x == 0) {
        *finisher = 0;
        s_xpanel = -1;
    }
    auto rows_of = [&](int b) { return min(kPanel, n - kPanel * b); };
    // X = L_qq⁻¹ for the panel-block products of panel q: the kept copy (mixed
    // path) or recomputed from L_qq, the same bits whichever block does it.
    auto panel_inverse = [&](int q, int nq) {
        if (s_xpanel == q) return;
        if (keep_x) {
            for (int e = threadIdx.x; e < 32 * 32; e += kThreads) {
                const int r = e & 31, c = e >> 5;
                X[r * 33 + c] = ldcg(A + team_xoff(n, lda, q * 1024 + e));
            }
        } else {
            team_load_block(S, A, lda, nullptr, 0, false, kPanel * q, kPanel * q, nq, nq, true);
            __syncthreads();
            if (threadIdx.x < nq) inv[threadIdx.x] = 1.0 / S[threadIdx.x * 33 + threadIdx.x];
            __syncthreads();
            team_diag_inverse(S, inv, nq, X);
        }
        __syncthreads();
        if (threadIdx.x == 0) s_xpanel = q;
    };
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            const int bad = *(const volatile int*)(tc.ctr + 2);
            s_item = bad ? -1 - bad : atomicAdd(tc.ctr, 1);
        }
        __syncthreads();
        const int idx = s_item;
        if (idx < 0) return -1 - idx;  // another block found the failing column
        if (idx >= total) break;
        const TeamItem itm = team_item(P, idx);
        const int p = itm.p, bi = itm.bi, bj = itm.bj;
        if (itm.kind == 0) {
            // F(p): for p >= 1 the panel block (p, p-1) and the last update of
            // the diagonal block (the arithmetic of R(p-1, p) and T(p-1, p, p)),
            // then the factor and inverse of the diagonal block (D(p)).
            const int nb = rows_of(p);
            const int w = p >= 1 ? team_wait_states(tc, team_state(tc, p - 1, p - 1), p, team_state(tc, p, p - 1), p - 1,
                                                    team_state(tc, p, p), p - 1)
                                 : team_wait_states(tc, nullptr, 0, nullptr, 0, nullptr, 0);
            if (w) return w;
            if (p >= 1) {
                const int q = p - 1, nq = rows_of(q);
                panel_inverse(q, nq);
                team_load_block(W1, A, lda, W32, ldw, W32 && q == 0, kPanel * p, kPanel * q, nb, nq, false);
                __syncthreads();
                team_apply_inverse(W1, X, nq);
                __syncthreads();
                team_store_block(W1, A, lda, W32, ldw, kPanel * p, kPanel * q, nb, nq, false);
                team_publish(team_state(tc, p, q), p);
                // S = lower(A_pp) - L_pq · L_pqᵀ, A_pp from the FP32 source on
                // its first touch (q == 0), in the T item's order.
                team_syrk_lower(S, W1, A, lda, W32, ldw, W32 && q == 0, kPanel * p, nb);
            } else {
                team_load_block(S, A, lda, W32, ldw, W32 != nullptr, 0, 0, nb, nb, true);
            }
            for (int e = threadIdx.x; e < 32 * 32; e += kThreads) {
                const int j = e >> 5, c = e & 31;
                X[j * 33 + c] = (j == c && j < nb) ? 1.0 : 0.0;
            }
            __syncthreads();
            const int info = team_factor_invert(nb, S, X, inv);
            if (info) {
                if (threadIdx.x == 0) {
                    atomicCAS(tc.ctr + 2, 0, kPanel * p + info);
                    *finisher = 1;
                }
                __syncthreads();
                return kPanel * p + info;
            }
            team_store_block(S, A, lda, W32, ldw, kPanel * p, kPanel * p, nb, nb, true);
            if (keep_x)
                for (int e = threadIdx.x; e < 32 * 32; e += kThreads) {
                    const int r = e & 31, c = e >> 5;
                    A[team_xoff(n, lda, p * 1024 + e)] = X[r * 33 + c];
                }
            // With the inverse kept, every R item uses these same bits; else
            // every R item recomputes it (the same way, whichever block).
            if (threadIdx.x == 0) s_xpanel = keep_x ? p : -1;
            team_publish(team_state(tc, p, p), p + 1);
        } else if (itm.kind == 1) {
            // R(p, bi): panel block (bi, p) <- A_ip · L_pp⁻ᵀ = A_ip · Xᵀ.
            const int nb = rows_of(p), rb = rows_of(bi);
            const int w = team_wait_states(tc, team_state(tc, p, p), p + 1, team_state(tc, bi, p), p, nullptr, 0);
            if (w) return w;
            panel_inverse(p, nb);
            team_load_block(W1, A, lda, W32, ldw, W32 && p == 0, kPanel * bi, kPanel * p, rb, nb, false);
            __syncthreads();
            team_apply_inverse(W1, X, nb);
            __syncthreads();
            team_store_block(W1, A, lda, W32, ldw, kPanel * bi, kPanel * p, rb, nb, false);
            team_publish(team_state(tc, bi, p), p + 1);
        } else {
            // T(p, bi, bj): A_ij -= L_ip · L_jpᵀ (lower part of a diagonal block).
            const int ri = rows_of(bi), rj = rows_of(bj);
            const int w = team_wait_states(tc, team_state(tc, bi, p), p + 1, team_state(tc, bj, p), p + 1,
                                           team_state(tc, bi, bj), p);
            if (w) return w;
            team_load_block(W1, A, lda, nullptr, 0, false, kPanel * bi, kPanel * p, ri, kPanel, false);
            team_load_block(W2, A, lda, nullptr, 0, false, kPanel * bj, kPanel * p, rj, kPanel, false);
            __syncthreads();
            const bool diag = bi == bj;
            const bool wide = W32 && p == 0;
            const int r = threadIdx.x & 31, g = threadIdx.x >> 5;
            const int gi = kPanel * bi + r;
            double cv[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int j = g + 8 * k, gj = kPanel * bj + j;
                const bool ok = r < ri && j < rj && (!diag || r >= j);
                cv[k] = !ok ? 0.0 : (wide ? (double)__ldcg(W32 + gi + (size_t)gj * ldw) : ldcg(A + gi + (size_t)gj * lda));
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int j = g + 8 * k, gj = kPanel * bj + j;
                if (r < ri && j < rj && (!diag || r >= j)) {
                    double a = 0.0;
#pragma unroll 8
                    for (int c = 0; c < kPanel; ++c) a = fma(W1[r * 33 + c], W2[j * 33 + c], a);
                    A[gi + (size_t)gj * lda] = cv[k] - a;
                }
            }
            team_publish(team_state(tc, bi, bj), p + 1);
        }
        if (threadIdx.x == 0 && atomicAdd(tc.ctr + 1, 1) == total - 1) *finisher = 1;
    }
    return 0;
}

}  // namespace ttg
