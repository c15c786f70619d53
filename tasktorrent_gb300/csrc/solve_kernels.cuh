// solve_kernels.cuh — device kernels of the triangular solves, the FP64
// residual and the Krylov vector operations (ttg_solve.cu).
//
// Layouts: factor tiles are the Cholesky plan's packed lower tiles (tile
// (i,j) at off[i + j*nb], column-major, ld = bs[i]); block vectors X are
// N × nrhs column-major (ld = N); the dense copy of A is N × N column-major.
#pragma once
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "tile_f64.cuh"

namespace ttg {
namespace solve {

namespace cg = cooperative_groups;

constexpr int kMaxRhs = 16;
constexpr int kRows = 32;  // output rows per work item of the sweeps

struct TileLayout {
    const int64_t* off;  // [nb*nb]
    const int* bs;       // [nb]
    const int* displ;    // [nb+1]
    int nb;
    int N;
};

// Y[rows] = M · V, M row-major access through column-major storage: thread per
// output row, loop over columns (coalesced for column-major M).  M is m×k
// with leading dimension ldm; V is k×nrhs (ldv); Y is m×nrhs (ldy).
// Mode: 0 store, 1 subtract (Y -= M V).
template <class T, class TM>
__device__ void gemv_n_rows(int r0, int r1, int k, const TM* M, int ldm, const T* V, int ldv, T* Y, int ldy, int nrhs,
                            int mode, T* sV) {
    // Stage V (k × nrhs) through shared memory in chunks of 256 rows.
    for (int c0 = 0; c0 < k; c0 += 256) {
        const int kc = min(256, k - c0);
        __syncthreads();
        for (int e = threadIdx.x; e < kc * nrhs; e += blockDim.x) {
            const int c = e % kc, q = e / kc;
            sV[c + q * 256] = ldcg(V + (c0 + c) + (size_t)q * ldv);
        }
        __syncthreads();
        for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
            T acc[kMaxRhs];
#pragma unroll
            for (int q = 0; q < kMaxRhs; ++q) acc[q] = T(0);
            for (int c = 0; c < kc; ++c) {
                const T m = (T)ldcg(M + r + (size_t)(c0 + c) * ldm);
#pragma unroll
                for (int q = 0; q < kMaxRhs; ++q)
                    if (q < nrhs) acc[q] = fma(m, sV[c + q * 256], acc[q]);
            }
#pragma unroll
            for (int q = 0; q < kMaxRhs; ++q) {
                if (q >= nrhs) break;
                T* y = Y + r + (size_t)q * ldy;
                if (mode == 0) *y = (c0 == 0) ? acc[q] : ldcg(y) + acc[q];
                else *y = ldcg(y) - acc[q];
            }
        }
    }
}

// Y[rows] (op) Mᵀ · V: output row r is column r of M (contiguous): warp per
// output row, lanes over the column, shuffle reduction.  M is k×m (ldm).
template <class T, class TM>
__device__ void gemv_t_rows(int r0, int r1, int k, const TM* M, int ldm, const T* V, int ldv, T* Y, int ldy, int nrhs, int mode) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int r = r0 + warp; r < r1; r += nw) {
        T acc[kMaxRhs];
#pragma unroll
        for (int q = 0; q < kMaxRhs; ++q) acc[q] = T(0);
        const TM* col = M + (size_t)r * ldm;
        for (int c = lane; c < k; c += 32) {
            const T m = (T)ldcg(col + c);
#pragma unroll
            for (int q = 0; q < kMaxRhs; ++q)
                if (q < nrhs) acc[q] = fma(m, ldcg(V + c + (size_t)q * ldv), acc[q]);
        }
#pragma unroll
        for (int q = 0; q < kMaxRhs; ++q) {
            T v = acc[q];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            acc[q] = v;
        }
        if (lane < nrhs) {
            T v = acc[0];
#pragma unroll
            for (int q = 1; q < kMaxRhs; ++q)
                if (q == lane) v = acc[q];
            T* y = Y + r + (size_t)lane * ldy;
            *y = mode == 0 ? v : ldcg(y) - v;
        }
    }
}

// Forward sweep L Y = R (R is overwritten as scratch), with the transposed
// inverses of the diagonal tiles (invT: tile j at off[j + j*nb], ld = bs[j],
// holding L_jj^-T column-major).  One cooperative launch; grid syncs between
// the diagonal apply and the updates of each block row.
template <class T, class TM>
__global__ void sweep_forward(TileLayout lay, const TM* L, const TM* invT, T* R, T* Y, int nrhs) {
    cg::grid_group grid = cg::this_grid();
    __shared__ T sV[256 * kMaxRhs];
    const int N = lay.N;
    for (int i = 0; i < lay.nb; ++i) {
        const int bi = lay.bs[i], di = lay.displ[i];
        // Y_i = L_ii^-1 R_i = (invT)^T R_i: output row r is column r of invT.
        const TM* Ti = invT + lay.off[i + (size_t)i * lay.nb];
        const int items = (bi + kRows - 1) / kRows;
        for (int it = blockIdx.x; it < items; it += gridDim.x) {
            const int r0 = it * kRows, r1 = min(bi, r0 + kRows);
            gemv_t_rows<T, TM>(r0, r1, bi, Ti, bi, R + di, N, Y + di, N, nrhs, 0);
        }
        grid.sync();
        // R_k -= L_ki Y_i for k > i.
        long total = 0;
        for (int k = i + 1; k < lay.nb; ++k) total += (lay.bs[k] + kRows - 1) / kRows;
        for (long it = blockIdx.x; it < total; it += gridDim.x) {
            long rem = it;
            int k = i + 1;
            while (rem >= (lay.bs[k] + kRows - 1) / kRows) {
                rem -= (lay.bs[k] + kRows - 1) / kRows;
                ++k;
            }
            const int bk = lay.bs[k];
            const int r0 = (int)rem * kRows, r1 = min(bk, r0 + kRows);
            const TM* Lki = L + lay.off[k + (size_t)i * lay.nb];
            gemv_n_rows<T, TM>(r0, r1, bi, Lki, bk, Y + di, N, R + lay.displ[k], N, nrhs, 1, sV);
        }
        grid.sync();
    }
}

// Backward sweep Lᵀ X = Y (Y is overwritten as scratch).
template <class T, class TM>
__global__ void sweep_backward(TileLayout lay, const TM* L, const TM* invT, T* Yv, T* X, int nrhs) {
    cg::grid_group grid = cg::this_grid();
    __shared__ T sV[256 * kMaxRhs];
    const int N = lay.N;
    for (int i = lay.nb - 1; i >= 0; --i) {
        const int bi = lay.bs[i], di = lay.displ[i];
        // X_i = L_ii^-T Y_i = invT Y_i (thread per row).
        const TM* Ti = invT + lay.off[i + (size_t)i * lay.nb];
        const int items = (bi + kRows - 1) / kRows;
        for (int it = blockIdx.x; it < items; it += gridDim.x) {
            const int r0 = it * kRows, r1 = min(bi, r0 + kRows);
            gemv_n_rows<T, TM>(r0, r1, bi, Ti, bi, Yv + di, N, X + di, N, nrhs, 0, sV);
        }
        grid.sync();
        // Y_j -= L_ijᵀ X_i for j < i (output rows of block j are columns of L_ij).
        long total = 0;
        for (int j = 0; j < i; ++j) total += (lay.bs[j] + kRows - 1) / kRows;
        for (long it = blockIdx.x; it < total; it += gridDim.x) {
            long rem = it;
            int j = 0;
            while (rem >= (lay.bs[j] + kRows - 1) / kRows) {
                rem -= (lay.bs[j] + kRows - 1) / kRows;
                ++j;
            }
            const int bj = lay.bs[j];
            const int r0 = (int)rem * kRows, r1 = min(bj, r0 + kRows);
            const TM* Lij = L + lay.off[i + (size_t)j * lay.nb];
            gemv_t_rows<T, TM>(r0, r1, bi, Lij, bi, X + di, N, Yv + lay.displ[j], N, nrhs, 1);
        }
        grid.sync();
    }
}

// invT of every diagonal tile: the right-side TRSM of the identity gives
// I·L^-T = L^-T.  Grid (nb, parts): block (j, p) handles a row slice.
template <class TM>
__global__ void invert_diag_tiles(TileLayout lay, const TM* L, TM* invT, int parts) {
    extern __shared__ __align__(128) double smem_inv[];
    const int j = blockIdx.x, p = blockIdx.y;
    const int b = lay.bs[j];
    if (b == 0) return;
    const TM* Ljj = L + lay.off[j + (size_t)j * lay.nb];
    TM* T = invT + lay.off[j + (size_t)j * lay.nb];
    const int per = ((b + parts - 1) / parts + 15) / 16 * 16;
    const int r0 = min(b, p * per), r1 = min(b, r0 + per);
    for (long e = threadIdx.x; e < (long)(r1 - r0) * b; e += blockDim.x) {
        const int r = r0 + (int)(e % (r1 - r0)), c = (int)(e / (r1 - r0));
        T[r + (size_t)c * b] = r == c ? TM(1) : TM(0);
    }
    __syncthreads();
    trsm_rltn_tile<TM>(b, b, TM(1), Ljj, b, T, b, reinterpret_cast<TM*>(smem_inv), p, parts);
}

// Dense N×N column-major symmetric matrix from packed lower tiles (both
// triangles), converted to TD.  rowblk[r] is the block row of row r.
template <class TS, class TD>
__global__ void dense_from_tiles(TileLayout lay, const int* __restrict__ rowblk, const TS* tiles, TD* A) {
    const int N = lay.N;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)N * N; e += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(e % N), c = (int)(e / N);
        const int gi = r >= c ? r : c, gj = r >= c ? c : r;  // lower-triangle element (gi >= gj)
        const int bi = rowblk[gi], bj = rowblk[gj];
        const int li = gi - lay.displ[bi], lj = gj - lay.displ[bj];
        A[e] = (TD)tiles[lay.off[bi + (size_t)bj * lay.nb] + li + (int64_t)lj * lay.bs[bi]];
    }
}

// Y = A X (mode 0) or Y = B - A X (mode 2) for dense column-major A (N×N),
// X, B, Y N × nrhs.  Grid (row blocks of 128, K splits); partial sums of the
// K splits go to P[split] and are added by reduce_partials in a fixed order.
template <class T>
__global__ void dense_matmul_partial(int N, const T* __restrict__ A, const T* __restrict__ X, int nrhs, T* P, int splits) {
    __shared__ T sX[128 * kMaxRhs];
    const int rb = blockIdx.x, sp = blockIdx.y;
    const int r = rb * 128 + (threadIdx.x & 127);
    const int half = threadIdx.x >> 7;  // two threads per row: rhs halves
    const int kper = (N + splits - 1) / splits;
    const int k0 = sp * kper, k1 = min(N, k0 + kper);
    T acc[kMaxRhs / 2];
#pragma unroll
    for (int q = 0; q < kMaxRhs / 2; ++q) acc[q] = T(0);
    for (int c0 = k0; c0 < k1; c0 += 128) {
        const int kc = min(128, k1 - c0);
        __syncthreads();
        for (int e = threadIdx.x; e < kc * nrhs; e += blockDim.x) {
            const int c = e % kc, q = e / kc;
            sX[c + q * 128] = X[(c0 + c) + (size_t)q * N];
        }
        __syncthreads();
        if (r < N) {
            for (int c = 0; c < kc; ++c) {
                const T a = A[r + (size_t)(c0 + c) * N];
#pragma unroll
                for (int q = 0; q < kMaxRhs / 2; ++q) {
                    const int qq = half * (kMaxRhs / 2) + q;
                    if (qq < nrhs) acc[q] = fma(a, sX[c + qq * 128], acc[q]);
                }
            }
        }
    }
    if (r < N) {
#pragma unroll
        for (int q = 0; q < kMaxRhs / 2; ++q) {
            const int qq = half * (kMaxRhs / 2) + q;
            if (qq < nrhs) P[(size_t)sp * N * nrhs + r + (size_t)qq * N] = acc[q];
        }
    }
}

template <class T>
__global__ void reduce_partials(int N, int nrhs, const T* P, int splits, const T* B, T* Y, int mode) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)N * nrhs; e += (int64_t)gridDim.x * blockDim.x) {
        T s = T(0);
        for (int sp = 0; sp < splits; ++sp) s += P[(size_t)sp * N * nrhs + e];
        Y[e] = mode == 2 ? B[e] - s : s;
    }
}

// max that propagates NaN (fmax would drop it and hide a broken column).
__device__ __forceinline__ double nanmax(double a, double b) { return (a != a || b != b) ? __longlong_as_double(0x7ff8000000000000LL) : fmax(a, b); }

// Per-column reductions over N × nrhs blocks.  kind 0: dot(X, Y); 1: max|X|.
// Partials per block, then a fixed-order final pass (deterministic).
template <class T>
__global__ void column_reduce_partial(int N, int nrhs, const T* X, const T* Y, int kind, double* part) {
    __shared__ double red[256];
    for (int q = 0; q < nrhs; ++q) {
        double acc = 0.0;
        for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x) {
            const double x = (double)X[r + (size_t)q * N];
            if (kind == 0) acc += x * (double)Y[r + (size_t)q * N];
            else acc = nanmax(acc, fabs(x));
        }
        red[threadIdx.x] = acc;
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s) red[threadIdx.x] = kind == 0 ? red[threadIdx.x] + red[threadIdx.x + s] : nanmax(red[threadIdx.x], red[threadIdx.x + s]);
            __syncthreads();
        }
        if (threadIdx.x == 0) part[(size_t)q * gridDim.x + blockIdx.x] = red[0];
        __syncthreads();
    }
}

__global__ void column_reduce_final(int nrhs, int nparts, const double* part, int kind, double* out) {
    const int q = threadIdx.x;
    if (q >= nrhs) return;
    double acc = 0.0;
    for (int p = 0; p < nparts; ++p) acc = kind == 0 ? acc + part[(size_t)q * nparts + p] : nanmax(acc, part[(size_t)q * nparts + p]);
    out[q] = acc;
}

// Y[:, q] = a[q] * X[:, q] + b[q] * Y[:, q] with per-column coefficients
// (device arrays, double), any element types.
template <class TX, class TY>
__global__ void column_axpby(int N, int nrhs, const double* a, const TX* X, const double* b, TY* Y) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)N * nrhs; e += (int64_t)gridDim.x * blockDim.x) {
        const int q = (int)(e / N);
        const double y = b ? b[q] * (double)Y[e] : 0.0;
        Y[e] = (TY)(a[q] * (double)X[e] + y);
    }
}

// ‖A‖∞ of the symmetric matrix (max absolute row sum) from the dense copy.
template <class T>
__global__ void row_abs_sums(int N, const T* A, double* rowsum) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < N; r += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int c = 0; c < N; ++c) s += fabs((double)A[r + (size_t)c * N]);
        rowsum[r] = s;
    }
}

}  // namespace solve
}  // namespace ttg
