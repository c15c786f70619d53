// solve_kernels.cuh — device kernels of the triangular solves, the FP64
// residual and the Krylov vector operations (ttg_solve.cu).
//
// Layouts: factor tiles are the Cholesky plan's packed lower tiles (tile
// (i,j) at off[i + j*nb], column-major, ld = bs[i]); block vectors X are
// N × nrhs column-major (ld = N); the dense copy of A is N × N column-major.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "tile_f64.cuh"

namespace ttg {
namespace solve {

constexpr int kMaxRhs = 16;
constexpr int kRows = 32;  // output rows per work item of the sweeps

struct TileLayout {
    const int64_t* off;  // [nb*nb]
    const int* bs;       // [nb]
    const int* displ;    // [nb+1]
    int nb;
    int N;
};

// ------------------------------------------------------------------------
// Block triangular sweeps as a dataflow over row strips.
//
// Forward (L Y = R): for block rows i = 0..nb-1 in turn, Y_i = L_ii⁻¹ R_i
// (the "diagonal" items, one per 64-row strip of block row i), then
// R_k -= L_ki Y_i for every k > i (the "update" items, one per strip of each
// block row k).  Backward (Lᵀ X = Y) runs i = nb-1..0 with X_i = L_ii⁻ᵀ Y_i
// and Y_j -= L_ijᵀ X_i for j < i.  Every item is the same operation
//     out[strip] (=, or -=) M[strip rows, 0:kc] · V[0:kc, 0:nrhs]
// on a column-major operand: L_ii⁻¹ (forward diagonal), L_ki (forward
// update), L_ii⁻ᵀ (backward diagonal) and the transposed off-diagonal tiles
// L_ijᵀ (backward update), so every operand is read with coalesced column
// segments.
//
// Items are claimed from one counter in processing order: step by step, the
// diagonal items first, then the update items, the strips nearest the
// diagonal (which the next step's diagonal items wait for) first.  Each item
// waits for exactly what it reads: a diagonal item
// of step s for every strip of its block row to have received s updates, an
// update item for the step's diagonal items and for its own strip to have
// received the s earlier updates.  Everything an item waits for was claimed
// before it by a block that is running, so the sweep cannot deadlock, needs no
// grid-wide barrier and no co-residency guarantee, and applies the updates of
// every strip in step order (the result is deterministic).  Waits are bounded.
constexpr int kStrip = 64;    // output rows per item
constexpr int kChunk = 512;   // operand columns staged per pass

struct SweepArgs {
    const int64_t* off;        // packed tile offsets [nb*nb]
    const int64_t* doff;       // compact diagonal tile offsets [nb]
    const int* bs;             // [nb]
    const int* displ;          // [nb+1]
    const int* strip_pre;      // [nb+1] strips before each block row
    const int* step_start;     // [nb+1] items before each step
    int nb, N, nrhs, backward;
    int* applied;              // per strip: updates applied
    int* ready;                // per block row: diagonal strips done
    int* claim;                // item counter
    int* err;                  // nonzero after a timeout
    long long timeout_ns;
    long long* trace;          // per item: claimed, inputs ready, done (ns), SM; nullptr = off
    // Folded form (FP32 factors): the update of a block row by the row
    // processed just before it is folded into W_i = Md_i · Mu(i, prev), so a
    // step's critical chain is one item.  zready[i]: Z items of row i done.
    int fold;
    const int64_t* woff;       // [nb] offset of W_i in Wd (ld bs[i])
    int* zready;               // [nb]
    // The TMA sweep's claim order (folded form): claim k takes item
    // order[k] (an index in step order); null in the other sweeps.
    const int* order;
};

__device__ __forceinline__ long long sweep_clock() {
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Shared memory of a sweep block: the staged vector chunk (kChunk × kMaxRhs
// T, reused for the warp partials).
template <class T, class TM>
__host__ __device__ constexpr int sweep_smem_bytes() {
    return kChunk * kMaxRhs * (int)sizeof(T);
}

// out[0:rows, q] (mode 0: =, 1: -=) Σ_c M[r + c·ldm] · V[c + q·ldv], rows <=
// kStrip, on the whole block (256 threads).  Warp w takes columns w, w+8, ...
// of each staged chunk, lane l rows 2l and 2l+1; the eight warp partials are
// added in warp order.
//
// An item is a chain of memory round trips unless many loads are in flight:
// V is staged kStage values per thread at a time, with FP32 operands the
// next U columns of M are loaded while the current U are used (FP64
// accumulators leave no registers for that), and the output rows are read
// together before they are written.
template <class T, class TM>
__device__ void strip_gemv(int rows, int kc, const TM* __restrict__ M, int ldm, const T* V, int ldv, int nrhs, T* out,
                           int ldo, int mode, unsigned char* smem_raw) {
    constexpr int U = 8;
    constexpr int kStage = sizeof(T) == 4 ? 16 : 4;
    T* smem = reinterpret_cast<T*>(smem_raw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ra = 2 * lane, rb = 2 * lane + 1;
    const bool oka = ra < rows, okb = rb < rows;
    T acc0[kMaxRhs], acc1[kMaxRhs];
#pragma unroll
    for (int q = 0; q < kMaxRhs; ++q) acc0[q] = acc1[q] = T(0);
    for (int c0 = 0; c0 < kc; c0 += kChunk) {
        const int kcc = min(kChunk, kc - c0);
        const int total = kcc * kMaxRhs;
        __syncthreads();
        for (int e0 = threadIdx.x; e0 < total; e0 += (int)blockDim.x * kStage) {
            T tmp[kStage];
#pragma unroll
            for (int j = 0; j < kStage; ++j) {
                const int e = e0 + j * (int)blockDim.x;
                const int c = e % kcc, q = e / kcc;
                tmp[j] = (e < total && q < nrhs) ? ldcg(V + (c0 + c) + (size_t)q * ldv) : T(0);
            }
#pragma unroll
            for (int j = 0; j < kStage; ++j) {
                const int e = e0 + j * (int)blockDim.x;
                if (e < total) smem[(e % kcc) * kMaxRhs + e / kcc] = tmp[j];
            }
        }
        __syncthreads();
        const TM* Mc = M + (size_t)c0 * ldm;
        TM ma[U], mb[U];
        auto load = [&](int cb, TM(&xa)[U], TM(&xb)[U]) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int c = cb + 8 * u;
                xa[u] = (c < kcc && oka) ? Mc[ra + (size_t)c * ldm] : TM(0);
                xb[u] = (c < kcc && okb) ? Mc[rb + (size_t)c * ldm] : TM(0);
            }
        };
        auto use = [&](int cb) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int c = cb + 8 * u;
                if (c < kcc) {
                    const T* v = smem + c * kMaxRhs;
                    const T a = (T)ma[u], b = (T)mb[u];
#pragma unroll
                    for (int q = 0; q < kMaxRhs; ++q) {
                        const T vq = v[q];
                        acc0[q] = fma(a, vq, acc0[q]);
                        acc1[q] = fma(b, vq, acc1[q]);
                    }
                }
            }
        };
        if constexpr (sizeof(T) == 4) {
            load(warp, ma, mb);
            for (int cb = warp; cb < kcc; cb += 8 * U) {
                TM na[U], nb[U];
                load(cb + 8 * U, na, nb);
                use(cb);
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    ma[u] = na[u];
                    mb[u] = nb[u];
                }
            }
        } else {
            for (int cb = warp; cb < kcc; cb += 8 * U) {
                load(cb, ma, mb);
                use(cb);
            }
        }
    }
    // Warp partials: smem[(w·kMaxRhs + q)·kStrip + r].
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kMaxRhs; ++q) {
        smem[(warp * kMaxRhs + q) * kStrip + ra] = acc0[q];
        smem[(warp * kMaxRhs + q) * kStrip + rb] = acc1[q];
    }
    __syncthreads();
    constexpr int kOut = kStrip * kMaxRhs / 256;  // outputs per thread
    T prev[kOut];
#pragma unroll
    for (int j = 0; j < kOut; ++j) {
        const int e = threadIdx.x + j * (int)blockDim.x;
        const int r = e % kStrip, q = e / kStrip;
        prev[j] = (mode != 0 && r < rows && q < nrhs) ? ldcg(out + r + (size_t)q * ldo) : T(0);
    }
#pragma unroll
    for (int j = 0; j < kOut; ++j) {
        const int e = threadIdx.x + j * (int)blockDim.x;
        const int r = e % kStrip, q = e / kStrip;
        if (r >= rows || q >= nrhs) continue;
        T sum = T(0);
#pragma unroll
        for (int w = 0; w < 8; ++w) sum += smem[(w * kMaxRhs + q) * kStrip + r];
        out[r + (size_t)q * ldo] = mode == 0 ? sum : prev[j] - sum;
    }
}

// ------------------------------------------------------------------------
// Double-float arithmetic for the FP64 Krylov variant: a value is the
// unevaluated sum hi + lo of two floats.  Products of the high parts are
// split exactly with an FMA (Dekker's two-product), sums with Knuth's
// two-sum; the small cross terms are added in FP32.  Relative accuracy is
// about 2^-46 per operation at FP32 instruction rates (64 times the FP64
// rate of GB300).  The _rn intrinsics keep the compiler from contracting the
// error-free steps into FMAs.
__device__ __forceinline__ void df_split(double x, float& hi, float& lo) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(x - (double)hi);
}

// (sh, sl) += (ah + al)·(xh + xl).
__device__ __forceinline__ void df_fma(float ah, float al, float xh, float xl, float& sh, float& sl) {
    const float p = __fmul_rn(ah, xh);
    float e = fmaf(ah, xh, -p);
    e = fmaf(ah, xl, e);
    e = fmaf(al, xh, e);
    const float s = __fadd_rn(sh, p);
    const float z = __fsub_rn(s, sh);
    const float t = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, z)), __fsub_rn(p, z));
    sl = __fadd_rn(sl, __fadd_rn(t, e));
    sh = s;
}

// (sh, sl) += a·(xh + xl) for an FP32 a.
__device__ __forceinline__ void df_fma1(float a, float xh, float xl, float& sh, float& sl) {
    const float p = __fmul_rn(a, xh);
    float e = fmaf(a, xh, -p);
    e = fmaf(a, xl, e);
    const float s = __fadd_rn(sh, p);
    const float z = __fsub_rn(s, sh);
    const float t = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, z)), __fsub_rn(p, z));
    sl = __fadd_rn(sl, __fadd_rn(t, e));
    sh = s;
}

// (sh, sl) <- the same value with |sl| <= ulp(sh)/2 (fast two-sum).
__device__ __forceinline__ void df_renorm(float& sh, float& sl) {
    const float s = __fadd_rn(sh, sl);
    sl = __fsub_rn(sl, __fsub_rn(s, sh));
    sh = s;
}

// strip_gemv for FP64 vectors and an FP32 factor in double-float arithmetic:
// out[0:rows, q] (mode 0: =, 1: -=) Σ_c M[r + c·ldm] · V[c + q·ldv].  The
// same thread layout as strip_gemv; V is staged as (hi, lo) float pairs.
__device__ void strip_gemv_df(int rows, int kc, const float* __restrict__ M, int ldm, const double* V, int ldv, int nrhs,
                              double* out, int ldo, int mode, unsigned char* smem_raw) {
    float* vh = reinterpret_cast<float*>(smem_raw);   // [kChunk][kMaxRhs]
    float* vl = vh + kChunk * kMaxRhs;                  // [kChunk][kMaxRhs]
    double* part = reinterpret_cast<double*>(smem_raw);  // warp partials (after the chunks)
    constexpr int kStage = 8;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ra = 2 * lane, rb = 2 * lane + 1;
    const bool oka = ra < rows, okb = rb < rows;
    float h0[kMaxRhs], l0[kMaxRhs], h1[kMaxRhs], l1[kMaxRhs];
#pragma unroll
    for (int q = 0; q < kMaxRhs; ++q) h0[q] = l0[q] = h1[q] = l1[q] = 0.0f;
    for (int c0 = 0; c0 < kc; c0 += kChunk) {
        const int kcc = min(kChunk, kc - c0);
        const int total = kcc * kMaxRhs;
        __syncthreads();
        for (int e0 = threadIdx.x; e0 < total; e0 += (int)blockDim.x * kStage) {
            double tmp[kStage];
#pragma unroll
            for (int j = 0; j < kStage; ++j) {
                const int e = e0 + j * (int)blockDim.x;
                const int c = e % kcc, q = e / kcc;
                tmp[j] = (e < total && q < nrhs) ? ldcg(V + (c0 + c) + (size_t)q * ldv) : 0.0;
            }
#pragma unroll
            for (int j = 0; j < kStage; ++j) {
                const int e = e0 + j * (int)blockDim.x;
                if (e < total) {
                    float hi, lo;
                    df_split(tmp[j], hi, lo);
                    vh[(e % kcc) * kMaxRhs + e / kcc] = hi;
                    vl[(e % kcc) * kMaxRhs + e / kcc] = lo;
                }
            }
        }
        __syncthreads();
        const float* Mc = M + (size_t)c0 * ldm;
        // The factor values of the next U columns are loaded while the
        // current U are used (a column is ~350 instructions per thread, so U
        // columns cover the memory latency).
        constexpr int U = 4;
        float ca[U], cb[U];
        auto load = [&](int cbase, float(&xa)[U], float(&xb)[U]) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int c = cbase + 8 * u;
                xa[u] = (c < kcc && oka) ? Mc[ra + (size_t)c * ldm] : 0.0f;
                xb[u] = (c < kcc && okb) ? Mc[rb + (size_t)c * ldm] : 0.0f;
            }
        };
        load(warp, ca, cb);
        for (int cbase = warp; cbase < kcc; cbase += 8 * U) {
            float na[U], nb[U];
            load(cbase + 8 * U, na, nb);
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int c = cbase + 8 * u;
                if (c < kcc) {
                    const float* xh = vh + c * kMaxRhs;
                    const float* xl = vl + c * kMaxRhs;
#pragma unroll
                    for (int q = 0; q < kMaxRhs; ++q) {
                        df_fma1(ca[u], xh[q], xl[q], h0[q], l0[q]);
                        df_fma1(cb[u], xh[q], xl[q], h1[q], l1[q]);
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                ca[u] = na[u];
                cb[u] = nb[u];
            }
        }
#pragma unroll
        for (int q = 0; q < kMaxRhs; ++q) {
            df_renorm(h0[q], l0[q]);
            df_renorm(h1[q], l1[q]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kMaxRhs; ++q) {
        part[(warp * kMaxRhs + q) * kStrip + ra] = (double)h0[q] + (double)l0[q];
        part[(warp * kMaxRhs + q) * kStrip + rb] = (double)h1[q] + (double)l1[q];
    }
    __syncthreads();
    constexpr int kOut = kStrip * kMaxRhs / 256;
    double prev[kOut];
#pragma unroll
    for (int j = 0; j < kOut; ++j) {
        const int e = threadIdx.x + j * (int)blockDim.x;
        const int r = e % kStrip, q = e / kStrip;
        prev[j] = (mode != 0 && r < rows && q < nrhs) ? ldcg(out + r + (size_t)q * ldo) : 0.0;
    }
#pragma unroll
    for (int j = 0; j < kOut; ++j) {
        const int e = threadIdx.x + j * (int)blockDim.x;
        const int r = e % kStrip, q = e / kStrip;
        if (r >= rows || q >= nrhs) continue;
        double sum = 0.0;
#pragma unroll
        for (int w = 0; w < 8; ++w) sum += part[(w * kMaxRhs + q) * kStrip + r];
        out[r + (size_t)q * ldo] = mode == 0 ? sum : prev[j] - sum;
    }
}

// Largest idx with tab[idx] <= v (tab ascending, tab[0] = 0 <= v).
__device__ __forceinline__ int upper_index(const int* tab, int n, int v) {
    int lo = 0, hi = n;  // tab[lo] <= v < tab[hi] (tab[n] > v)
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (tab[mid] <= v) lo = mid;
        else hi = mid;
    }
    return lo;
}

// One sweep.  Forward: Vin = R (updated in place), Vout = Y, Mu = the factor
// tiles, Md = L_ii⁻¹ (compact diagonal).  Backward: Vin = Y (updated in
// place), Vout = X, Mu = the transposed tiles (L_ijᵀ at off[i + j·nb], ld
// bs[j]), Md = L_ii⁻ᵀ.
//
// Folded form (a.fold, Wd = W_i at woff[i]): with i the row of step s, p the
// row of step s-1 and n the row of step s+1, a step's items are
//   D  (strips of i)  s = 0: Vout_i = Md_i · Vin_i;  s >= 1: Vout_i -= W_i · Vout_p,
//                     where Vout_i already holds Z_i (ready[i]++);
//   Z  (strips of n)  Vout_n = Md_n · Vin_n, Vin_n holding the updates of steps
//                     0 .. s-1 (zready[n]++);
//   U  (strips of the rows after n)  Vin_k -= Mu(k, i) · Vout_i (applied = s+1).
// The update of n by i never runs: it is W_n · Vout_i inside n's D items.
template <class T, class TM>
__global__ void __launch_bounds__(256) sweep_kernel(SweepArgs a, const TM* __restrict__ Mu, const TM* __restrict__ Md,
                                                    const TM* __restrict__ Wd, T* Vin, T* Vout) {
    extern __shared__ __align__(16) unsigned char sweep_smem[];
    unsigned char* smem = sweep_smem;
    __shared__ int s_item, s_abort;
    const int nb = a.nb, N = a.N;
    const int total = a.step_start[nb];
    auto row_of = [&](int step) { return a.backward ? nb - 1 - step : step; };
    auto strips = [&](int row) { return a.strip_pre[row + 1] - a.strip_pre[row]; };
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(a.claim, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= total) break;
        if (a.trace && threadIdx.x == 0) a.trace[4 * (size_t)it] = sweep_clock();
        const int s = upper_index(a.step_start, nb, it);
        const int i = row_of(s);
        int u = it - a.step_start[s];
        const int Si = strips(i);
        // kind 0: diagonal (D), 1: next row's Z (folded form), 2: update (U).
        int kind, k, g;  // target block row and its global strip
        if (u < Si) {
            kind = 0;
            k = i;
            g = a.strip_pre[i] + u;
        } else {
            u -= Si;
            const int nx = s + 1 < nb ? row_of(s + 1) : -1;
            const int Sn = (a.fold && nx >= 0) ? strips(nx) : 0;
            if (u < Sn) {
                kind = 1;
                k = nx;
                g = a.strip_pre[nx] + u;
            } else {
                u -= Sn;
                kind = 2;
                // Strips of the rows after i (folded: after n), nearest first.
                const int skip = a.fold ? 1 : 0;
                g = a.backward ? a.strip_pre[i - skip] - 1 - u : a.strip_pre[i + 1 + skip] + u;
                k = upper_index(a.strip_pre, nb, g);
            }
        }
        const int p = s > 0 ? row_of(s - 1) : -1;
        // Wait for the inputs of this item.
        if (threadIdx.x == 0) {
            int abort = 0;
            const long long t0 = sweep_clock();
            unsigned spin = 0;
            for (;;) {
                bool ok = true;
                if (kind == 0) {
                    if (a.fold) {
                        if (s > 0)
                            ok = *(const volatile int*)(a.zready + i) >= Si && *(const volatile int*)(a.ready + p) >= strips(p);
                    } else {
                        for (int h = a.strip_pre[i]; h < a.strip_pre[i + 1] && ok; ++h)
                            ok = *(const volatile int*)(a.applied + h) >= s;
                    }
                } else if (kind == 1) {
                    for (int h = a.strip_pre[k]; h < a.strip_pre[k + 1] && ok; ++h) ok = *(const volatile int*)(a.applied + h) >= s;
                } else {
                    ok = *(const volatile int*)(a.ready + i) >= Si && *(const volatile int*)(a.applied + g) >= s;
                }
                if (ok) break;
                if ((++spin & 63) == 0) {
                    if (*(const volatile int*)a.err) {
                        abort = 1;
                        break;
                    }
                    if (sweep_clock() - t0 > a.timeout_ns) {
                        atomicCAS(a.err, 0, 1);
                        abort = 1;
                        break;
                    }
                }
                __nanosleep(32);
            }
            __threadfence();
            s_abort = abort;
            if (a.trace) a.trace[4 * (size_t)it + 1] = sweep_clock();
        }
        __syncthreads();
        if (s_abort) break;
        const int bk = a.bs[k], bi = a.bs[i];
        const int r0 = (g - a.strip_pre[k]) * kStrip;
        const int rows = min(kStrip, bk - r0);
        // FP64 vectors with an FP32 factor (the FP64 Krylov variant) are
        // swept in double-float arithmetic.
        auto gemv = [&](int rws, int kc, const TM* M, int ldm, const T* V, T* o, int mode) {
            if constexpr (sizeof(T) == 8 && sizeof(TM) == 4)
                strip_gemv_df(rws, kc, M, ldm, V, N, a.nrhs, o, N, mode, smem);
            else
                strip_gemv<T, TM>(rws, kc, M, ldm, V, N, a.nrhs, o, N, mode, smem);
        };
        if (kind == 0) {
            if (a.fold && s > 0)
                gemv(rows, a.bs[p], Wd + a.woff[i] + r0, bi, Vout + a.displ[p], Vout + a.displ[i] + r0, 1);
            else
                gemv(rows, bi, Md + a.doff[i] + r0, bi, Vin + a.displ[i], Vout + a.displ[i] + r0, 0);
        } else if (kind == 1) {
            gemv(rows, bk, Md + a.doff[k] + r0, bk, Vin + a.displ[k], Vout + a.displ[k] + r0, 0);
        } else {
            const int64_t o = a.backward ? a.off[i + (size_t)k * nb] : a.off[k + (size_t)i * nb];
            gemv(rows, bi, Mu + o + r0, bk, Vout + a.displ[i], Vin + a.displ[k] + r0, 1);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            if (kind == 0) atomicAdd(a.ready + i, 1);
            else if (kind == 1) atomicAdd(a.zready + k, 1);
            else atomicExch(a.applied + g, s + 1);
            if (a.trace) {
                unsigned sm;
                asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
                a.trace[4 * (size_t)it + 2] = sweep_clock();
                a.trace[4 * (size_t)it + 3] = sm;
            }
        }
    }
}

// W_i = A_i · B_i for the folded sweeps (column-major, NN): block (t, q)
// computes part q of gridDim.y of product t.
struct WdDesc {
    int64_t a, b, c;  // offsets into A, B, C
    int m, n, k;      // C is m×n (ld m), A m×k (ld m), B k×n (ld k)
};

template <class TM>
__global__ void wd_gemm_kernel(const WdDesc* __restrict__ d, const TM* A, const TM* B, TM* C) {
    extern __shared__ __align__(16) unsigned char wd_smem[];
    const WdDesc w = d[blockIdx.x];
    gemm_tile<TM, true, false>(w.m, w.n, w.k, TM(1), A + w.a, w.m, B + w.b, w.k, TM(0), C + w.c, w.m,
                               reinterpret_cast<TM*>(wd_smem), blockIdx.y, gridDim.y);
}

// Transposes of tiles: dst[doff_t + c + r·rows_t] = src[soff_t + r + c·rows_t]
// for the tiles of a descriptor list (rows × cols each, column-major source
// with ld rows, column-major destination with ld cols).  Block = 64×4
// threads over 64×64 sub-tiles (16 loads in flight per thread, one
// descriptor search per sub-tile); sub_pre[t] = sub-tiles before tile t.
struct TransposeDesc {
    int64_t src, dst;
    int rows, cols;
};
constexpr int kTrEdge = 64;

template <class TM>
__global__ void __launch_bounds__(256) transpose_tiles(const TransposeDesc* __restrict__ d, const int64_t* __restrict__ sub_pre,
                                                       int n_desc, const TM* __restrict__ src, TM* __restrict__ dst) {
    constexpr int E = kTrEdge, K = E / 4;
    __shared__ TM t[E][E + 1];
    const int64_t total = sub_pre[n_desc];
    const int tx = threadIdx.x & (E - 1), ty = threadIdx.x / E;
    for (int64_t b = blockIdx.x; b < total; b += gridDim.x) {
        int lo = 0, hi = n_desc;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (sub_pre[mid] <= b) lo = mid;
            else hi = mid;
        }
        const TransposeDesc td = d[lo];
        const int64_t sb = b - sub_pre[lo];
        const int nbr = (td.rows + E - 1) / E;
        const int br = (int)(sb % nbr), bc = (int)(sb / nbr);
        const int r = br * E + tx;
        TM v[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int c = bc * E + ty + 4 * k;
            v[k] = (r < td.rows && c < td.cols) ? src[td.src + r + (int64_t)c * td.rows] : TM(0);
        }
        __syncthreads();  // the previous sub-tile's reads of t are done
#pragma unroll
        for (int k = 0; k < K; ++k) t[ty + 4 * k][tx] = v[k];
        __syncthreads();
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int c = bc * E + tx, rr = br * E + ty + 4 * k;  // destination (c, rr) in a cols × rows tile
            if (rr < td.rows && c < td.cols) dst[td.dst + c + (int64_t)rr * td.cols] = t[tx][ty + 4 * k];
        }
    }
}

// invT of every diagonal tile: the right-side TRSM of the identity gives
// I·L^-T = L^-T, stored at doff[j] (ld bs[j]).  Grid (nb, parts): block (j, p)
// handles a row slice.
template <class TM>
__global__ void invert_diag_tiles(TileLayout lay, const int64_t* doff, const TM* L, TM* invT, int parts) {
    extern __shared__ __align__(128) double smem_inv[];
    const int j = blockIdx.x, p = blockIdx.y;
    const int b = lay.bs[j];
    if (b == 0) return;
    const TM* Ljj = L + lay.off[j + (size_t)j * lay.nb];
    TM* T = invT + doff[j];
    const int per = ((b + parts - 1) / parts + 15) / 16 * 16;
    const int r0 = min(b, p * per), r1 = min(b, r0 + per);
    for (long e = threadIdx.x; e < (long)(r1 - r0) * b; e += blockDim.x) {
        const int r = r0 + (int)(e % (r1 - r0)), c = (int)(e / (r1 - r0));
        T[r + (size_t)c * b] = r == c ? TM(1) : TM(0);
    }
    __syncthreads();
    trsm_rltn_tile<TM>(b, b, TM(1), Ljj, b, T, b, reinterpret_cast<TM*>(smem_inv), p, parts);
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

// Y = A X partials for FP32 (the FP32 Krylov matvec): a block takes 1024
// rows and one K split; thread (warp w, lane l) owns rows 128w + 4l .. +3 of
// the block and all 16 right-hand sides (64 accumulators), reading its four
// rows of a column with one 16-byte load (scalar loads when N % 4 != 0) and
// the staged X row as four 16-byte shared-memory loads: 64 FMAs per column
// against 5 loads.  The next kMmU columns are loaded while the current are
// used.  Partials P[split] are added by reduce_partials in a fixed order.
constexpr int kMmRows = 1024, kMmChunk = 256, kMmU = 4;
__global__ void __launch_bounds__(256, 2) dense_matmul_f32_partial(int N, const float* __restrict__ A, const float* __restrict__ X,
                                                                   int nrhs, float* P, int splits) {
    __shared__ __align__(16) float sX[kMmChunk * kMaxRhs];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r0 = blockIdx.x * kMmRows + warp * 128 + 4 * lane;
    const int sp = blockIdx.y;
    const int kper = (N + splits - 1) / splits;
    const int k0 = min(N, sp * kper), k1 = min(N, k0 + kper);
    const bool vec = (N & 3) == 0 && r0 + 3 < N;
    float acc[4][kMaxRhs];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < kMaxRhs; ++q) acc[i][q] = 0.0f;
    auto load_col = [&](int c) -> float4 {
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        const float* col = A + (size_t)c * N + r0;
        if (vec) {
            v = *reinterpret_cast<const float4*>(col);
        } else {
            if (r0 < N) v.x = col[0];
            if (r0 + 1 < N) v.y = col[1];
            if (r0 + 2 < N) v.z = col[2];
            if (r0 + 3 < N) v.w = col[3];
        }
        return v;
    };
    for (int c0 = k0; c0 < k1; c0 += kMmChunk) {
        const int kc = min(kMmChunk, k1 - c0);
        __syncthreads();
        {
            constexpr int kPer = kMmChunk * kMaxRhs / 256;
            float tmp[kPer];
#pragma unroll
            for (int j = 0; j < kPer; ++j) {
                const int e = threadIdx.x + 256 * j;
                const int c = e % kMmChunk, q = e / kMmChunk;
                tmp[j] = (c < kc && q < nrhs) ? __ldcg(X + (c0 + c) + (size_t)q * N) : 0.0f;
            }
#pragma unroll
            for (int j = 0; j < kPer; ++j) {
                const int e = threadIdx.x + 256 * j;
                sX[(e % kMmChunk) * kMaxRhs + e / kMmChunk] = tmp[j];
            }
        }
        __syncthreads();
        float4 cur[kMmU];
#pragma unroll
        for (int u = 0; u < kMmU; ++u) cur[u] = u < kc ? load_col(c0 + u) : make_float4(0.f, 0.f, 0.f, 0.f);
        for (int c = 0; c < kc; c += kMmU) {
            float4 nxt[kMmU];
#pragma unroll
            for (int u = 0; u < kMmU; ++u) nxt[u] = c + kMmU + u < kc ? load_col(c0 + c + kMmU + u) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int u = 0; u < kMmU; ++u) {
                if (c + u < kc) {
                    const float4* xv = reinterpret_cast<const float4*>(sX + (c + u) * kMaxRhs);
                    const float a[4] = {cur[u].x, cur[u].y, cur[u].z, cur[u].w};
#pragma unroll
                    for (int j = 0; j < kMaxRhs / 4; ++j) {
                        const float4 x = xv[j];
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            acc[i][4 * j + 0] = fmaf(a[i], x.x, acc[i][4 * j + 0]);
                            acc[i][4 * j + 1] = fmaf(a[i], x.y, acc[i][4 * j + 1]);
                            acc[i][4 * j + 2] = fmaf(a[i], x.z, acc[i][4 * j + 2]);
                            acc[i][4 * j + 3] = fmaf(a[i], x.w, acc[i][4 * j + 3]);
                        }
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < kMmU; ++u) cur[u] = nxt[u];
        }
    }
    float* out = P + (size_t)sp * N * nrhs;
#pragma unroll
    for (int q = 0; q < kMaxRhs; ++q) {
        if (q >= nrhs) break;
        if (vec) {
            *reinterpret_cast<float4*>(out + r0 + (size_t)q * N) = make_float4(acc[0][q], acc[1][q], acc[2][q], acc[3][q]);
        } else {
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if (r0 + i < N) out[r0 + i + (size_t)q * N] = acc[i][q];
        }
    }
}

// Y = A X partials in double-float arithmetic: A = Ah + Al (two FP32
// copies, Al = fl32(A - Ah)), X FP64 (split per staged chunk).  Grid (row
// blocks of 256, K splits); thread t takes rows 256·bx + (t & 127) and that
// + 128 for the right-hand sides 8·(t >> 7) .. +7, so each staged x pair
// (read as float4) serves two rows.  Partial sums of split y go to
// P[y·N·nrhs + ...] and are added by reduce_partials in a fixed order.
__global__ void __launch_bounds__(256) dense_matmul_df_partial(int N, const float* __restrict__ Ah, const float* __restrict__ Al,
                                                               const double* __restrict__ X, int nrhs, double* P, int splits) {
    constexpr int H = kMaxRhs / 2;
    __shared__ __align__(16) float sXh[128 * kMaxRhs], sXl[128 * kMaxRhs];
    const int rb = blockIdx.x, sp = blockIdx.y;
    const int half = threadIdx.x >> 7;
    const int ra = rb * 256 + (threadIdx.x & 127), rbw = ra + 128;
    const bool oka = ra < N, okb = rbw < N;
    const int kper = (N + splits - 1) / splits;
    const int k0 = min(N, sp * kper), k1 = min(N, k0 + kper);
    float ha[H], la[H], hb[H], lb[H];
#pragma unroll
    for (int q = 0; q < H; ++q) ha[q] = la[q] = hb[q] = lb[q] = 0.0f;
    for (int c0 = k0; c0 < k1; c0 += 128) {
        const int kc = min(128, k1 - c0);
        __syncthreads();
        for (int e = threadIdx.x; e < 128 * kMaxRhs; e += blockDim.x) {
            const int c = e % 128, q = e / 128;
            float hi = 0.0f, lo = 0.0f;
            if (c < kc && q < nrhs) df_split(X[(c0 + c) + (size_t)q * N], hi, lo);
            sXh[c * kMaxRhs + q] = hi;
            sXl[c * kMaxRhs + q] = lo;
        }
        __syncthreads();
        // Column c + 1 of A is loaded while column c is used (the loads are
        // otherwise the main stall).
        auto load = [&](int c, float& ah_, float& al_, float& bh_, float& bl_) {
            const size_t col = (size_t)(c0 + c) * N;
            ah_ = oka ? Ah[ra + col] : 0.0f;
            al_ = oka ? Al[ra + col] : 0.0f;
            bh_ = okb ? Ah[rbw + col] : 0.0f;
            bl_ = okb ? Al[rbw + col] : 0.0f;
        };
        float nah = 0.0f, nal = 0.0f, nbh = 0.0f, nbl = 0.0f;
        if (kc > 0) load(0, nah, nal, nbh, nbl);
#pragma unroll 2
        for (int c = 0; c < kc; ++c) {
            const float aah = nah, aal = nal, abh = nbh, abl = nbl;
            if (c + 1 < kc) load(c + 1, nah, nal, nbh, nbl);
            const float4* xh4 = reinterpret_cast<const float4*>(sXh + c * kMaxRhs + half * H);
            const float4* xl4 = reinterpret_cast<const float4*>(sXl + c * kMaxRhs + half * H);
#pragma unroll
            for (int v = 0; v < H / 4; ++v) {
                const float4 xh = xh4[v], xl = xl4[v];
                const float xhs[4] = {xh.x, xh.y, xh.z, xh.w}, xls[4] = {xl.x, xl.y, xl.z, xl.w};
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int q = 4 * v + j;
                    df_fma(aah, aal, xhs[j], xls[j], ha[q], la[q]);
                    df_fma(abh, abl, xhs[j], xls[j], hb[q], lb[q]);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < H; ++q) {
            df_renorm(ha[q], la[q]);
            df_renorm(hb[q], lb[q]);
        }
    }
#pragma unroll
    for (int q = 0; q < H; ++q) {
        const int qq = half * H + q;
        if (qq < nrhs) {
            if (oka) P[(size_t)sp * N * nrhs + ra + (size_t)qq * N] = (double)ha[q] + (double)la[q];
            if (okb) P[(size_t)sp * N * nrhs + rbw + (size_t)qq * N] = (double)hb[q] + (double)lb[q];
        }
    }
}

// h = fl32(v) and l = fl32(v - h) (round to nearest even), bit for bit those
// of the FP64 formula, from integer operations on v's bits for 2^-60 <= |v|
// < 2^101: on this GPU FP64 arithmetic and conversions from FP64 run at the
// FP64 rate, 1/64 of the FP32 one.  The remainder v - h is the low 29
// mantissa bits (rounded down) or their complement to the next unit of h
// (rounded up), an integer times 2^(e-52), which the FP32 conversion rounds
// to nearest and an exact power-of-two scale places.  Other values (zero,
// tiny, huge, non-finite) take the FP64 formula.
// Also compiled for the host (ttg_split_f64_f32), where the bit casts are
// copies and the FP32 operations round to nearest as on the device.
__host__ __device__ __forceinline__ void split_f64_f32(double v, float& h, float& l) {
#ifdef __CUDA_ARCH__
    const unsigned hiw = (unsigned)__double2hiint(v), low = (unsigned)__double2loint(v);
    auto as_float = [](unsigned u) { return __uint_as_float(u); };
#else
    unsigned long long bits;
    memcpy(&bits, &v, sizeof bits);
    const unsigned hiw = (unsigned)(bits >> 32), low = (unsigned)bits;
    auto as_float = [](unsigned u) {
        float f;
        memcpy(&f, &u, sizeof f);
        return f;
    };
#endif
    const unsigned sign = hiw >> 31;
    const int ex = (int)((hiw >> 20) & 0x7FFu) - 1023;
    if (ex < -60 || ex > 100) {
        h = (float)v;
        l = (float)(v - (double)h);
        return;
    }
    const unsigned top = ((hiw & 0xFFFFFu) << 3) | (low >> 29);  // 23 mantissa bits of h before rounding
    const unsigned rem = low & 0x1FFFFFFFu;                       // the 29 bits below them
    const unsigned up = (rem > (1u << 28) || (rem == (1u << 28) && (top & 1u))) ? 1u : 0u;
    h = as_float(((sign << 31) | ((unsigned)(ex + 127) << 23) | top) + up);  // a carry moves to the exponent
    const unsigned rm = up ? (1u << 29) - rem : rem;
    // rm · 2^(e-52): rm has at most 29 bits, so the conversion rounds to
    // nearest once and the power-of-two scale is exact.
    const float lv = (float)rm * as_float((unsigned)(ex + 1023 - 948) << 23);
    l = rm == 0 ? 0.0f : ((sign ^ up) ? -lv : lv);
}

// Al = fl32(A - Ah): the low FP32 half of the dense copy.
__global__ void split_low_half(int64_t n, const double* __restrict__ A, float* __restrict__ Al) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        float h, l;
        split_f64_f32(A[e], h, l);
        Al[e] = l;
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

// ‖A‖∞: rowsum[r] = Σ_y part[y·N + r], added in order (the same value on
// every run).
__global__ void row_abs_final(int N, int splits, const double* __restrict__ part, double* rowsum) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < N; r += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int y = 0; y < splits; ++y) s += part[(size_t)y * N + r];
        rowsum[r] = s;
    }
}

// Dense N×N copies of the symmetric matrix held as packed lower tiles: FP64
// (A64), and when set its FP32 rounding (A32) and the FP32 rounding of the
// remainder (A32lo = fl32(A - A32), the low half of the double-float form),
// with the row sums of |A| by 64-column block: Q[j·N + r] = Σ_{c in block j}
// |A(r, c)|, each written once.  Work unit: a 64×64 sub-block of the lower
// triangle, read once with coalesced column segments (16 loads in flight per
// thread), written in place and, through a shared-memory transpose, at the
// mirrored position.  Block 64×4 threads; sub-block sb = R(R+1)/2 + C, R >= C.
constexpr int kDenseSb = 64;
__global__ void __launch_bounds__(256) dense_sym_from_tiles(TileLayout lay, const int* __restrict__ rowblk,
                                                            const double* __restrict__ tiles, double* __restrict__ A64,
                                                            float* __restrict__ A32, float* __restrict__ A32lo, double* __restrict__ Q) {
    constexpr int E = kDenseSb, K = E / 4;
    __shared__ double T[E][E + 1];   // T[a][b] = A(r0 + b, c0 + a)
    __shared__ double red[2][4][E];  // per-thread partial row sums: in place, mirrored
    const int N = lay.N;
    const int nsb = (N + E - 1) / E;
    const int64_t total = (int64_t)nsb * (nsb + 1) / 2;
    const int tx = threadIdx.x & (E - 1), ty = threadIdx.x / E;
    auto lower = [&](int gi, int gj) {  // element (gi, gj), gi >= gj, of the tiles
        const int bi = rowblk[gi], bj = rowblk[gj];
        return tiles[lay.off[bi + (size_t)bj * lay.nb] + (gi - lay.displ[bi]) + (int64_t)(gj - lay.displ[bj]) * lay.bs[bi]];
    };
    auto put = [&](size_t e, double v) {
        A64[e] = v;
        if (A32) {
            float h, l;
            split_f64_f32(v, h, l);
            A32[e] = h;
            if (A32lo) A32lo[e] = l;
        }
    };
    for (int64_t sb = blockIdx.x; sb < total; sb += gridDim.x) {
        int R = (int)((sqrt(8.0 * (double)sb + 1.0) - 1.0) * 0.5);
        while ((int64_t)R * (R + 1) / 2 > sb) --R;
        while ((int64_t)(R + 1) * (R + 2) / 2 <= sb) ++R;
        const int C = (int)(sb - (int64_t)R * (R + 1) / 2);
        const int r0 = E * R, c0 = E * C;
        // A sub-block inside one tile (the usual case) reads it with one base
        // offset and the tile's leading dimension.
        const int bi = rowblk[r0], bj = rowblk[c0];
        const bool one_tile = bi == rowblk[min(r0 + E - 1, N - 1)] && bj == rowblk[min(c0 + E - 1, N - 1)];
        const int ld = lay.bs[bi];
        const double* base = tiles + lay.off[bi + (size_t)bj * lay.nb] + (r0 - lay.displ[bi]) + (int64_t)(c0 - lay.displ[bj]) * ld;
        const int r = r0 + tx;
        double v[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int yy = ty + 4 * k, c = c0 + yy;
            v[k] = 0.0;
            if (r < N && c < N) {
                if (one_tile) v[k] = r >= c ? base[tx + (int64_t)yy * ld] : base[yy + (int64_t)tx * ld];
                else v[k] = r >= c ? lower(r, c) : lower(c, r);
            }
        }
        double pin = 0.0;
#pragma unroll
        for (int k = 0; k < K; ++k) pin += fabs(v[k]);
        __syncthreads();  // the previous sub-block's reads of T and red are done
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int yy = ty + 4 * k, c = c0 + yy;
            if (r < N && c < N) put(r + (size_t)c * N, v[k]);
            T[yy][tx] = v[k];
        }
        red[0][ty][tx] = pin;
        if (R != C) {  // a diagonal sub-block covered both triangles
            __syncthreads();
            double pm = 0.0;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const int yy = ty + 4 * k;
                const int rr = c0 + tx, cc = r0 + yy;  // mirrored element (c0 + tx, r0 + yy) = T[tx][yy]
                const double w = T[tx][yy];
                pm += fabs(w);
                if (rr < N && cc < N) put(rr + (size_t)cc * N, w);
            }
            red[1][ty][tx] = pm;
        }
        __syncthreads();
        if (Q) {
            const int m = threadIdx.x / E;  // 0: rows r0.. (column block C), 1: rows c0.. (column block R)
            if (m == 0 && r0 + tx < N)
                Q[(size_t)C * N + r0 + tx] = ((red[0][0][tx] + red[0][1][tx]) + red[0][2][tx]) + red[0][3][tx];
            else if (m == 1 && R != C && c0 + tx < N)
                Q[(size_t)R * N + c0 + tx] = ((red[1][0][tx] + red[1][1][tx]) + red[1][2][tx]) + red[1][3][tx];
        }
    }
}

}  // namespace solve
}  // namespace ttg
