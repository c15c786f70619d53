// sliced_matmul_tc.cuh — Y = A·X with FP64 accuracy on the BF16 tensor
// cores, for the residuals r = b − A·x of the refinement (the FP64 product
// of 2d_cholesky.cpp:646-689's solve check, at N×16).
//
// Method: error-free slicing of both operands into small integers (Ozaki,
// Ogita, Oishi, Rump, "Error-free transformations of matrix multiplication by
// using fast routines of matrix multiplication", Numer. Algorithms 59, 2012).
//
//   Row i of A is scaled by σ_i = 2^E_i (|A_ij| < σ_i/2) and written as eight
//   signed base-256 digits, A_ij = σ_i (Σ_s a_s(i,j) 2^-8s + ε), |ε| < 2^-64,
//   each digit an integer in [-128, 128] (exact in BF16), cut from the FP64
//   bits with integer operations.  Column q of X the same with τ_q = 2^F_q:
//   X_jq = τ_q (Σ_t x_t(j,q) 2^-8t + ε').
//   (A X)_iq = σ_i τ_q Σ_d 2^-8d S_d(i,q),  S_d = Σ_{s+t=d} Σ_j a_s x_t,
//   kept for d = s + t ≤ 9 (the dropped pairs weigh ≤ 2^-72 of σ_i τ_q per
//   term).
//
// Exactness: a digit product is at most 2^14, a group d has at most eight
// (s, t) pairs, so 128 values of j sum to at most 2^24 in magnitude — every
// partial sum of the FP32 tensor-core accumulator is an integer below 2^24
// and therefore exact.  Each group is flushed to int64 registers every 128
// columns of A, so S_d is exact over any N; only the final combination
// Σ_d 2^-8d S_d (eight terms) and the scaling round, in FP64.
//
// The product on the tensor cores: for each A slice s, one
// tcgen05.mma.cta_group::1.kind::f16 with M = 128 rows of A (the A slice,
// K-major), N = 16·(9−s) columns (the X slices t = 1 … 9−s stacked, 16
// right-hand sides each) writes its pairs (s, t) straight into the TMEM
// columns of the groups d = s+1 … 9 — eight MMAs per K step of 16 cover all
// 36 pairs.  TMA loads (64B swizzle) bring per K slab of 32 the eight A
// slices (64 KB) and the X slices (8 KB) into a three-stage ring.
//
// Work: items of 128 rows × a range of columns (K split), handed out to a
// persistent grid; each item writes its exact int64 group sums, and
// sliced_combine adds the splits and applies the scales.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "tile_bf16_tc.cuh"

namespace ttg {
namespace sliced {

constexpr int kSlices = 8;         // digits per value (A and X)
constexpr int kGroups = 8;         // d = s + t in 2 … 9
constexpr int kRhs = 16;           // columns of X per slice (right-hand sides, zero-padded)
constexpr int kRows = 128;         // rows of A per item (TMEM lanes)
constexpr int kSlab = 32;          // K per stage (one 64-byte swizzle row of BF16)
constexpr int kChunk = 128;        // K between flushes of the accumulator
constexpr int kStages = 3;
constexpr int kStageA = kSlices * kRows * kSlab * 2;          // 64 KB: the eight A slices
constexpr int kStageX = kSlices * kRhs * kSlab * 2;           // 8 KB: the eight X slices
constexpr int kStageBytes = kStageA + kStageX;
constexpr int kSmemBytes = kStages * kStageBytes + 1024;      // + alignment slack
constexpr int kAccCols = kGroups * kRhs;                      // 128 TMEM columns per buffer
constexpr uint32_t kTmemCols = 2 * kAccCols;                  // two buffers
constexpr int kThreads = 384;                                 // warps 0-3 control, 4-11 drain
constexpr int kEpiWarps = 8;

struct Shared {
    uint64_t full[kStages];
    uint64_t empty[kStages];
    uint64_t accf[2];
    uint64_t afree[2];
    uint32_t tmem_base;
    uint32_t produced;
    uint32_t consumed;
    int failed;
};

struct Params {
    int N;          // rows and columns of A
    int n_items;    // row blocks × K splits
    int ksplit;     // K splits per row block
    int kitem;      // columns of A per item (multiple of kChunk)
    long long npad; // row stride of the partial sums
    long long* part;  // [ksplit][kGroups][kRhs][npad] exact group sums
    int* err;       // set to 1 when a bounded wait gives up
    long long timeout_ns;
};

__device__ __forceinline__ void tmem_alloc_cols(uint32_t* dst) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc::smem_u32(dst)), "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc_cols(uint32_t taddr) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(kTmemCols) : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            tc::smem_u32(dst)),
        "l"((uint64_t)map), "r"(tc::smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

// The product kernel.  Grid: persistent (≤ one block per SM); block: 384
// threads.  mapA: 3D (column j, row i, slice s) BF16 digits of A, box
// (32, 128, 8); mapX: 2D (column j, row (t-1)·16 + q) BF16 digits of X, box
// (32, 128).  Both 64B-swizzled; loads past N read zeros.
__global__ void __launch_bounds__(kThreads, 1)
    sliced_matmul_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapX, Params p) {
    extern __shared__ __align__(1024) uint8_t sm_raw[];
    uint8_t* ring = (uint8_t*)(((uintptr_t)sm_raw + 1023) & ~(uintptr_t)1023);
    __shared__ Shared sh;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            tc::mbar_init(&sh.full[s], 1);
            tc::mbar_init(&sh.empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&sh.accf[b], 1);
            tc::mbar_init(&sh.afree[b], kEpiWarps);
        }
        sh.produced = 0;
        sh.consumed = 0;
        sh.failed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        tc::fence_proxy_async_smem();
    }
    __syncwarp();
    if (warp == 0) tmem_alloc_cols(&sh.tmem_base);
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = sh.tmem_base;
    const long long limit = p.timeout_ns;
    const int chunks = p.kitem / kChunk;
    const int slabs = kChunk / kSlab;

    if (threadIdx.x == 0) {
        // Producer: per slab, the eight A slices and the X slices.
        uint32_t q = 0;
        for (int it = blockIdx.x; it < p.n_items && !sh.failed; it += gridDim.x) {
            const int rb = it / p.ksplit, ks = it % p.ksplit;
            const int row0 = rb * kRows, k0 = ks * p.kitem;
            for (int g = 0; g < chunks * slabs; ++g, ++q) {
                const int st = q % kStages;
                if (!tc::mbar_wait(&sh.empty[st], ((q / kStages) & 1) ^ 1, limit)) {
                    sh.failed = 1;
                    break;
                }
                uint8_t* dst = ring + (size_t)st * kStageBytes;
                tc::mbar_expect_tx(&sh.full[st], kStageBytes);
                tc::tma_load_3d(dst, &mapA, &sh.full[st], k0 + g * kSlab, row0, 0);
                tma_load_2d(dst + kStageA, &mapX, &sh.full[st], k0 + g * kSlab, 0);
            }
        }
        sh.produced = q;
    } else if (threadIdx.x == 32) {
        // MMA issuer: per K step of 16, slice s of A against X slices
        // 1 … 9−s into the groups s+1 … 9 (TMEM columns 16·(s−1) …).
        uint32_t q = 0, chunk = 0;
        bool good = true;
        for (int it = blockIdx.x; it < p.n_items && good; it += gridDim.x) {
            for (int c = 0; c < chunks && good; ++c, ++chunk) {
                const int buf = chunk & 1;
                if (!tc::mbar_wait(&sh.afree[buf], ((chunk >> 1) & 1) ^ 1, limit)) {
                    sh.failed = 1;
                    good = false;
                    break;
                }
                tc::tc_fence_after();
                const uint32_t dacc = tmem + (uint32_t)(kAccCols * buf);
                for (int sl = 0; sl < slabs; ++sl, ++q) {
                    const int st = q % kStages;
                    if (!tc::mbar_wait(&sh.full[st], (q / kStages) & 1, limit)) {
                        sh.failed = 1;
                        good = false;
                        break;
                    }
                    tc::tc_fence_after();
                    const uint32_t abase = tc::smem_u32(ring + (size_t)st * kStageBytes);
                    const uint32_t xbase = abase + kStageA;
#pragma unroll
                    for (int kk = 0; kk < kSlab / 16; ++kk) {
#pragma unroll
                        for (int s = 1; s <= kSlices; ++s) {
                            const uint64_t ad = tc::smem_desc_kmajor_sw64(abase + (uint32_t)((s - 1) * kRows * kSlab * 2) + kk * 32);
                            const uint64_t bd = tc::smem_desc_kmajor_sw64(xbase + kk * 32);
                            const uint32_t idesc = tc::idesc_bf16_f32(kRows, kRhs * (kGroups + 1 - s));
                            const bool acc = !(sl == 0 && kk == 0 && s == 1);
                            tc::umma_bf16(dacc + (uint32_t)(kRhs * (s - 1)), ad, bd, idesc, acc ? 1u : 0u);
                        }
                    }
                    tc::umma_commit(&sh.empty[st]);
                }
                if (good) tc::umma_commit(&sh.accf[buf]);
            }
        }
        sh.consumed = q;
    } else if (warp >= 4) {
        // Drain: warp w reads TMEM lanes 32·(w%4) … (rows of the item);
        // warps 4-7 the groups d = 2 … 5, warps 8-11 the groups 6 … 9.
        const int wq = warp & 3, half = (warp - 4) >> 2;
        const int r = 32 * wq + lane;
        uint32_t chunk = 0;
        bool good = true;
        for (int it = blockIdx.x; it < p.n_items && good; it += gridDim.x) {
            const int rb = it / p.ksplit, ks = it % p.ksplit;
            long long acc[4][kRhs];
#pragma unroll
            for (int g = 0; g < 4; ++g)
#pragma unroll
                for (int c = 0; c < kRhs; ++c) acc[g][c] = 0;
            for (int c = 0; c < chunks; ++c, ++chunk) {
                const int buf = chunk & 1;
                if (!tc::mbar_wait(&sh.accf[buf], (chunk >> 1) & 1, limit)) {
                    sh.failed = 1;
                    good = false;
                    break;
                }
                tc::tc_fence_after();
#pragma unroll
                for (int g = 0; g < 4; ++g) {
                    uint32_t v[16];
                    tmem_ld16(tmem + ((uint32_t)(32 * wq) << 16) + (uint32_t)(kAccCols * buf + kRhs * (4 * half + g)), v);
#pragma unroll
                    for (int c2 = 0; c2 < kRhs; ++c2) acc[g][c2] += (long long)__float2int_rn(__uint_as_float(v[c2]));
                }
                tc::tc_fence_before();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&sh.afree[buf]);
            }
            if (!good) break;
            const long long row = (long long)rb * kRows + r;
            if (row < p.N) {
#pragma unroll
                for (int g = 0; g < 4; ++g)
#pragma unroll
                    for (int c2 = 0; c2 < kRhs; ++c2)
                        p.part[(((long long)ks * kGroups + 4 * half + g) * kRhs + c2) * p.npad + row] = acc[g][c2];
            }
        }
    }
    __syncthreads();
    if (sh.failed) {
        if (threadIdx.x == 0) {
            atomicExch(p.err, 1);
            // Loads that were issued and never consumed land before exit.
            for (uint32_t q = sh.consumed; q < sh.produced; ++q)
                if (!tc::mbar_wait(&sh.full[q % kStages], (q / kStages) & 1, limit)) break;
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (warp == 0) tmem_dealloc_cols(tmem);
}

// Y_iq = σ_i τ_q Σ_d 2^-8d S_d(i,q), S_d the exact sum of the K splits;
// mode 0: Y = A X, mode 2: Y = B − A X (column-major, ld N).
__global__ void sliced_combine(int N, int nrhs, int ksplit, long long npad, const long long* __restrict__ part,
                               const int* __restrict__ rowexp, const int* __restrict__ colexp, const double* B, double* Y,
                               int mode) {
    const long long n = (long long)N * nrhs;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % N), q = (int)(e / N);
        double y = 0.0;
        for (int g = kGroups - 1; g >= 0; --g) {  // smallest weight first
            long long sd = 0;
            for (int ks = 0; ks < ksplit; ++ks) sd += part[(((long long)ks * kGroups + g) * kRhs + q) * npad + i];
            y += ldexp((double)sd, -8 * (g + 2));
        }
        y = ldexp(y, rowexp[i] + colexp[q]);
        Y[e] = mode == 2 ? B[e] - y : y;
    }
}

// Scale exponent of a set of values from the bits of the largest magnitude
// (|bits| as an integer orders like the value): E with max < 2^(E-1), so
// every value / 2^E lies in (-1/2, 1/2); 0 for an all-zero set.
__device__ __forceinline__ int slice_exponent(unsigned long long maxbits) {
    if (maxbits == 0) return 0;
    const int be = (int)(maxbits >> 52);   // biased exponent (0 for subnormals)
    return (be == 0 ? -1021 : be - 1021);  // max < 2^(be-1022) = 2^(E-1)
}

// The eight signed base-256 digits of v / 2^E (|v| / 2^E < 1/2), from the
// FP64 bits with integer operations only (the FP64 pipe of this GPU is
// slow): F = trunc(v · 2^(64-E)) is a 64-bit integer with |F| < 2^63, cut
// from the low end into digits in [-128, 127]; the top digit takes what is
// left, in [-128, 128].  v·2^-E = Σ_s d_s 2^-8s + ε with |ε| < 2^-64.
__device__ __forceinline__ void slice_digits(double v, int E, float (&d)[kSlices]) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int be = (int)((b >> 52) & 0x7FF);
    const unsigned long long mant = (b & 0xFFFFFFFFFFFFFULL) | (be ? (1ULL << 52) : 0ULL);
    // v = ±mant · 2^(e2), e2 = max(be, 1) - 1075; F = mant · 2^(e2 + 64 - E).
    const int sh = (be ? be : 1) - 1075 + 64 - E;
    unsigned long long mag;
    if (sh >= 0) mag = sh >= 64 ? 0ULL : (mant << sh);
    else mag = -sh >= 64 ? 0ULL : (mant >> (-sh));
    long long x = (b >> 63) ? -(long long)mag : (long long)mag;
#pragma unroll
    for (int s = kSlices - 1; s >= 1; --s) {
        const int lo = (int)(signed char)(x & 0xFF);
        d[s] = (float)lo;
        x = (x - lo) >> 8;
    }
    d[0] = (float)x;
}

// Digits of A (dense column-major N×N, symmetric: column i is row i).  One
// block per column i: σ_i = 2^E_i from the largest |A_ji|, then the eight
// digits of every entry into D[s][i][j] (row stride ld).
__global__ void __launch_bounds__(256) slice_rows(int N, const double* __restrict__ A, long long ld, __nv_bfloat16* D,
                                                   int* rowexp) {
    __shared__ unsigned long long red[8];
    __shared__ int sexp;
    const long long NN = (long long)ld * N;
    for (int i = blockIdx.x; i < N; i += gridDim.x) {
        const double* col = A + (size_t)i * N;
        unsigned long long m = 0;
        for (int j = threadIdx.x; j < N; j += blockDim.x)
            m = max(m, (unsigned long long)__double_as_longlong(col[j]) & 0x7FFFFFFFFFFFFFFFULL);
        for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long mm = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) mm = max(mm, red[w]);
            sexp = slice_exponent(mm);
            rowexp[i] = sexp;
        }
        __syncthreads();
        const int E = sexp;
        for (int j = threadIdx.x; j < N; j += blockDim.x) {
            float dg[kSlices];
            slice_digits(__ldcg(col + j), E, dg);
            __nv_bfloat16* d = D + (size_t)i * ld + j;
#pragma unroll
            for (int s = 0; s < kSlices; ++s) d[(size_t)s * NN] = __float2bfloat16_rn(dg[s]);
        }
        __syncthreads();
    }
}

// Column maxima of |X| as bits (non-negative doubles order like their bit
// patterns); colmax must be zeroed first.
__global__ void slice_colmax(int N, int nrhs, const double* __restrict__ X, unsigned long long* colmax) {
    const int q = blockIdx.y;
    unsigned long long m = 0;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < N; j += gridDim.x * blockDim.x)
        m = max(m, (unsigned long long)__double_as_longlong(X[(size_t)q * N + j]) & 0x7FFFFFFFFFFFFFFFULL);
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(colmax + q, m);
}

// Digits of X: rows t·16 + q of D (row stride ld), τ_q = 2^F_q.  Rows of
// columns q ≥ nrhs are not written (their products are never combined).
__global__ void slice_cols(int N, int nrhs, const double* __restrict__ X, const unsigned long long* __restrict__ colmax,
                           long long ld, __nv_bfloat16* D, int* colexp) {
    const long long n = (long long)N * nrhs;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(e % N), q = (int)(e / N);
        const int F = slice_exponent(colmax[q]);
        if (j == 0) colexp[q] = F;
        float dg[kSlices];
        slice_digits(X[e], F, dg);
#pragma unroll
        for (int t = 0; t < kSlices; ++t) D[(size_t)(t * kRhs + q) * ld + j] = __float2bfloat16_rn(dg[t]);
    }
}

}  // namespace sliced
}  // namespace ttg
