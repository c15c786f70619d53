// ttg_mixed.cu — mixed-precision tile path of the executor.
//
// A mixed Cholesky keeps its working tiles in FP32 and runs:
//   POTRF  FP64: the FP32 diagonal tile is widened into an FP64 scratch tile,
//          factored there (potrf_l_f64), and the factor rounded back to FP32;
//   TRSM   FP32 (rows split across blocks);
//   SYRK/GEMM trailing updates: FP32 (kind 1) or BF16 on tensor cores with
//          FP32 accumulation (kind 0).
// The same persistent executor loop runs these tasks (exec_kernel_mixed); a
// graph that contains any TTG_PREC_MIXED task is launched on it, FP64 tasks
// of such a graph run as in the FP64 executor.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/ttg.h"
#include "exec.cuh"
#include "op_runner.cuh"
#include "tile_bf16_tc.cuh"
#include "tile_f64.cuh"
#include "ttg_internal.h"
#include "ttg_mixed_api.h"

namespace ttg {

// Mixed-op variants carried in ttg_op::flags.
enum { kMixedF32 = 1, kMixedBF16 = 2, kMixedBF16x3 = 3, kMixedF16x2 = 4 };
// Operand slices of a tensor-core update kind (tc_gemm_blocks' split).
__host__ __device__ constexpr int mixed_split(int flags) { return flags == kMixedBF16x3 ? 3 : (flags == kMixedF16x2 ? 2 : 1); }
// TTG_OP_CONVERT flags: a is float, c is float, and (mixed graphs) wait for
// the task's input column to arrive first (gate words in aux, column in k).
enum { kConvertAFloat = 1, kConvertCFloat = 2, kConvertGated = 4 };
// Gate word 0 with this bit: the input is converted already (the tasks do nothing).
constexpr uint32_t kGateConverted = 0x80000000u;

// Device tables of the BF16 path: panel copies (one b×b K-major slot per lower
// tile), the scale of each slot, and the power-of-two scale of each block row.
struct MixedTables {
    __nv_bfloat16* b16;      // 3 slices of n_slots slots (hi, mid, lo)
    float* slot_scale;
    const float* rowscale;
    int b;
    int n_slots;
    // Tensor map over b16 in device memory (a system of a batch or a serving
    // request), or null: the kernel parameter's map (a Cholesky plan).
    const CUtensorMap* map;
};

// Kernel parameters of the mixed executor (the tensor map must live in the
// parameter space: __grid_constant__).
struct __align__(64) MixedGlobals {
    CUtensorMap tmap;  // 3D map over the BF16 slots: (K = b, rows = b, slot)
    int has_tc;        // the graph has tensor-core updates
};

// Rows [r0, r1) of the FP32 tile W (column-major, ldw, n columns) to the
// K-major BF16 slot dst (row r at dst + r·b), multiplied by inv.
// The same rows as three BF16 slices hi + mid + lo = v (dst + s·slice), each
// the BF16 rounding of what the previous slices leave of v: together they
// hold v to FP32 accuracy.
__device__ inline void rows_to_bf16x3(const float* W, int ldw, int r0, int r1, int n, __nv_bfloat16* dst, size_t slice, int b,
                                      float inv) {
    const long total = (long)(r1 - r0) * n;
    for (long e = threadIdx.x; e < total; e += kThreads) {
        const int r = r0 + (int)(e / n), c = (int)(e % n);
        const float v = __ldcg(W + r + (size_t)c * ldw) * inv;
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        const float r1v = v - __bfloat162float(h);
        const __nv_bfloat16 mi = __float2bfloat16_rn(r1v);
        const __nv_bfloat16 lo = __float2bfloat16_rn(r1v - __bfloat162float(mi));
        const size_t o = (size_t)r * b + c;
        dst[o] = h;
        dst[slice + o] = mi;
        dst[2 * slice + o] = lo;
    }
}

// Split FP16 slices of v (|v| <= 1): hi = fp16(v), lo = fp16((v − hi)·2^11);
// v = hi + 2^-11·lo to ~2^-22 (the scale keeps lo out of FP16's subnormals).
__device__ __forceinline__ void f16x2_split(float v, unsigned short& hi, unsigned short& lo) {
    const __half h = __float2half_rn(v);
    hi = __half_as_ushort(h);
    lo = __half_as_ushort(__float2half_rn((v - __half2float(h)) * 2048.0f));
}

__device__ inline void rows_to_f16x2(const float* W, int ldw, int r0, int r1, int n, __nv_bfloat16* dst, size_t slice, int b,
                                     float inv) {
    unsigned short* d = reinterpret_cast<unsigned short*>(dst);
    const long total = (long)(r1 - r0) * n;
    for (long e = threadIdx.x; e < total; e += kThreads) {
        const int r = r0 + (int)(e / n), c = (int)(e % n);
        unsigned short h, l;
        f16x2_split(__ldcg(W + r + (size_t)c * ldw) * inv, h, l);
        const size_t o = (size_t)r * b + c;
        d[o] = h;
        d[slice + o] = l;
    }
}

__device__ inline void rows_to_bf16(const float* W, int ldw, int r0, int r1, int n, __nv_bfloat16* dst, int b, float inv) {
    const long total = (long)(r1 - r0) * n;
    for (long e = threadIdx.x; e < total; e += kThreads) {
        const int r = r0 + (int)(e / n), c = (int)(e % n);
        dst[(size_t)r * b + c] = __float2bfloat16_rn(__ldcg(W + r + (size_t)c * ldw) * inv);
    }
}

// ------------------------------------------------------------------------
// FP32 TRSM of the mixed path with the part's rows resident in shared memory.
//
// Part `part` owns rows [r0, r0 + rows) (rows <= kTrsmRows) of B (m×n, ldb)
// and computes B <- alpha·B·L⁻ᵀ (L n×n lower, ldl; cblas_dtrsm R,L,T,N of
// 2d_cholesky.cpp:479), n <= 512:
//   Bs[c·64 + r]   the row slice, column-major, 128 KB;
//   Ls[l·nL + c]   panel p of L: Ls[l·nL + c] = L(c, p + l) for c >= p;
//   iv[l]          1 / L(p + l, p + l).
// Per 32-column panel the panel is copied in with 16-byte asynchronous copies
// (all in flight at once), the panel columns of each row are solved by one
// thread per row (forward substitution), and the columns right of the panel
// are updated from shared memory in 4×8 register tiles.  The tile never goes
// back to global memory between panels: the per-panel GEMMs of the generic
// kernel were chains of global round trips (≈ 25 µs per 128×128 block).
constexpr int kTrsmRows = 64;
constexpr int kTrsmMaxN = 512;
constexpr int kTrsmSmemBytes = (kTrsmRows * kTrsmMaxN + 32 * kTrsmMaxN + 32) * 4;

__device__ __forceinline__ void cp_async16_mx(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(__cvta_generic_to_global(src))
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all_mx() { asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory"); }

// The resident form applies: n <= 512, 16-byte aligned operands and column
// starts, whole 16-byte row groups.
__device__ __forceinline__ bool trsm_resident_ok(int m, int n, const float* L, int ldl, const float* B, int ldb) {
    return n > 0 && n <= kTrsmMaxN && (n & 3) == 0 && (m & 3) == 0 && (ldl & 3) == 0 && (ldb & 3) == 0 &&
           ((uintptr_t)L & 15) == 0 && ((uintptr_t)B & 15) == 0;
}

// Rows [r0, r0 + rows) (r0 and rows multiples of 4, rows <= 64) solved in
// shared memory; on return Bs holds the solved slice (also written to B).
static __device__ __noinline__ void trsm_rltn_f32_resident(int n, float alpha, const float* L, int ldl, float* B, int ldb, int r0, int rows,
                                       float* smem) {
    float* Bs = smem;
    float* Ls = smem + kTrsmRows * kTrsmMaxN;
    float* iv = Ls + 32 * kTrsmMaxN;
    const int nL = (n + 7) & ~7;
    const int tid = threadIdx.x;
    const int q4 = rows >> 2;  // 16-byte groups per column of the slice
    for (int e = tid; e < n * q4; e += kThreads) {
        const int c = e / q4, q = e - c * q4;
        cp_async16_mx(Bs + c * kTrsmRows + 4 * q, B + r0 + 4 * q + (size_t)c * ldb);
    }
    cp_async_wait_all_mx();
    __syncthreads();
    if (alpha != 1.0f) {
        for (int e = tid; e < n * kTrsmRows; e += kThreads) Bs[e] *= alpha;
        __syncthreads();
    }
    const int rg = tid & 15, cg = tid >> 4;
    for (int p = 0; p < n; p += 32) {
        const int nb = min(32, n - p);
        const int seg = (n - p) >> 2;  // 16-byte groups of a panel column from row p
        for (int e = tid; e < nb * seg; e += kThreads) {
            const int l = e / seg, q = e - l * seg;
            cp_async16_mx(Ls + l * nL + p + 4 * q, L + p + 4 * q + (size_t)(p + l) * ldl);
        }
        cp_async_wait_all_mx();
        __syncthreads();
        if (tid < nb) iv[tid] = 1.0f / Ls[tid * nL + p + tid];
        __syncthreads();
        if (tid < rows) {
            float x[32];
#pragma unroll
            for (int c = 0; c < 32; ++c) x[c] = c < nb ? Bs[(p + c) * kTrsmRows + tid] : 0.0f;
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                if (c < nb) {
                    float sum = x[c];
#pragma unroll
                    for (int l = 0; l < c; ++l) sum = fmaf(-x[l], Ls[l * nL + p + c], sum);
                    x[c] = sum * iv[c];
                }
            }
#pragma unroll
            for (int c = 0; c < 32; ++c)
                if (c < nb) Bs[(p + c) * kTrsmRows + tid] = x[c];
        }
        __syncthreads();
        // Columns right of the panel: Bs[:, c] -= X_p · L(c, p:p+nb)ᵀ.
        for (int cb = p + nb + 8 * cg; cb < n; cb += 128) {
            float acc[4][8];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
            for (int l = 0; l < nb; ++l) {
                const float4 xv = *reinterpret_cast<const float4*>(Bs + (p + l) * kTrsmRows + 4 * rg);
                const float4 la = *reinterpret_cast<const float4*>(Ls + l * nL + cb);
                const float4 lb = *reinterpret_cast<const float4*>(Ls + l * nL + cb + 4);
                const float xs[4] = {xv.x, xv.y, xv.z, xv.w};
                const float ls[8] = {la.x, la.y, la.z, la.w, lb.x, lb.y, lb.z, lb.w};
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(xs[i], ls[j], acc[i][j]);
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (cb + j < n) {
                    float4* o = reinterpret_cast<float4*>(Bs + (cb + j) * kTrsmRows + 4 * rg);
                    float4 v = *o;
                    v.x -= acc[0][j];
                    v.y -= acc[1][j];
                    v.z -= acc[2][j];
                    v.w -= acc[3][j];
                    *o = v;
                }
            }
        }
        __syncthreads();
    }
    for (int e = tid; e < n * q4; e += kThreads) {
        const int c = e / q4, q = e - c * q4;
        *reinterpret_cast<float4*>(B + r0 + 4 * q + (size_t)c * ldb) = *reinterpret_cast<const float4*>(Bs + c * kTrsmRows + 4 * q);
    }
}

// Rows [r0, r0 + rows) of the resident slice Bs (n columns) as BF16 slices
// of the K-major slot dst (row r at dst + r·b), times inv: one slice (hi) or
// three (hi, mid, lo; slice s at dst + s·slice).  Each slice goes through a
// padded row-major buffer in the panel area, so the slot rows are written
// with consecutive columns.
// split: 1 plain BF16, 3 three BF16 slices, 2 split FP16 (mixed_split).
static __device__ __noinline__ void publish_bf16_resident(const float* smem, int n, int r0, int rows, __nv_bfloat16* dst, size_t slice, int b, float inv,
                                      int split) {
    const int nslices = split;
    const float* Bs = smem;
    __nv_bfloat16* T = reinterpret_cast<__nv_bfloat16*>(const_cast<float*>(smem) + kTrsmRows * kTrsmMaxN);
    constexpr int kTs = kTrsmMaxN + 2;  // row stride (odd number of 4-byte words)
    for (int sl = 0; sl < nslices; ++sl) {
        __syncthreads();
        for (int e = threadIdx.x; e < rows * n; e += kThreads) {
            const int r = e % rows, c = e / rows;
            const float v = Bs[c * kTrsmRows + r] * inv;
            __nv_bfloat16 out;
            if (split == 2) {
                unsigned short h, l;
                f16x2_split(v, h, l);
                out = __ushort_as_bfloat16(sl == 0 ? h : l);
            } else {
                const __nv_bfloat16 h = __float2bfloat16_rn(v);
                out = h;
                if (sl > 0) {
                    const float r1v = v - __bfloat162float(h);
                    const __nv_bfloat16 mi = __float2bfloat16_rn(r1v);
                    out = sl == 1 ? mi : __float2bfloat16_rn(r1v - __bfloat162float(mi));
                }
            }
            T[r * kTs + c] = out;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < rows * n; e += kThreads) {
            const int r = e / n, c = e - (e / n) * n;
            dst[(size_t)sl * slice + (size_t)(r0 + r) * b + c] = T[r * kTs + c];
        }
    }
    __syncthreads();
}

// An input task's share of its tile column: FP64 -> FP32 (round to nearest,
// as convert_f64_to_f32) over a contiguous chunk, 16 values per thread in
// flight (16-byte loads; the column starts on a tile boundary and holds an
// even number of values).
__device__ inline void convert_input_chunk(const double* __restrict__ src, float* __restrict__ dst, int len, int part, int parts) {
    const long per = ((long)len / parts + 2047) / 2048 * 2048;
    const long e0 = min((long)len, part * per), e1 = min((long)len, e0 + per);
    if (((uintptr_t)src & 15) || ((uintptr_t)dst & 7)) {  // odd tile edges: one value at a time
        for (long e = e0 + threadIdx.x; e < e1; e += kThreads) dst[e] = (float)__ldcg(src + e);
        __syncthreads();
        return;
    }
    constexpr int U = 8;  // double2 loads per thread per round
    for (long base = e0 + 2L * threadIdx.x; base < e1; base += 2L * kThreads * U) {
        double2 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long e = base + 2L * kThreads * u;
            v[u] = e + 1 < e1 ? __ldcg((const double2*)(src + e)) : make_double2(e < e1 ? __ldcg(src + e) : 0.0, 0.0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long e = base + 2L * kThreads * u;
            if (e + 1 < e1) *(float2*)(dst + e) = make_float2((float)v[u].x, (float)v[u].y);
            else if (e < e1) dst[e] = (float)v[u].x;
        }
    }
    __syncthreads();
}

// A task's tables, read through L2: in an open graph they are written while
// the launch runs, and an earlier system at the same address may sit in L1.
__device__ inline MixedTables load_tables(const void* aux) {
    static_assert(sizeof(MixedTables) % 8 == 0, "MixedTables words");
    MixedTables t;
    const unsigned long long* s = (const unsigned long long*)aux;
    unsigned long long* d = (unsigned long long*)&t;
#pragma unroll
    for (int i = 0; i < (int)(sizeof(MixedTables) / 8); ++i) d[i] = __ldcg(s + i);
    return t;
}

// open: the launch serves an open graph, whose systems' tensor maps are
// written in device memory while it runs (possibly where an earlier map was).
__device__ int run_op_mixed(const ttg_op& op, int part, int parts, double* smem, int* team, int* fin, tc::TcShared* tsh,
                             uint8_t* ring, const CUtensorMap* tmap, int* err, long long limit_ns, bool open) {
    if (op.kind == kOpSignal) {
        // A request of an open graph is complete: tell the host (op.c is a
        // word of host-mapped memory).
        if (threadIdx.x == 0) {
            __threadfence_system();
            *(volatile int*)op.c = op.m;
            __threadfence_system();
        }
        return 0;
    }
    if (op.prec == TTG_PREC_F64) {
        if (op.kind == TTG_OP_POTRF_L) {
            if (team)
                return potrf_l_f64_team(op.n, (double*)op.c, op.ldc, smem, TeamCtx{team, limit_ns, err}, nullptr, 0, fin);
            return potrf_l_f64(op.n, (double*)op.c, op.ldc, smem);
        }
        return run_op_plain<double>(op, part, parts, smem);
    }
    float* fsm = reinterpret_cast<float*>(smem);
    switch (op.kind) {
        case TTG_OP_POTRF_L: {
            // FP32 tile c (ldc) -> FP64 scratch aux (ld n) -> factor -> FP32.
            const int n = op.n;
            float* W = (float*)op.c;
            double* D = (double*)op.aux;
            if (team) return potrf_l_f64_team(n, D, n, smem, TeamCtx{team, limit_ns, err}, W, op.ldc, fin);
            for (long e = threadIdx.x; e < (long)n * n; e += kThreads) {
                const int i = (int)(e % n), j = (int)(e / n);
                D[e] = i >= j ? (double)ldcg(W + i + (size_t)j * op.ldc) : 0.0;
            }
            __syncthreads();
            const int info = potrf_l_f64(n, D, n, smem);
            __syncthreads();
            if (info == 0) {
                for (long e = threadIdx.x; e < (long)n * n; e += kThreads) {
                    const int i = (int)(e % n), j = (int)(e / n);
                    if (i >= j) W[i + (size_t)j * op.ldc] = (float)ldcg(D + e);
                }
            }
            __syncthreads();
            return info;
        }
        case TTG_OP_TRSM_RLTN:
            if (trsm_resident_ok(op.m, op.n, (const float*)op.a, op.lda, (const float*)op.c, op.ldc)) {
                // The part's rows: the same slices as the publish below.
                const int per = ((op.m + parts - 1) / parts + 15) / 16 * 16;
                const int r0 = min(op.m, part * per), r1 = min(op.m, r0 + per);
                if (r1 - r0 <= kTrsmRows) {
                    if (r1 > r0) trsm_rltn_f32_resident(op.n, (float)op.alpha, (const float*)op.a, op.lda, (float*)op.c, op.ldc, r0,
                                                        r1 - r0, fsm);
                    if (op.flags >= kMixedBF16) {
                        const MixedTables tbv = load_tables(op.aux);
                        const MixedTables* tb = &tbv;
                        const float s = __ldcg(tb->rowscale + op.k);
                        const size_t slice = (size_t)tb->n_slots * tb->b * tb->b;
                        if (r1 > r0)
                            publish_bf16_resident(fsm, op.n, r0, r1 - r0, tb->b16 + (size_t)op.ldb * tb->b * tb->b, slice, tb->b,
                                                  1.0f / s, mixed_split(op.flags));
                        if (threadIdx.x == 0 && part == 0) tb->slot_scale[op.ldb] = s;
                        tc::fence_proxy_async_global();
                    }
                    __syncthreads();
                    return 0;
                }
            }
            if (op.flags < kMixedBF16) return run_op_plain<float>(op, part, parts, fsm);
            trsm_rltn_tile<float>(op.m, op.n, (float)op.alpha, (const float*)op.a, op.lda, (float*)op.c, op.ldc, fsm, part,
                                  parts);
            {
                // Publish this row slice as the tile's BF16 panel copy.
                const MixedTables tbv = load_tables(op.aux);
                const MixedTables* tb = &tbv;
                const int per = ((op.m + parts - 1) / parts + 15) / 16 * 16;
                const int r0 = min(op.m, part * per), r1 = min(op.m, r0 + per);
                const float s = __ldcg(tb->rowscale + op.k);
                __syncthreads();
                const size_t slice = (size_t)tb->n_slots * tb->b * tb->b;
                if (op.flags == kMixedBF16x3)
                    rows_to_bf16x3((const float*)op.c, op.ldc, r0, r1, op.n, tb->b16 + (size_t)op.ldb * tb->b * tb->b, slice, tb->b,
                                   1.0f / s);
                else if (op.flags == kMixedF16x2)
                    rows_to_f16x2((const float*)op.c, op.ldc, r0, r1, op.n, tb->b16 + (size_t)op.ldb * tb->b * tb->b, slice, tb->b,
                                  1.0f / s);
                else
                    rows_to_bf16((const float*)op.c, op.ldc, r0, r1, op.n, tb->b16 + (size_t)op.ldb * tb->b * tb->b, tb->b, 1.0f / s);
                if (threadIdx.x == 0 && part == 0) tb->slot_scale[op.ldb] = s;
                tc::fence_proxy_async_global();
                __syncthreads();
            }
            return 0;
        case TTG_OP_SYRK_LN:
        case TTG_OP_GEMM_NT:
            if (op.flags >= kMixedBF16) {
                const MixedTables tbv = load_tables(op.aux);
                const MixedTables* tb = &tbv;
                const bool lower = op.kind == TTG_OP_SYRK_LN;
                // The part's share of the 128×256 output blocks, in turn.
                const int nblk = tc::tc_num_blocks(op.m, op.n, lower);
                const int per = (nblk + parts - 1) / parts;
                const float f = (float)op.alpha * __ldcg(tb->slot_scale + op.lda) * __ldcg(tb->slot_scale + op.ldb);
                const int b0 = min(nblk, part * per), b1 = min(nblk, (part + 1) * per);
                const CUtensorMap* mp = tb->map ? tb->map : tmap;
                // The map was written by a copy after this launch began: drop
                // any stale copy of that address from the descriptor cache.
                if (open && tb->map)
                    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(tb->map) : "memory");
                if (b1 > b0 && !tc::tc_gemm_blocks(tsh, ring, mp, op.lda, op.ldb, b0, b1 - b0, op.k, f, (float*)op.c, op.ldc, op.m,
                                                   op.n, lower, limit_ns, mixed_split(op.flags), tb->n_slots) &&
                    threadIdx.x == 0)
                    atomicCAS(err, 0, TTG_ETIMEOUT);
                return 0;
            }
            return run_op_plain<float>(op, part, parts, fsm);
        case TTG_OP_CONVERT:
            if (op.flags & kConvertGated) {
                // An input task: wait (bounded) until its tile column is in
                // device memory (gate word 1 + k equals the run's generation).
                __shared__ int s_late;
                if (threadIdx.x == 0) {
                    const volatile uint32_t* gate = (const volatile uint32_t*)op.aux;
                    const long long t0 = globaltimer();
                    int late = 0;
                    if (gate[0] & kGateConverted) late = -1;  // nothing to do
                    for (unsigned it = 0; late == 0 && gate[1 + op.k] != gate[0]; ++it) {
                        if ((it & 63) == 63 && globaltimer() - t0 > limit_ns) {
                            late = 1;
                            break;
                        }
                        __nanosleep(128);
                    }
                    __threadfence();
                    s_late = late;
                }
                __syncthreads();
                if (s_late > 0 && threadIdx.x == 0) atomicCAS(err, 0, TTG_ETIMEOUT);
                if (s_late) return 0;
            }
            if (op.flags & kConvertGated) {
                convert_input_chunk((const double*)op.a, (float*)op.c, op.m, part, parts);
                return 0;
            }
            convert_tile(op.m, op.n, op.alpha, op.a, op.lda, op.beta, op.c, op.ldc, op.flags & (kConvertAFloat | kConvertCFloat),
                         part, parts);
            return 0;
        default:
            return run_op_plain<float>(op, part, parts, fsm);
    }
}

// Dynamic shared memory: the FP64/FP32 tile kernels use the front, the
// tensor-core ring (1024-aligned) the rest; both are never live together.
constexpr int kMixedSmemBytes = tc::kSmemBytes > kPlainSmemDoubles * 8 ? tc::kSmemBytes : kPlainSmemDoubles * 8;
static_assert(kTrsmSmemBytes <= kMixedSmemBytes, "resident TRSM shared memory");
static_assert(kTrsmRows * kTrsmMaxN * 4 + kTrsmRows * (kTrsmMaxN + 2) * 2 <= kMixedSmemBytes, "BF16 publish buffer");

__global__ void __launch_bounds__(kThreads, 1) exec_kernel_mixed(ExecParams p, const __grid_constant__ MixedGlobals g) {
    extern __shared__ __align__(1024) double smem_mx[];
    __shared__ tc::TcShared tsh;
    uint8_t* ring = reinterpret_cast<uint8_t*>(((uintptr_t)smem_mx + 1023) & ~(uintptr_t)1023);
    if (g.has_tc) tc::tc_setup(&tsh);
    const CUtensorMap* tmap = &g.tmap;
    executor_loop(p, smem_mx, [&](const ttg_op& op, int part, int parts, double* smem, int* team, int* fin) {
        return run_op_mixed(op, part, parts, smem, team, fin, &tsh, ring, tmap, p.err, p.timeout_ns, p.pub != nullptr);
    });
    if (g.has_tc) tc::tc_teardown(&tsh, p.timeout_ns);
}

// Power-of-two scale of each block row: the smallest 2^e >= sqrt(max diag)
// (a bound on the entries of the Cholesky factor's block row).
__global__ void block_row_scales(const double* tiles, const int64_t* diag_off, int b, int nb, float* rowscale) {
    const int i = blockIdx.x;
    __shared__ double red[256];
    double mx = 0.0;
    for (int r = threadIdx.x; r < b; r += blockDim.x) mx = fmax(mx, fabs(tiles[diag_off[i] + r + (size_t)r * b]));
    red[threadIdx.x] = mx;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        int e = 0;
        frexp(sqrt(fmax(red[0], 1e-300)), &e);
        rowscale[i] = ldexpf(1.0f, e);
    }
}

__global__ void convert_f64_to_f32(const double* __restrict__ src, float* __restrict__ dst, int64_t n) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        dst[e] = (float)src[e];
}

// W(i,i) += shift·|W(i,i)| on one diagonal tile (ld = b).
__global__ void shift_diagonal(float* W, int b, double shift) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < b) {
        float* p = W + i + (size_t)i * b;
        *p = (float)((double)*p + shift * fabs((double)*p));
    }
}

__global__ void convert_f32_to_f64(const float* __restrict__ src, double* __restrict__ dst, int64_t n) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        dst[e] = (double)src[e];
}

}  // namespace ttg

using namespace ttg;

struct MixedCtx {
    int max_workers = 0;
    MixedGlobals globals{};  // tensor map of the plan whose graph is uploaded
};

ttg_status ttg_mixed_init(ttg_ctx* c) {
    MixedCtx* m = new MixedCtx();
    const int smem = kMixedSmemBytes;
    cudaError_t e = cudaFuncSetAttribute(exec_kernel_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int per_sm = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, exec_kernel_mixed, kThreads, smem);
    if (e != cudaSuccess) {
        delete m;
        ttg_set_last_cuda_error(e, "exec_kernel_mixed attributes", __FILE__, __LINE__);
        return TTG_ECUDA;
    }
    m->max_workers = std::max(1, per_sm) * c->sms;
    c->mixed = m;
    return TTG_OK;
}

int ttg_mixed_max_workers(const ttg_ctx* c) { return c->mixed ? ((const MixedCtx*)c->mixed)->max_workers : 0; }

void ttg_mixed_free(ttg_ctx* c) {
    delete (MixedCtx*)c->mixed;
    c->mixed = nullptr;
}

ttg_status ttg_launch_mixed(ttg_ctx* c, const ExecParams& p, cudaStream_t s) {
    MixedCtx* m = (MixedCtx*)c->mixed;
    if (!m || c->workers > m->max_workers) return TTG_EINVAL;
    const int smem = kMixedSmemBytes;
    void* args[] = {(void*)&p, (void*)&m->globals};
    ttg_note_launch();
    TTG_CUDA_CHECK(ttg_launch_executor_kernel(c, (const void*)exec_kernel_mixed, args, smem, s));
    return TTG_OK;
}

// ------------------------------------------------------------ plan state

struct ttg_mixed_state {
    ttg_ctx* ctx = nullptr;
    uint32_t* gate = nullptr;  // [1 + nb]: run generation, then the generation of each arrived tile column
    uint32_t gen = 0;
    int N = 0, nb = 0, kind = 1, b = 0;
    std::vector<int> bs;
    std::vector<int64_t> off;
    int64_t elems = 0;
    double* tiles64 = nullptr;  // the plan's FP64 tiles (input, then scratch)
    float* w32 = nullptr;       // FP32 working tiles -> low-precision factor
    // BF16 tensor-core path (kind 0)
    __nv_bfloat16* b16 = nullptr;  // one K-major b×b slot per lower tile
    float* slot_scale = nullptr;
    float* rowscale = nullptr;
    int64_t* diag_off = nullptr;
    MixedTables* tables = nullptr;  // device copy
    MixedGlobals globals{};
};

static int slot_of(const ttg_mixed_state* m, int i, int j) { return (int)(m->off[i + (size_t)j * m->nb] / ((int64_t)m->b * m->b)); }

// Tensor map over n_slots b×b K-major slots of three slices (slice s of
// slot t at z = t + s·n_slots): boxes of 32 columns × 128 rows, 64-byte swizzle.
static ttg_status encode_slot_map(CUtensorMap* map, void* b16, int b, int n_slots) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || !fn || q != cudaDriverEntryPointSuccess) {
        ttg_set_last_cuda_error(e, "cudaGetDriverEntryPointByVersion(cuTensorMapEncodeTiled)", __FILE__, __LINE__);
        return TTG_ECUDA;
    }
    auto encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    cuuint64_t dims[3] = {(cuuint64_t)b, (cuuint64_t)b, (cuuint64_t)(3 * n_slots)};  // three slices
    cuuint64_t strides[2] = {(cuuint64_t)b * 2, (cuuint64_t)b * b * 2};
    cuuint32_t box[3] = {(cuuint32_t)tc::kBK, 128u, 1u};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, b16, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        ttg_set_last_cuda_error(cudaErrorInvalidValue, "cuTensorMapEncodeTiled", __FILE__, __LINE__);
        return TTG_EINVAL;
    }
    return TTG_OK;
}

static ttg_status encode_tmap(ttg_mixed_state* m, int n_slots) {
    const ttg_status st = encode_slot_map(&m->globals.tmap, (void*)m->b16, m->b, n_slots);
    if (st == TTG_OK) m->globals.has_tc = 1;
    return st;
}

// ------------------------------------------------ per-system tensor-core data

// Header of one system in device memory: its tensor map, then its tables.
struct __align__(128) TcSysHeader {
    CUtensorMap map;
    MixedTables tables;
};
static_assert(sizeof(TcSysHeader) <= kTcHeaderBytes, "tensor-core system header");

size_t ttg_mixed_tc_slot_elems(int b, int nb) { return (size_t)3 * (size_t)(nb * (nb + 1) / 2) * b * b; }

ttg_status ttg_mixed_tc_header(void* host_hdr, void* dev_hdr, __nv_bfloat16* slots, float* slot_scale, const float* rowscale, int b,
                               int nb, void** tables) {
    if (!host_hdr || !dev_hdr || !slots || !slot_scale || !rowscale || b <= 0 || b % 128 != 0 || b > 512 || nb < 1 ||
        ((uintptr_t)dev_hdr & 127) != 0 || ((uintptr_t)slots & 127) != 0)
        return TTG_EINVAL;
    TcSysHeader* h = reinterpret_cast<TcSysHeader*>(host_hdr);
    memset(h, 0, sizeof(TcSysHeader));
    const int n_slots = nb * (nb + 1) / 2;
    const ttg_status st = encode_slot_map(&h->map, slots, b, n_slots);
    if (st != TTG_OK) return st;
    TcSysHeader* d = reinterpret_cast<TcSysHeader*>(dev_hdr);
    h->tables = MixedTables{slots, slot_scale, rowscale, b, n_slots, &d->map};
    if (tables) *tables = &d->tables;
    return TTG_OK;
}

namespace ttg {
// One block per item: 2^e >= sqrt(max |diag|) of the item's diagonal tile.
__global__ void row_scales_list(const TcRowScaleItem* items, int n) {
    __shared__ double red[128];
    for (int it = blockIdx.x; it < n; it += gridDim.x) {
        const TcRowScaleItem x = items[it];
        double mx = 0.0;
        for (int r = threadIdx.x; r < x.bs; r += blockDim.x) mx = fmax(mx, fabs(x.diag[r + (size_t)r * x.ld]));
        red[threadIdx.x] = mx;
        __syncthreads();
        for (int s2 = blockDim.x / 2; s2 > 0; s2 >>= 1) {
            if (threadIdx.x < s2) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s2]);
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            int e = 0;
            frexp(sqrt(fmax(red[0], 1e-300)), &e);
            *x.out = ldexpf(1.0f, e);
        }
        __syncthreads();
    }
}
}  // namespace ttg

ttg_status ttg_mixed_row_scales(const TcRowScaleItem* d_items, int n, void* stream) {
    if (n <= 0) return TTG_OK;
    if (!d_items) return TTG_EINVAL;
    ttg_note_launch();
    row_scales_list<<<std::min(n, 4096), 128, 0, (cudaStream_t)stream>>>(d_items, n);
    TTG_CUDA_CHECK(cudaGetLastError());
    return TTG_OK;
}

ttg_status ttg_mixed_row_scales_preload() {
    cudaFuncAttributes fa;
    TTG_CUDA_CHECK(cudaFuncGetAttributes(&fa, row_scales_list));
    return TTG_OK;
}

void ttg_mixed_set_tc(ttg_ctx* c, bool on) {
    if (c->mixed) ((MixedCtx*)c->mixed)->globals.has_tc = on ? 1 : 0;
}

ttg_status ttg_mixed_state_create(ttg_ctx* ctx, int N, int nb, const int* bs, const int64_t* off, double* tiles64, int kind,
                                  ttg_mixed_state** out) {
    *out = nullptr;
    if (kind != 0 && kind != 1) return TTG_EINVAL;
    if (kind == 0) {
        // Tensor-core updates: uniform tiles, a multiple of 128.
        for (int i = 0; i < nb; ++i)
            if (bs[i] != bs[0]) return TTG_EINVAL;
        if (bs[0] <= 0 || bs[0] % 128 != 0) return TTG_EINVAL;
    }
    ttg_mixed_state* m = new ttg_mixed_state();
    m->ctx = ctx;
    m->N = N;
    m->nb = nb;
    m->kind = kind;
    m->b = bs[0];
    m->bs.assign(bs, bs + nb);
    m->off.assign(off, off + (size_t)nb * nb);
    m->elems = 0;
    for (int i = 0; i < nb; ++i)
        for (int j = 0; j <= i; ++j) m->elems += (int64_t)bs[i] * bs[j];
    m->tiles64 = tiles64;
    auto fail = [&](cudaError_t e, const char* what) {
        ttg_set_last_cuda_error(e, what, __FILE__, __LINE__);
        ttg_mixed_state_destroy(m);
        return e == cudaErrorMemoryAllocation ? TTG_ENOMEM : TTG_ECUDA;
    };
    cudaError_t e = cudaMalloc((void**)&m->w32, sizeof(float) * std::max<int64_t>(1, m->elems));
    if (e != cudaSuccess) return fail(e, "cudaMalloc w32");
    if ((e = cudaMalloc((void**)&m->gate, sizeof(uint32_t) * (nb + 1))) != cudaSuccess) return fail(e, "cudaMalloc gate");
    if ((e = cudaMemset(m->gate, 0, sizeof(uint32_t) * (nb + 1))) != cudaSuccess) return fail(e, "memset gate");
    if (kind == 0) {
        const int n_slots = nb * (nb + 1) / 2;
        // Three slices of slots: the BF16 copies (slice 0) and, for split
        // updates, the two residual slices.
        if ((e = cudaMalloc((void**)&m->b16, sizeof(__nv_bfloat16) * 3 * m->elems)) != cudaSuccess) return fail(e, "cudaMalloc b16");
        if ((e = cudaMemset(m->b16, 0, sizeof(__nv_bfloat16) * 3 * m->elems)) != cudaSuccess) return fail(e, "memset b16");
        if ((e = cudaMalloc((void**)&m->slot_scale, sizeof(float) * n_slots)) != cudaSuccess) return fail(e, "cudaMalloc");
        if ((e = cudaMalloc((void**)&m->rowscale, sizeof(float) * nb)) != cudaSuccess) return fail(e, "cudaMalloc");
        if ((e = cudaMalloc((void**)&m->diag_off, sizeof(int64_t) * nb)) != cudaSuccess) return fail(e, "cudaMalloc");
        if ((e = cudaMalloc((void**)&m->tables, sizeof(MixedTables))) != cudaSuccess) return fail(e, "cudaMalloc");
        std::vector<int64_t> doff(nb);
        for (int i = 0; i < nb; ++i) doff[i] = off[i + (size_t)i * nb];
        cudaMemcpy(m->diag_off, doff.data(), sizeof(int64_t) * nb, cudaMemcpyHostToDevice);
        MixedTables t{m->b16, m->slot_scale, m->rowscale, m->b, n_slots, nullptr};
        cudaMemcpy(m->tables, &t, sizeof(t), cudaMemcpyHostToDevice);
        ttg_status st = encode_tmap(m, n_slots);
        if (st != TTG_OK) {
            ttg_mixed_state_destroy(m);
            return st;
        }
    }
    *out = m;
    return TTG_OK;
}

void ttg_mixed_state_destroy(ttg_mixed_state* m) {
    if (!m) return;
    if (m->w32) cudaFree(m->w32);
    if (m->gate) cudaFree(m->gate);
    if (m->b16) cudaFree(m->b16);
    if (m->slot_scale) cudaFree(m->slot_scale);
    if (m->rowscale) cudaFree(m->rowscale);
    if (m->diag_off) cudaFree(m->diag_off);
    if (m->tables) cudaFree(m->tables);
    delete m;
}

bool ttg_mixed_has_tc(const ttg_mixed_state* m) { return m && m->kind == 0; }

static ttg_op mixed_op(const ttg_mixed_state* m, int kind, int upd) {
    ttg_op op{};
    op.kind = kind;
    op.prec = TTG_PREC_MIXED;
    op.flags = m->kind != 0 || upd == TTG_UPD_FP32
                   ? kMixedF32
                   : (upd == TTG_UPD_BF16X3 ? kMixedBF16x3 : (upd == TTG_UPD_F16X2 ? kMixedF16x2 : kMixedBF16));
    op.alpha = 1.0;
    return op;
}

ttg_op ttg_mixed_potrf_op(ttg_mixed_state* m, int j, int upd) {
    ttg_op op = mixed_op(m, TTG_OP_POTRF_L, upd);
    const int64_t o = m->off[j + (size_t)j * m->nb];
    op.m = op.n = m->bs[j];
    op.c = m->w32 + o;
    op.ldc = std::max(1, m->bs[j]);
    op.aux = m->tiles64 + o;  // FP64 scratch: the diagonal tile's own FP64 slot
    return op;
}

ttg_op ttg_mixed_trsm_op(ttg_mixed_state* m, int i, int j, int upd) {
    ttg_op op = mixed_op(m, TTG_OP_TRSM_RLTN, upd);
    op.m = m->bs[i];
    op.n = m->bs[j];
    op.a = m->w32 + m->off[j + (size_t)j * m->nb];
    op.lda = std::max(1, m->bs[j]);
    op.c = m->w32 + m->off[i + (size_t)j * m->nb];
    op.ldc = std::max(1, m->bs[i]);
    if (op.flags >= kMixedBF16) {
        op.aux = m->tables;
        op.ldb = slot_of(m, i, j);  // BF16 slot written by this task
        op.k = i;                   // block row: its power-of-two scale
    }
    return op;
}

ttg_op ttg_mixed_update_op(ttg_mixed_state* m, int k, int i, int j, int upd) {
    ttg_op op = mixed_op(m, i == j ? TTG_OP_SYRK_LN : TTG_OP_GEMM_NT, upd);
    op.m = m->bs[i];
    op.n = m->bs[j];
    op.k = m->bs[k];
    op.alpha = -1.0;
    op.beta = 1.0;
    op.c = m->w32 + m->off[i + (size_t)j * m->nb];
    op.ldc = std::max(1, m->bs[i]);
    if (op.flags >= kMixedBF16) {
        op.aux = m->tables;
        op.lda = slot_of(m, i, k);
        op.ldb = slot_of(m, j, k);
        return op;
    }
    op.a = m->w32 + m->off[i + (size_t)k * m->nb];
    op.lda = std::max(1, m->bs[i]);
    op.b = m->w32 + m->off[j + (size_t)k * m->nb];
    op.ldb = std::max(1, m->bs[j]);
    return op;
}

ttg_status ttg_mixed_prepare(ttg_mixed_state* m, void* stream, double shift, int upd, const double* src, bool in_graph) {
    const bool tc = upd != TTG_UPD_FP32;
    cudaStream_t s = (cudaStream_t)stream;
    if (!src || (in_graph && shift > 0)) return TTG_EINVAL;
    if (!in_graph) {
        ttg_note_launch();
        convert_f64_to_f32<<<m->ctx->sms * 8, 256, 0, s>>>(src, m->w32, m->elems);
        TTG_CUDA_CHECK(cudaGetLastError());
    }
    if (shift > 0) {
        for (int j = 0; j < m->nb; ++j) {
            const int64_t o = m->off[j + (size_t)j * m->nb];
            ttg_note_launch();
            shift_diagonal<<<(m->bs[j] + 255) / 256, 256, 0, s>>>(m->w32 + o, m->bs[j], shift);
        }
        TTG_CUDA_CHECK(cudaGetLastError());
    }
    MixedCtx* mc = (MixedCtx*)m->ctx->mixed;
    if (m->kind == 0 && tc) {
        ttg_note_launch();
        block_row_scales<<<m->nb, 256, 0, s>>>(src, m->diag_off, m->b, m->nb, m->rowscale);
        TTG_CUDA_CHECK(cudaGetLastError());
        mc->globals = m->globals;
    } else {
        mc->globals.has_tc = 0;
    }
    return TTG_OK;
}

ttg_op ttg_mixed_input_op(ttg_mixed_state* m, int j, const double* src) {
    // The column's tiles (j..nb-1, j) are contiguous: convert them as one
    // vector of `len` values, split into parts of at most 256K values.
    const int64_t o = m->off[j + (size_t)j * m->nb];
    int64_t len = 0;
    for (int i = j; i < m->nb; ++i) len += (int64_t)m->bs[i] * m->bs[j];
    ttg_op op{};
    op.kind = TTG_OP_CONVERT;
    op.prec = TTG_PREC_MIXED;
    op.m = (int)len;
    op.n = 1;
    op.k = j;  // the gate word of the column
    op.a = src + o;
    op.lda = (int)std::max<int64_t>(1, len);
    op.c = m->w32 + o;
    op.ldc = op.lda;
    op.alpha = 1.0;
    op.beta = 0.0;
    op.flags = kConvertCFloat | kConvertGated;
    op.aux = m->gate;
    op.parts = (int)std::min<int64_t>(64, std::max<int64_t>(1, (len + 262143) / 262144));
    return op;
}

uint32_t* ttg_mixed_gate(ttg_mixed_state* m) { return m->gate; }

__global__ void gate_fill(uint32_t* gate, int n, uint32_t gen) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) gate[i] = gen;
}

uint32_t ttg_mixed_gate_begin(ttg_mixed_state* m, void* stream, bool converted) {
    if (++m->gen >= kGateConverted) m->gen = 1;  // 0 is the value of a fresh gate
    ttg_note_launch();
    gate_fill<<<1, 32, 0, (cudaStream_t)stream>>>(m->gate, 1, converted ? (m->gen | kGateConverted) : m->gen);
    return m->gen;
}

const double* ttg_mixed_factor_tiles(ttg_mixed_state* m) {
    ttg_note_launch();
    convert_f32_to_f64<<<m->ctx->sms * 8, 256>>>(m->w32, m->tiles64, m->elems);
    if (cudaStreamSynchronize(nullptr) != cudaSuccess) return nullptr;
    return m->tiles64;
}

const float* ttg_mixed_factor32(ttg_mixed_state* m) { return m->w32; }
