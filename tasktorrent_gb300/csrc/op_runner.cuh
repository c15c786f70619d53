// op_runner.cuh — one part of a plain tile task (FP64, or FP32 for the
// TTG_PREC_MIXED tasks without tensor-core or FP64-scratch variants) on the
// whole block; shared by the FP64 and the mixed executors.
#pragma once
#include "../../include/ttg.h"
#include "tile_f64.cuh"
#include "tile_small.cuh"

namespace ttg {

// Shared memory (doubles) the plain tile kernels need.
constexpr int kPlainSmemDoubles = kF64SmemDoubles > kSmallSmem ? kF64SmemDoubles : kSmallSmem;

// TTG_OP_SPIN: the block is busy for `seconds` of the global timer (thread 0
// spins, the others wait at the barrier).  The host accepts 0 <= seconds <= 1.
__device__ inline void spin_block(double seconds) {
    if (threadIdx.x == 0) {
        long long t0;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
        const long long ns = (long long)(seconds * 1e9);
        for (;;) {
            long long t;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
            if (t - t0 >= ns) break;
        }
    }
    __syncthreads();
}

// Returns 0.  POTRF (FP64 only) is run by the caller.
template <class T>
__device__ int run_op_plain(const ttg_op& op, int part, int parts, T* smem) {
    const T alpha = (T)op.alpha, beta = (T)op.beta;
    switch (op.kind) {
        case TTG_OP_TRSM_RLTN:
            if (op.m <= kSmallM)
                trsm_rows_small<T, true>(op.m, op.n, alpha, (const T*)op.a, op.lda, (T*)op.c, op.ldc, smem, part, parts);
            else
                trsm_rltn_tile<T>(op.m, op.n, alpha, (const T*)op.a, op.lda, (T*)op.c, op.ldc, smem, part, parts);
            return 0;
        case TTG_OP_TRSM_RLNN:
            trsm_rows_small<T, false>(op.m, op.n, alpha, (const T*)op.a, op.lda, (T*)op.c, op.ldc, smem, part, parts);
            return 0;
        case TTG_OP_SYRK_LN:
            gemm_tile_auto<T, false, true>(op.n, op.n, op.k, alpha, (const T*)op.a, op.lda, (const T*)op.a, op.lda, beta, (T*)op.c,
                                      op.ldc, smem, part, parts);
            return 0;
        case TTG_OP_GEMM_NT:
            if (op.m <= kSmallM)
                gemm_small_m<T, false>(op.m, op.n, op.k, alpha, (const T*)op.a, op.lda, (const T*)op.b, op.ldb, beta, (T*)op.c,
                                       op.ldc, smem, part, parts);
            else
                gemm_tile_auto<T, false, false>(op.m, op.n, op.k, alpha, (const T*)op.a, op.lda, (const T*)op.b, op.ldb, beta,
                                           (T*)op.c, op.ldc, smem, part, parts);
            return 0;
        case TTG_OP_GEMM_NN:
            if (op.m <= kSmallM)
                gemm_small_m<T, true>(op.m, op.n, op.k, alpha, (const T*)op.a, op.lda, (const T*)op.b, op.ldb, beta, (T*)op.c,
                                      op.ldc, smem, part, parts);
            else
                gemm_tile_auto<T, true, false>(op.m, op.n, op.k, alpha, (const T*)op.a, op.lda, (const T*)op.b, op.ldb, beta,
                                          (T*)op.c, op.ldc, smem, part, parts);
            return 0;
        case TTG_OP_GEADD:
            geadd_tile<T>(op.m, op.n, alpha, (const T*)op.a, op.lda, beta, (T*)op.c, op.ldc, part, parts);
            return 0;
        case TTG_OP_CONVERT:
            convert_tile(op.m, op.n, op.alpha, op.a, op.lda, op.beta, op.c, op.ldc, op.flags, part, parts);
            return 0;
        case TTG_OP_SPIN:
            spin_block(op.alpha);
            return 0;
        default:
            return 0;
    }
}

}  // namespace ttg
