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
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "../../include/ttg.h"
#include "exec.cuh"
#include "tile_f64.cuh"
#include "ttg_internal.h"
#include "ttg_mixed_api.h"

namespace ttg {

// Mixed-op variants carried in ttg_op::flags.
enum { kMixedF32 = 1 };

__device__ int run_op_mixed(const ttg_op& op, int part, int parts, double* smem) {
    if (op.prec == TTG_PREC_F64) {
        switch (op.kind) {
            case TTG_OP_POTRF_L:
                return potrf_l_f64(op.n, (double*)op.c, op.ldc, smem);
            case TTG_OP_TRSM_RLTN:
                trsm_rltn_f64(op.m, op.n, op.alpha, (const double*)op.a, op.lda, (double*)op.c, op.ldc, smem, part, parts);
                return 0;
            case TTG_OP_SYRK_LN:
                gemm_f64<false, true>(op.n, op.n, op.k, op.alpha, (const double*)op.a, op.lda, (const double*)op.a, op.lda,
                                      op.beta, (double*)op.c, op.ldc, smem, part, parts);
                return 0;
            case TTG_OP_GEMM_NT:
                gemm_f64<false, false>(op.m, op.n, op.k, op.alpha, (const double*)op.a, op.lda, (const double*)op.b, op.ldb,
                                       op.beta, (double*)op.c, op.ldc, smem, part, parts);
                return 0;
            case TTG_OP_GEMM_NN:
                gemm_f64<true, false>(op.m, op.n, op.k, op.alpha, (const double*)op.a, op.lda, (const double*)op.b, op.ldb,
                                      op.beta, (double*)op.c, op.ldc, smem, part, parts);
                return 0;
            case TTG_OP_GEADD:
                geadd_f64(op.m, op.n, op.alpha, (const double*)op.a, op.lda, op.beta, (double*)op.c, op.ldc, part, parts);
                return 0;
            default:
                return 0;
        }
    }
    float* fsm = reinterpret_cast<float*>(smem);
    switch (op.kind) {
        case TTG_OP_POTRF_L: {
            // FP32 tile c (ldc) -> FP64 scratch aux (ld n) -> factor -> FP32.
            const int n = op.n;
            float* W = (float*)op.c;
            double* D = (double*)op.aux;
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
            trsm_rltn_tile<float>(op.m, op.n, (float)op.alpha, (const float*)op.a, op.lda, (float*)op.c, op.ldc, fsm, part,
                                  parts);
            return 0;
        case TTG_OP_SYRK_LN:
            gemm_tile<float, false, true>(op.n, op.n, op.k, (float)op.alpha, (const float*)op.a, op.lda, (const float*)op.a,
                                          op.lda, (float)op.beta, (float*)op.c, op.ldc, fsm, part, parts);
            return 0;
        case TTG_OP_GEMM_NT:
            gemm_tile<float, false, false>(op.m, op.n, op.k, (float)op.alpha, (const float*)op.a, op.lda, (const float*)op.b,
                                           op.ldb, (float)op.beta, (float*)op.c, op.ldc, fsm, part, parts);
            return 0;
        default:
            return 0;
    }
}

__global__ void __launch_bounds__(kThreads, 1) exec_kernel_mixed(ExecParams p) {
    extern __shared__ __align__(128) double smem_mx[];
    executor_loop(p, smem_mx, [](const ttg_op& op, int part, int parts, double* smem) {
        return run_op_mixed(op, part, parts, smem);
    });
}

__global__ void convert_f64_to_f32(const double* __restrict__ src, float* __restrict__ dst, int64_t n) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        dst[e] = (float)src[e];
}

__global__ void convert_f32_to_f64(const float* __restrict__ src, double* __restrict__ dst, int64_t n) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        dst[e] = (double)src[e];
}

}  // namespace ttg

using namespace ttg;

struct MixedCtx {
    int max_workers = 0;
};

ttg_status ttg_mixed_init(ttg_ctx* c) {
    MixedCtx* m = new MixedCtx();
    const int smem = kF64SmemDoubles * (int)sizeof(double);
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

void ttg_mixed_free(ttg_ctx* c) {
    delete (MixedCtx*)c->mixed;
    c->mixed = nullptr;
}

ttg_status ttg_launch_mixed(ttg_ctx* c, const ExecParams& p, cudaStream_t s) {
    MixedCtx* m = (MixedCtx*)c->mixed;
    if (!m || c->workers > m->max_workers) return TTG_EINVAL;
    const int smem = kF64SmemDoubles * (int)sizeof(double);
    void* args[] = {(void*)&p};
    TTG_CUDA_CHECK(cudaLaunchCooperativeKernel((const void*)exec_kernel_mixed, dim3(c->workers), dim3(kThreads), args, smem, s));
    return TTG_OK;
}

// ------------------------------------------------------------ plan state

struct ttg_mixed_state {
    ttg_ctx* ctx = nullptr;
    int N = 0, nb = 0, kind = 1;
    std::vector<int> bs;
    std::vector<int64_t> off;
    int64_t elems = 0;
    double* tiles64 = nullptr;  // the plan's FP64 tiles (input, then scratch)
    float* w32 = nullptr;       // FP32 working tiles -> low-precision factor
};

ttg_status ttg_mixed_state_create(ttg_ctx* ctx, int N, int nb, const int* bs, const int64_t* off, double* tiles64, int kind,
                                  ttg_mixed_state** out) {
    *out = nullptr;
    if (kind != 1) return TTG_EINVAL;  // only FP32 updates so far
    ttg_mixed_state* m = new ttg_mixed_state();
    m->ctx = ctx;
    m->N = N;
    m->nb = nb;
    m->kind = kind;
    m->bs.assign(bs, bs + nb);
    m->off.assign(off, off + (size_t)nb * nb);
    m->elems = 0;
    for (int i = 0; i < nb; ++i)
        for (int j = 0; j <= i; ++j) m->elems += (int64_t)bs[i] * bs[j];
    m->tiles64 = tiles64;
    cudaError_t e = cudaMalloc((void**)&m->w32, sizeof(float) * std::max<int64_t>(1, m->elems));
    if (e != cudaSuccess) {
        delete m;
        ttg_set_last_cuda_error(e, "cudaMalloc w32", __FILE__, __LINE__);
        return TTG_ENOMEM;
    }
    *out = m;
    return TTG_OK;
}

void ttg_mixed_state_destroy(ttg_mixed_state* m) {
    if (!m) return;
    if (m->w32) cudaFree(m->w32);
    delete m;
}

static ttg_op mixed_op(int kind) {
    ttg_op op{};
    op.kind = kind;
    op.prec = TTG_PREC_MIXED;
    op.flags = kMixedF32;
    op.alpha = 1.0;
    return op;
}

ttg_op ttg_mixed_potrf_op(ttg_mixed_state* m, int j) {
    ttg_op op = mixed_op(TTG_OP_POTRF_L);
    const int64_t o = m->off[j + (size_t)j * m->nb];
    op.m = op.n = m->bs[j];
    op.c = m->w32 + o;
    op.ldc = std::max(1, m->bs[j]);
    op.aux = m->tiles64 + o;  // FP64 scratch: the diagonal tile's own FP64 slot
    return op;
}

ttg_op ttg_mixed_trsm_op(ttg_mixed_state* m, int i, int j) {
    ttg_op op = mixed_op(TTG_OP_TRSM_RLTN);
    op.m = m->bs[i];
    op.n = m->bs[j];
    op.a = m->w32 + m->off[j + (size_t)j * m->nb];
    op.lda = std::max(1, m->bs[j]);
    op.c = m->w32 + m->off[i + (size_t)j * m->nb];
    op.ldc = std::max(1, m->bs[i]);
    return op;
}

ttg_op ttg_mixed_update_op(ttg_mixed_state* m, int k, int i, int j) {
    ttg_op op = mixed_op(i == j ? TTG_OP_SYRK_LN : TTG_OP_GEMM_NT);
    op.m = m->bs[i];
    op.n = m->bs[j];
    op.k = m->bs[k];
    op.alpha = -1.0;
    op.beta = 1.0;
    op.a = m->w32 + m->off[i + (size_t)k * m->nb];
    op.lda = std::max(1, m->bs[i]);
    op.b = m->w32 + m->off[j + (size_t)k * m->nb];
    op.ldb = std::max(1, m->bs[j]);
    op.c = m->w32 + m->off[i + (size_t)j * m->nb];
    op.ldc = std::max(1, m->bs[i]);
    return op;
}

ttg_status ttg_mixed_prepare(ttg_mixed_state* m, void* stream) {
    convert_f64_to_f32<<<m->ctx->sms * 8, 256, 0, (cudaStream_t)stream>>>(m->tiles64, m->w32, m->elems);
    TTG_CUDA_CHECK(cudaGetLastError());
    return TTG_OK;
}

const double* ttg_mixed_factor_tiles(ttg_mixed_state* m) {
    convert_f32_to_f64<<<m->ctx->sms * 8, 256>>>(m->w32, m->tiles64, m->elems);
    if (cudaStreamSynchronize(nullptr) != cudaSuccess) return nullptr;
    return m->tiles64;
}

const float* ttg_mixed_factor32(ttg_mixed_state* m) { return m->w32; }
