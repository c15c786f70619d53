// ttg_sliced.cu — host side of the FP64-accurate tensor-core product
// Y = A·X (sliced_matmul_tc.cuh): the digit buffers of A and X, their tensor
// maps, the partial sums, and the launches.  Used by the solver for the
// residuals b − A·x and the FP64 Krylov operator, and exported for tests as
// ttg_sliced_matmul (include/ttg_apps.h).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>

#include "../../include/ttg.h"
#include "../../include/ttg_apps.h"
#include "sliced_matmul_tc.cuh"
#include "ttg_internal.h"
#include "ttg_sliced_api.h"

using namespace ttg;

struct ttg_sliced {
    ttg_ctx* ctx = nullptr;
    int N = 0;
    long long ld = 0;                  // row stride of the digit arrays (multiple of 8)
    __nv_bfloat16* adig = nullptr;     // [8][N][ld]
    __nv_bfloat16* xdig = nullptr;     // [128][ld]
    int* rowexp = nullptr;             // [N]
    int* colexp = nullptr;             // [16]
    unsigned long long* colmax = nullptr;  // [16]
    long long* part = nullptr;         // [ksplit][8][16][ld]
    int* err = nullptr;                // bounded-wait flag
    int ksplit = 1, kitem = 0, n_items = 0, grid = 0;
    CUtensorMap mapA, mapX;
    bool have_matrix = false;
};

namespace {

ttg_status encode(CUtensorMap* map, void* base, int rank, const cuuint64_t* dims, const cuuint64_t* strides,
                  const cuuint32_t* box) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || !fn || q != cudaDriverEntryPointSuccess) {
        ttg_set_last_cuda_error(e, "cudaGetDriverEntryPointByVersion(cuTensorMapEncodeTiled)", __FILE__, __LINE__);
        return TTG_ECUDA;
    }
    auto enc = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, rank, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        ttg_set_last_cuda_error(cudaErrorInvalidValue, "cuTensorMapEncodeTiled (sliced product)", __FILE__, __LINE__);
        return TTG_EINVAL;
    }
    return TTG_OK;
}

}  // namespace

ttg_status ttg_sliced_create(ttg_ctx* ctx, int N, ttg_sliced** out) {
    *out = nullptr;
    if (!ctx || N < 1) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(ctx->device));
    ttg_sliced* S = new ttg_sliced();
    S->ctx = ctx;
    S->N = N;
    S->ld = ((long long)N + 7) / 8 * 8;
    // K split: enough items of 128 rows for several waves of the SMs.
    const int rowblocks = (N + sliced::kRows - 1) / sliced::kRows;
    const int kchunks = (N + sliced::kChunk - 1) / sliced::kChunk;
    int ks = std::max(1, std::min(kchunks, (8 * ctx->sms + rowblocks - 1) / rowblocks));
    S->kitem = (kchunks + ks - 1) / ks * sliced::kChunk;
    S->ksplit = (N + S->kitem - 1) / S->kitem;
    S->n_items = rowblocks * S->ksplit;
    S->grid = std::min(S->n_items, ctx->sms);
    auto fail = [&](cudaError_t e, const char* what) -> ttg_status {
        ttg_set_last_cuda_error(e, what, __FILE__, __LINE__);
        ttg_sliced_destroy(S);
        return e == cudaErrorMemoryAllocation ? TTG_ENOMEM : TTG_ECUDA;
    };
    cudaError_t e;
    const size_t NL = (size_t)S->ld * N;
    if ((e = cudaMalloc((void**)&S->adig, sizeof(__nv_bfloat16) * sliced::kSlices * NL)) != cudaSuccess) return fail(e, "cudaMalloc digits of A");
    if ((e = cudaMalloc((void**)&S->xdig, sizeof(__nv_bfloat16) * 128 * (size_t)S->ld)) != cudaSuccess) return fail(e, "cudaMalloc digits of X");
    if ((e = cudaMemset(S->xdig, 0, sizeof(__nv_bfloat16) * 128 * (size_t)S->ld)) != cudaSuccess) return fail(e, "memset");
    if ((e = cudaMalloc((void**)&S->rowexp, sizeof(int) * N)) != cudaSuccess) return fail(e, "cudaMalloc");
    if ((e = cudaMalloc((void**)&S->colexp, sizeof(int) * 16)) != cudaSuccess) return fail(e, "cudaMalloc");
    if ((e = cudaMalloc((void**)&S->colmax, sizeof(unsigned long long) * 16)) != cudaSuccess) return fail(e, "cudaMalloc");
    if ((e = cudaMalloc((void**)&S->err, sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc");
    if ((e = cudaMemset(S->err, 0, sizeof(int))) != cudaSuccess) return fail(e, "memset");
    const size_t np = (size_t)S->ksplit * sliced::kGroups * sliced::kRhs * S->ld;
    if ((e = cudaMalloc((void**)&S->part, sizeof(long long) * np)) != cudaSuccess) return fail(e, "cudaMalloc partial sums");
    if ((e = cudaFuncSetAttribute(sliced::sliced_matmul_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  sliced::kSmemBytes)) != cudaSuccess)
        return fail(e, "cudaFuncSetAttribute (sliced product)");
    {
        cuuint64_t dims[3] = {(cuuint64_t)N, (cuuint64_t)N, (cuuint64_t)sliced::kSlices};
        cuuint64_t strides[2] = {(cuuint64_t)S->ld * 2, (cuuint64_t)S->ld * N * 2};
        cuuint32_t box[3] = {(cuuint32_t)sliced::kSlab, (cuuint32_t)sliced::kRows, (cuuint32_t)sliced::kSlices};
        ttg_status st = encode(&S->mapA, S->adig, 3, dims, strides, box);
        if (st != TTG_OK) {
            ttg_sliced_destroy(S);
            return st;
        }
    }
    {
        cuuint64_t dims[2] = {(cuuint64_t)N, 128};
        cuuint64_t strides[1] = {(cuuint64_t)S->ld * 2};
        cuuint32_t box[2] = {(cuuint32_t)sliced::kSlab, 128};
        ttg_status st = encode(&S->mapX, S->xdig, 2, dims, strides, box);
        if (st != TTG_OK) {
            ttg_sliced_destroy(S);
            return st;
        }
    }
    *out = S;
    return TTG_OK;
}

void ttg_sliced_destroy(ttg_sliced* S) {
    if (!S) return;
    cudaSetDevice(S->ctx->device);
    for (void* p : {(void*)S->adig, (void*)S->xdig, (void*)S->rowexp, (void*)S->colexp, (void*)S->colmax, (void*)S->part,
                    (void*)S->err})
        if (p) cudaFree(p);
    delete S;
}

size_t ttg_sliced_bytes(int N) {
    const size_t ld = ((size_t)N + 7) / 8 * 8;
    return sizeof(__nv_bfloat16) * sliced::kSlices * ld * (size_t)N;
}

ttg_status ttg_sliced_set_matrix(ttg_sliced* S, const double* dA, cudaStream_t s) {
    if (!S || !dA) return TTG_EINVAL;
    ttg_note_launch();
    sliced::slice_rows<<<std::min(S->N, S->ctx->sms * 8), 256, 0, s>>>(S->N, dA, S->ld, S->adig, S->rowexp);
    TTG_CUDA_CHECK(cudaGetLastError());
    S->have_matrix = true;
    return TTG_OK;
}

ttg_status ttg_sliced_matmul_run(ttg_sliced* S, const double* X, int nrhs, const double* B, double* Y, int mode, cudaStream_t s) {
    if (!S || !S->have_matrix || !X || !Y || nrhs < 1 || nrhs > sliced::kRhs || (mode == 2 && !B)) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaMemsetAsync(S->colmax, 0, sizeof(unsigned long long) * 16, s));
    ttg_note_launch();
    sliced::slice_colmax<<<dim3(std::max(1, std::min(64, (S->N + 255) / 256)), nrhs), 256, 0, s>>>(S->N, nrhs, X, S->colmax);
    ttg_note_launch();
    sliced::slice_cols<<<S->ctx->sms * 4, 256, 0, s>>>(S->N, nrhs, X, S->colmax, S->ld, S->xdig, S->colexp);
    sliced::Params p;
    p.N = S->N;
    p.n_items = S->n_items;
    p.ksplit = S->ksplit;
    p.kitem = S->kitem;
    p.npad = S->ld;
    p.part = S->part;
    p.err = S->err;
    p.timeout_ns = (long long)(std::max(1.0, S->ctx->timeout_s) * 1e9);
    ttg_note_launch();
    sliced::sliced_matmul_kernel<<<S->grid, sliced::kThreads, sliced::kSmemBytes, s>>>(S->mapA, S->mapX, p);
    ttg_note_launch();
    sliced::sliced_combine<<<S->ctx->sms * 4, 256, 0, s>>>(S->N, nrhs, S->ksplit, S->ld, S->part, S->rowexp, S->colexp, B, Y,
                                                           mode);
    TTG_CUDA_CHECK(cudaGetLastError());
    return TTG_OK;
}

int* ttg_sliced_err(ttg_sliced* S) { return S ? S->err : nullptr; }

ttg_status ttg_sliced_reset_err(ttg_sliced* S, cudaStream_t s) {
    if (!S) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaMemsetAsync(S->err, 0, sizeof(int), s));
    return TTG_OK;
}

extern "C" ttg_status ttg_sliced_matmul(ttg_ctx* ctx, int32_t N, const double* d_A, int32_t nrhs, const double* d_X,
                                        const double* d_B, double* d_Y, int32_t mode, void* stream) {
    if (!ctx || N < 1 || !d_A || !d_X || !d_Y || nrhs < 1 || nrhs > 16 || (mode != 0 && mode != 2) || (mode == 2 && !d_B))
        return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(ctx->device));
    cudaStream_t s = (cudaStream_t)stream;
    ttg_sliced* S = nullptr;
    ttg_status st = ttg_sliced_create(ctx, N, &S);
    if (st != TTG_OK) return st;
    if ((st = ttg_sliced_set_matrix(S, d_A, s)) == TTG_OK) st = ttg_sliced_matmul_run(S, d_X, nrhs, d_B, d_Y, mode, s);
    int h_err = 0;
    cudaError_t e = cudaMemcpyAsync(&h_err, S->err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    ttg_sliced_destroy(S);
    if (st != TTG_OK) return st;
    TTG_CUDA_CHECK(e);
    return h_err ? TTG_ETIMEOUT : TTG_OK;
}
