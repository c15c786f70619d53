// ttg_sliced_api.h — internal interface of the FP64-accurate tensor-core
// product Y = Aᵀ·X (= A·X for the symmetric matrices of the solver) from
// sliced digits (ttg_sliced.cu, sliced_matmul_tc.cuh).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "../../include/ttg.h"

struct ttg_sliced;

// Buffers for an N×N matrix: 8 BF16 digit slices (16·N² bytes), the digits of
// up to 16 right-hand sides, the partial sums.
ttg_status ttg_sliced_create(ttg_ctx* ctx, int N, ttg_sliced** out);
void ttg_sliced_destroy(ttg_sliced* S);
// Device bytes of the digit slices of an N×N matrix.
size_t ttg_sliced_bytes(int N);
// Digits of dense column-major A (column i is used as row i), on stream s.
ttg_status ttg_sliced_set_matrix(ttg_sliced* S, const double* dA, cudaStream_t s);
// mode 0: Y = A·X; mode 2: Y = B − A·X (N×nrhs column-major, ld N), on s.
ttg_status ttg_sliced_matmul_run(ttg_sliced* S, const double* X, int nrhs, const double* B, double* Y, int mode, cudaStream_t s);
// Device flag set when a bounded wait of the product kernel gave up (kept
// across products until reset).
int* ttg_sliced_err(ttg_sliced* S);
ttg_status ttg_sliced_reset_err(ttg_sliced* S, cudaStream_t s);
