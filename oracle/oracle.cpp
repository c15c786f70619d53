/*
 * oracle.cpp — TEST INFRASTRUCTURE ONLY.  liboracle.so: the CPU oracle of the
 * tiled Cholesky and 2D block GEMM task graphs.  The graphs (dag.hpp) run on
 * a restatement of the reference's shared-memory runtime (runtime.hpp) with
 * CBLAS/LAPACKE tile math (oracle_blas.h).  Only tests/, the smoke check and
 * bench.py's CPU legs may load this library; the product never does.
 */
#include "dag.hpp"
#include "runtime.hpp"

extern "C" {

const char* orc_blas_name(void) { return orc::blas().name.c_str(); }

int orc_cholesky(const orc_chol_args* a, orc_chol_out* out) { return orc::cholesky_run<orc::Threadpool, orc::Taskflow>(a, out); }

int orc_gemm(const orc_gemm_args* a, orc_gemm_out* out) { return orc::gemm_run<orc::Threadpool, orc::Taskflow>(a, out); }

void orc_gen_gram(int N, double alpha, uint32_t seed, double* A) { orc::gen_gram(N, alpha, seed, A); }

int orc_block_sizes(int block_size, int num_blocks, int upper_block_size, int* sizes) {
    return orc::block_sizes(block_size, num_blocks, upper_block_size, sizes);
}

void orc_gemm_inputs(int N, int inputs, uint32_t seed, double* A, double* B) {
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
            const size_t e = i + (size_t)j * N;
            if (inputs == 0) {
                if (A) A[e] = orc::val_global(i, j);
                if (B) B[e] = orc::val_global(i, j);
            } else {
                if (A) A[e] = ttg_uniform_pm1_at(e, seed, TTG_STREAM_GEMM_A);
                if (B) B[e] = ttg_uniform_pm1_at(e, seed, TTG_STREAM_GEMM_B);
            }
        }
}

void orc_normals(uint64_t first, int count, uint32_t seed, uint32_t stream, double* out) {
    for (int i = 0; i < count; ++i) out[i] = ttg_normal_at(first + i, seed, stream);
}

void orc_uniforms(uint64_t first, int count, uint32_t seed, uint32_t stream, double* out) {
    for (int i = 0; i < count; ++i) out[i] = ttg_uniform_pm1_at(first + i, seed, stream);
}

void orc_qnormals(uint64_t first, int count, uint32_t seed, uint32_t stream, int* out) {
    for (int i = 0; i < count; ++i) out[i] = ttg_qnormal_at(first + i, seed, stream);
}

/* One entry of A = G·Gᵀ/N + αI (the definition gen_gram computes for the
 * whole matrix): an exact integer dot product of rows i and j of G. */
double orc_gram_entry(int N, int i, int j, double alpha, uint32_t seed) {
    int64_t s = 0;
    for (int k = 0; k < N; ++k)
        s += (int64_t)ttg_qnormal_at(i + (uint64_t)k * N, seed, TTG_STREAM_G) *
             ttg_qnormal_at(j + (uint64_t)k * N, seed, TTG_STREAM_G);
    double v = (double)s / (256.0 * (double)N);
    if (i == j) v = v + alpha;
    return v;
}

void orc_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
    ttg_u32x4 c;
    for (int i = 0; i < 4; ++i) c.v[i] = ctr[i];
    ttg_u32x4 r = ttg_philox4x32_10(c, key[0], key[1]);
    for (int i = 0; i < 4; ++i) out[i] = r.v[i];
}

}  // extern "C"
