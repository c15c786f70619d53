// ttg_gen.cu — seeded workload inputs built on the device (include/ttg_philox.h).
//
//   ttg_gen_gram_tiles: lower tiles of A = G·Gᵀ/N + αI.  G is the quantised
//     Gaussian (integers in [-127,127], scale 1/16), stored once as int8; each
//     tile entry is an exact int32 dot product (dp4a), divided once by 256·N
//     and shifted by α on the diagonal — the same IEEE operations the oracle
//     performs, so the tiles are bit-identical to the oracle's matrix.
//   ttg_gen_uniform / ttg_gen_normal: dense iid U[-1,1] / N(0,1) arrays.
#include <cuda_runtime.h>

#include <vector>

#include "../../include/ttg.h"
#include "../../include/ttg_philox.h"
#include "ttg_internal.h"

namespace {

// G as row-major int8 (row i = G(i, :)), padded to a multiple of 64 columns.
__global__ void gen_qgauss_kernel(int8_t* G, int N, int ldg, uint32_t seed) {
    const int64_t total = (int64_t)N * N;
    for (int64_t pair = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; 2 * pair < total;
         pair += (int64_t)gridDim.x * blockDim.x) {
        double z[2];
        ttg_normal2((uint64_t)pair, seed, TTG_STREAM_G, &z[0], &z[1]);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int64_t e = 2 * pair + h;  // column-major index of G(i,k)
            if (e >= total) break;
            double t = __dmul_rn(z[h], 16.0);
            t = fmin(fmax(t, -127.0), 127.0);
            const int i = (int)(e % N), k = (int)(e / N);
            G[(int64_t)i * ldg + k] = (int8_t)(int)rint(t);
        }
    }
}

// One 64×64 block of a tile T (ld bi) of A = G·Gᵀ/N + αI: rows r0.. of the
// tile (global row gi0 = first row of the block), columns c0.. (global gj0);
// 256 threads, 4×4 outputs each, K staged 64 bytes (16 words) at a time.
__device__ void gram_block(const int8_t* __restrict__ G, int N, int ldg, int gi0, int gj0, int r0, int c0, int bi, int bj,
                           double alpha, double* T) {
    __shared__ int Gi[64][17];
    __shared__ int Gj[64][17];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    int acc[4][4] = {};
    const int* G32 = reinterpret_cast<const int*>(G);
    const int ldw = ldg / 4;
    for (int k0 = 0; k0 < ldg; k0 += 64) {
        for (int e = threadIdx.x; e < 64 * 16; e += 256) {
            const int r = e / 16, q = e % 16;
            const int gi = gi0 + r, gj = gj0 + r;
            Gi[r][q] = (gi < N && r0 + r < bi) ? G32[(int64_t)gi * ldw + k0 / 4 + q] : 0;
            Gj[r][q] = (gj < N && c0 + r < bj) ? G32[(int64_t)gj * ldw + k0 / 4 + q] : 0;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            int a[4], b[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) a[r] = Gi[tx + 16 * r][q];
#pragma unroll
            for (int c = 0; c < 4; ++c) b[c] = Gj[ty + 16 * c][q];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[r][c] = __dp4a(a[r], b[c], acc[r][c]);
        }
        __syncthreads();
    }
    const double scale = 256.0 * (double)N;
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int lr = r0 + tx + 16 * r, lc = c0 + ty + 16 * c;
            if (lr < bi && lc < bj) {
                double v = __ddiv_rn((double)acc[r][c], scale);
                if (gi0 - r0 + lr == gj0 - c0 + lc) v = __dadd_rn(v, alpha);
                T[lr + (int64_t)lc * bi] = v;
            }
        }
}

// One 64×64 block of the lower tile (ti, tj) from a work list.
__global__ void gram_tiles_kernel(const int8_t* __restrict__ G, int N, int ldg, const int* __restrict__ blk,
                                  const int* __restrict__ displ, const int64_t* __restrict__ off, int nb,
                                  const int* __restrict__ work, int n_work, double alpha, double* tiles) {
    const int w = blockIdx.x;
    if (w >= n_work) return;
    const int ti = work[4 * w + 0], tj = work[4 * w + 1], r0 = work[4 * w + 2], c0 = work[4 * w + 3];
    gram_block(G, N, ldg, displ[ti] + r0, displ[tj] + c0, r0, c0, blk[ti], blk[tj], alpha, tiles + off[ti + (int64_t)tj * nb]);
}

// nrhs × n row block (ld nrhs): element (q, r) = entry (r, q) of the
// column-major n × nrhs N(0,1) array of (seed, stream 1).
__global__ void rhs_rows_kernel(int n, int nrhs, uint32_t seed, double* B) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * nrhs; e += gridDim.x * blockDim.x) {
        const int r = e % n, q = e / n;
        B[q + (int64_t)r * nrhs] = ttg_normal_at((uint64_t)e, seed, TTG_STREAM_RHS);
    }
}

// Uniform tiles of size `tile` (a multiple of 64, or >= N), the last one
// ragged: block (x, y) of the grid is the 64×64 block at global rows 64y,
// columns 64x; blocks above the diagonal tiles return.
__global__ void gram_grid_kernel(const int8_t* __restrict__ G, int N, int ldg, int tile, double alpha, double* tiles) {
    const int gr = blockIdx.y * 64, gc = blockIdx.x * 64;
    const int ti = gr / tile, tj = gc / tile;
    if (ti < tj || gr >= N || gc >= N) return;
    const int nb = (N + tile - 1) / tile;
    auto bs = [&](int i) { return i < nb - 1 ? tile : N - (nb - 1) * tile; };
    const int64_t off = (int64_t)tile * ((int64_t)tj * N - (int64_t)tile * tj * (tj - 1) / 2) + (int64_t)(ti - tj) * tile * bs(tj);
    gram_block(G, N, ldg, gr, gc, gr - ti * tile, gc - tj * tile, bs(ti), bs(tj), alpha, tiles + off);
}

__global__ void gen_uniform_kernel(double* out, int64_t count, uint32_t seed, uint32_t stream) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x)
        out[e] = ttg_uniform_pm1_at((uint64_t)e, seed, stream);
}

__global__ void gen_normal_kernel(double* out, int64_t count, uint32_t seed, uint32_t stream) {
    for (int64_t pair = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; 2 * pair < count;
         pair += (int64_t)gridDim.x * blockDim.x) {
        double z0, z1;
        ttg_normal2((uint64_t)pair, seed, stream, &z0, &z1);
        out[2 * pair] = z0;
        if (2 * pair + 1 < count) out[2 * pair + 1] = z1;
    }
}

// Lower tiles of the miniapp matrix val(i,j) = 1/((i-j)^2+1)
// (2d_cholesky.cpp:133).
__global__ void miniapp_tiles_kernel(const int* __restrict__ blk, const int* __restrict__ displ,
                                     const int64_t* __restrict__ off, int nb, double* tiles) {
    const int ti = blockIdx.y, tj = blockIdx.z;
    if (tj > ti) return;
    const int bi = blk[ti], bj = blk[tj];
    double* T = tiles + off[ti + (int64_t)tj * nb];
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)bi * bj; e += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(e % bi), c = (int)(e / bi);
        const int64_t d = (int64_t)(displ[ti] + r) - (displ[tj] + c);
        T[e] = 1.0 / (double)(d * d + 1);
    }
}

// Block-GEMM inputs in tile layout (tile (i,j) of b×b at (i + j·nb)·b²):
// val_global(i,j) = (i % 49) + 53 (j % 37) for A and B (inputs 0), or iid
// U[-1,1] by global column-major index from streams 2 (A) and 3 (B).
__global__ void gemm_tiles_kernel(int N, int b, int inputs, uint32_t seed, double* A, double* B) {
    const int nb = N / b;
    const int64_t total = (int64_t)N * N;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t tile = t / ((int64_t)b * b), in = t % ((int64_t)b * b);
        const int bi = (int)(tile % nb), bj = (int)(tile / nb);
        const int i = (int)(in % b), j = (int)(in / b);
        const int gi = bi * b + i, gj = bj * b + j;
        if (inputs == 0) {
            const double v = (double)((gi % 49) + (gj % 37) * 53);
            A[t] = v;
            B[t] = v;
        } else {
            const uint64_t e = (uint64_t)gi + (uint64_t)gj * N;
            A[t] = ttg_uniform_pm1_at(e, seed, TTG_STREAM_GEMM_A);
            B[t] = ttg_uniform_pm1_at(e, seed, TTG_STREAM_GEMM_B);
        }
    }
}

}  // namespace

ttg_status ttg_gen_gemm_tiles(ttg_ctx* c, int32_t N, int32_t b, int32_t inputs, uint32_t seed, double* d_A, double* d_B,
                              void* stream) {
    if (!c || N <= 0 || b <= 0 || N % b != 0 || !d_A || !d_B) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(c->device));
    ttg_note_launch();
    gemm_tiles_kernel<<<c->sms * 8, 256, 0, (cudaStream_t)stream>>>(N, b, inputs, seed, d_A, d_B);
    TTG_CUDA_CHECK(cudaGetLastError());
    TTG_CUDA_CHECK(cudaStreamSynchronize((cudaStream_t)stream));
    return TTG_OK;
}

ttg_status ttg_gen_miniapp_tiles(ttg_ctx* c, const int32_t* h_bs, int32_t nb, double* d_tiles, void* stream) {
    if (!c || nb <= 0 || !h_bs || !d_tiles) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(c->device));
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<int> displ(nb + 1, 0);
    for (int i = 0; i < nb; ++i) displ[i + 1] = displ[i] + h_bs[i];
    std::vector<int64_t> off((size_t)nb * nb, 0);
    ttg_tile_layout(h_bs, nb, off.data());
    int *d_blk = nullptr, *d_displ = nullptr;
    int64_t* d_off = nullptr;
    TTG_CUDA_CHECK(cudaMallocAsync((void**)&d_blk, sizeof(int) * nb, s));
    TTG_CUDA_CHECK(cudaMallocAsync((void**)&d_displ, sizeof(int) * (nb + 1), s));
    TTG_CUDA_CHECK(cudaMallocAsync((void**)&d_off, sizeof(int64_t) * nb * nb, s));
    TTG_CUDA_CHECK(cudaMemcpyAsync(d_blk, h_bs, sizeof(int) * nb, cudaMemcpyHostToDevice, s));
    TTG_CUDA_CHECK(cudaMemcpyAsync(d_displ, displ.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice, s));
    TTG_CUDA_CHECK(cudaMemcpyAsync(d_off, off.data(), sizeof(int64_t) * nb * nb, cudaMemcpyHostToDevice, s));
    dim3 grid(8, nb, nb);
    ttg_note_launch();
    miniapp_tiles_kernel<<<grid, 256, 0, s>>>(d_blk, d_displ, d_off, nb, d_tiles);
    TTG_CUDA_CHECK(cudaGetLastError());
    TTG_CUDA_CHECK(cudaStreamSynchronize(s));
    cudaFreeAsync(d_blk, s);
    cudaFreeAsync(d_displ, s);
    cudaFreeAsync(d_off, s);
    return TTG_OK;
}

extern "C" ttg_status ttg_gen_gram_tiles(ttg_ctx* c, int32_t n, const int32_t* h_bs, int32_t nb, double alpha,
                                         uint32_t seed, double* d_tiles, void* stream) {
    if (!c || n <= 0 || nb <= 0 || !h_bs || !d_tiles) return TTG_EINVAL;
    int64_t sum = 0;
    for (int i = 0; i < nb; ++i) {
        if (h_bs[i] < 0) return TTG_EINVAL;
        sum += h_bs[i];
    }
    // int32 dot products of N values in [-127,127] stay below 2^31 up to N = 131072.
    if (sum != n || n > 131072) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(c->device));
    cudaStream_t s = (cudaStream_t)stream;
    const int ldg = (n + 63) / 64 * 64;
    std::vector<int> displ(nb + 1, 0);
    for (int i = 0; i < nb; ++i) displ[i + 1] = displ[i] + h_bs[i];
    std::vector<int64_t> off((size_t)nb * nb, 0);
    ttg_tile_layout(h_bs, nb, off.data());
    std::vector<int> work;
    for (int tj = 0; tj < nb; ++tj)
        for (int ti = tj; ti < nb; ++ti)
            for (int c0 = 0; c0 < h_bs[tj]; c0 += 64)
                for (int r0 = 0; r0 < h_bs[ti]; r0 += 64) {
                    work.push_back(ti);
                    work.push_back(tj);
                    work.push_back(r0);
                    work.push_back(c0);
                }
    const int n_work = (int)(work.size() / 4);
    int8_t* G = nullptr;
    int *d_blk = nullptr, *d_displ = nullptr, *d_work = nullptr;
    int64_t* d_off = nullptr;
    ttg_status st = TTG_OK;
    auto fail = [&](cudaError_t e, const char* what) {
        ttg_set_last_cuda_error(e, what, __FILE__, __LINE__);
        st = e == cudaErrorMemoryAllocation ? TTG_ENOMEM : TTG_ECUDA;
    };
    cudaError_t e;
    if ((e = cudaMallocAsync((void**)&G, (size_t)n * ldg, s)) != cudaSuccess) fail(e, "alloc G");
    if (st == TTG_OK && (e = cudaMallocAsync((void**)&d_blk, sizeof(int) * nb, s)) != cudaSuccess) fail(e, "alloc");
    if (st == TTG_OK && (e = cudaMallocAsync((void**)&d_displ, sizeof(int) * (nb + 1), s)) != cudaSuccess) fail(e, "alloc");
    if (st == TTG_OK && (e = cudaMallocAsync((void**)&d_off, sizeof(int64_t) * nb * nb, s)) != cudaSuccess) fail(e, "alloc");
    if (st == TTG_OK && (e = cudaMallocAsync((void**)&d_work, sizeof(int) * std::max<size_t>(4, work.size()), s)) != cudaSuccess)
        fail(e, "alloc");
    if (st == TTG_OK) {
        cudaMemsetAsync(G, 0, (size_t)n * ldg, s);
        cudaMemcpyAsync(d_blk, h_bs, sizeof(int) * nb, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(d_displ, displ.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(d_off, off.data(), sizeof(int64_t) * nb * nb, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(d_work, work.data(), sizeof(int) * work.size(), cudaMemcpyHostToDevice, s);
        ttg_note_launch();
        gen_qgauss_kernel<<<c->sms * 8, 256, 0, s>>>(G, n, ldg, seed);
        if (n_work > 0) {
            ttg_note_launch();
            gram_tiles_kernel<<<n_work, 256, 0, s>>>(G, n, ldg, d_blk, d_displ, d_off, nb, d_work, n_work, alpha, d_tiles);
        }
        if ((e = cudaGetLastError()) != cudaSuccess) fail(e, "gram kernels");
        // Host vectors above must outlive the async copies.
        if (st == TTG_OK && (e = cudaStreamSynchronize(s)) != cudaSuccess) fail(e, "sync");
    }
    if (G) cudaFreeAsync(G, s);
    if (d_blk) cudaFreeAsync(d_blk, s);
    if (d_displ) cudaFreeAsync(d_displ, s);
    if (d_off) cudaFreeAsync(d_off, s);
    if (d_work) cudaFreeAsync(d_work, s);
    return st;
}

extern "C" ttg_status ttg_gen_uniform(ttg_ctx* c, int64_t count, uint32_t seed, uint32_t stream_id, double* d_out,
                                      void* stream) {
    if (!c || count < 0 || (count > 0 && !d_out)) return TTG_EINVAL;
    if (count == 0) return TTG_OK;
    TTG_CUDA_CHECK(cudaSetDevice(c->device));
    ttg_note_launch();
    gen_uniform_kernel<<<c->sms * 8, 256, 0, (cudaStream_t)stream>>>(d_out, count, seed, stream_id);
    TTG_CUDA_CHECK(cudaGetLastError());
    return TTG_OK;
}

extern "C" ttg_status ttg_gen_normal(ttg_ctx* c, int64_t count, uint32_t seed, uint32_t stream_id, double* d_out,
                                     void* stream) {
    if (!c || count < 0 || (count > 0 && !d_out)) return TTG_EINVAL;
    if (count == 0) return TTG_OK;
    TTG_CUDA_CHECK(cudaSetDevice(c->device));
    ttg_note_launch();
    gen_normal_kernel<<<c->sms * 8, 256, 0, (cudaStream_t)stream>>>(d_out, count, seed, stream_id);
    TTG_CUDA_CHECK(cudaGetLastError());
    return TTG_OK;
}

ttg_status ttg_gen_gram_async(ttg_ctx* c, int n, int tile, double alpha, uint32_t seed, double* d_tiles, cudaStream_t s) {
    if (!c || n <= 0 || n > 131072 || tile <= 0 || (tile < n && tile % 64 != 0) || !d_tiles) return TTG_EINVAL;
    const int ldg = (n + 63) / 64 * 64;
    int8_t* G = nullptr;
    TTG_CUDA_CHECK(cudaMallocAsync((void**)&G, (size_t)n * ldg, s));
    TTG_CUDA_CHECK(cudaMemsetAsync(G, 0, (size_t)n * ldg, s));
    ttg_note_launch();
    gen_qgauss_kernel<<<c->sms * 8, 256, 0, s>>>(G, n, ldg, seed);
    const int nB = (n + 63) / 64;
    ttg_note_launch();
    gram_grid_kernel<<<dim3(nB, nB), 256, 0, s>>>(G, n, ldg, tile < n ? tile : n, alpha, d_tiles);
    TTG_CUDA_CHECK(cudaGetLastError());
    TTG_CUDA_CHECK(cudaFreeAsync(G, s));
    return TTG_OK;
}

ttg_status ttg_gen_preload() {
    cudaFuncAttributes fa;
    TTG_CUDA_CHECK(cudaFuncGetAttributes(&fa, gen_qgauss_kernel));
    TTG_CUDA_CHECK(cudaFuncGetAttributes(&fa, gram_grid_kernel));
    TTG_CUDA_CHECK(cudaFuncGetAttributes(&fa, rhs_rows_kernel));
    return TTG_OK;
}

ttg_status ttg_gen_rhs_rows_async(int n, int nrhs, uint32_t seed, double* d_B, cudaStream_t s) {
    if (n <= 0 || nrhs < 1 || !d_B) return TTG_EINVAL;
    ttg_note_launch();
    rhs_rows_kernel<<<std::min(1024, (n * nrhs + 255) / 256), 256, 0, s>>>(n, nrhs, seed, d_B);
    TTG_CUDA_CHECK(cudaGetLastError());
    return TTG_OK;
}

