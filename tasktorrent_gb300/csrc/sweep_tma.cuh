// sweep_tma.cuh — the FP32 block sweeps (the preconditioner M⁻¹ = L̃⁻ᵀL̃⁻¹
// of the refinement) with every item's factor strip staged by TMA.
//
// Same work items, waits and flags as sweep_kernel<float, float>
// (solve_kernels.cuh): an item is out[strip] (=, or -=) M[strip, 0:kc] ·
// V[0:kc, 0:nrhs] for a 64-row strip.  Items are claimed in the order the
// host builds (SweepArgs::order: each step's chain items ahead of the
// previous step's bulk; N = 32768, tile 512: 1.67 -> 1.51 ms per sweep).
// The other difference is how M reaches the SM.  The generic kernel streams it through registers and keeps ~16 KB of
// loads in flight per block, which left each item at ~15 µs (a 128 KB strip
// at ~10 GB/s per block).  Here one thread issues the whole strip as TMA
// boxes of 64 rows × 128 columns as soon as the item is claimed — the factor
// is complete, so the copy does not wait for the item's inputs — and the
// block stages V and computes from shared memory: warp w takes a quarter of
// the columns (w / 2) and eight right-hand sides (w % 2), lane l rows 2l and
// 2l+1, and the four column quarters are added in order.
//
// Uniform tiles only, edge b a multiple of 128 and at most 512 (the tile
// rows are the inner dimension of each 2D tensor map: element (r, c) of an
// operand at element offset o, a multiple of b, is (row r, column o/b + c)).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "solve_kernels.cuh"
#include "tile_bf16_tc.cuh"

namespace ttg {
namespace solve {

constexpr int kTmaCols = 128;                          // columns per TMA box
constexpr int kTmaMaxK = 512;                          // largest tile edge
constexpr int kTmaMBytes = kStrip * kTmaMaxK * 4;      // 128 KB: the strip of M
constexpr int kTmaVLd = 20;                            // floats per staged V column (16 + pad)
constexpr int kTmaVBytes = kTmaMaxK * kTmaVLd * 4;     // 40 KB
constexpr int kTmaSmem = kTmaMBytes + kTmaVBytes + 128 + 128;  // + barrier + alignment

// The three operand arrays of one sweep direction as 2D FP32 tensor maps
// (inner dimension: the b rows of a tile; box 64 × kTmaCols).
struct SweepMaps {
    CUtensorMap mu;  // off-diagonal tiles (forward L_ki, backward L_ikᵀ)
    CUtensorMap md;  // inverted diagonal tiles (forward L_ii⁻¹, backward L_ii⁻ᵀ)
    CUtensorMap wd;  // folded products W_i
    int b;           // uniform tile edge
};

__device__ __forceinline__ void tma_load_2d_f32(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            tc::smem_u32(dst)),
        "l"((uint64_t)map), "r"(tc::smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

__global__ void __launch_bounds__(256, 1) sweep_kernel_f32_tma(SweepArgs a, const __grid_constant__ SweepMaps maps, float* Vin,
                                                               float* Vout) {
    extern __shared__ unsigned char tma_smem_raw[];
    unsigned char* base = (unsigned char*)(((uintptr_t)tma_smem_raw + 127) & ~(uintptr_t)127);
    float* Ms = (float*)base;                               // [kc][64]
    float* Vs = (float*)(base + kTmaMBytes);                // [kc][kTmaVLd]
    uint64_t* bar = (uint64_t*)(base + kTmaMBytes + kTmaVBytes);
    __shared__ int s_item, s_abort;
    const int nb = a.nb, N = a.N, b = maps.b;
    const int total = a.step_start[nb];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    auto row_of = [&](int step) { return a.backward ? nb - 1 - step : step; };
    auto strips = [&](int row) { return a.strip_pre[row + 1] - a.strip_pre[row]; };
    if (threadIdx.x == 0) {
        tc::mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        tc::fence_proxy_async_smem();
    }
    __syncthreads();
    uint32_t phase = 0;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            const int k = atomicAdd(a.claim, 1);
            s_item = k < total ? __ldg(a.order + k) : total;
        }
        __syncthreads();
        const int it = s_item;
        if (it >= total) break;
        if (a.trace && threadIdx.x == 0) a.trace[4 * (size_t)it] = sweep_clock();
        const int s = upper_index(a.step_start, nb, it);
        const int i = row_of(s);
        int u = it - a.step_start[s];
        const int Si = strips(i);
        int kind, k, g;
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
                const int skip = a.fold ? 1 : 0;
                g = a.backward ? a.strip_pre[i - skip] - 1 - u : a.strip_pre[i + 1 + skip] + u;
                k = upper_index(a.strip_pre, nb, g);
            }
        }
        const int p = s > 0 ? row_of(s - 1) : -1;
        const int r0 = (g - a.strip_pre[k]) * kStrip;
        // The item's operand (map, element offset), inner size, vector and output.
        const CUtensorMap* map;
        int64_t o;
        const float* V;
        float* out;
        int mode;
        if (kind == 0 && a.fold && s > 0) {
            map = &maps.wd;
            o = a.woff[i];
            V = Vout + a.displ[p];
            out = Vout + a.displ[i] + r0;
            mode = 1;
        } else if (kind == 0) {
            map = &maps.md;
            o = a.doff[i];
            V = Vin + a.displ[i];
            out = Vout + a.displ[i] + r0;
            mode = 0;
        } else if (kind == 1) {
            map = &maps.md;
            o = a.doff[k];
            V = Vin + a.displ[k];
            out = Vout + a.displ[k] + r0;
            mode = 0;
        } else {
            map = &maps.mu;
            o = a.backward ? a.off[i + (size_t)k * nb] : a.off[k + (size_t)i * nb];
            V = Vout + a.displ[i];
            out = Vin + a.displ[k] + r0;
            mode = 1;
        }
        const int kc = b;
        // The strip of M: the factor is complete, so its copy starts now.
        if (threadIdx.x == 0) {
            tc::mbar_expect_tx(bar, (uint32_t)(kStrip * kc * 4));
            const int col = (int)(o / b);
            for (int c0 = 0; c0 < kc; c0 += kTmaCols) tma_load_2d_f32(Ms + (size_t)c0 * kStrip, map, bar, r0, col + c0);
        }
        // Wait for the inputs of this item (as sweep_kernel).
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
            if (abort) tc::mbar_wait(bar, phase, a.timeout_ns);  // the strip's copy lands before the block leaves
        }
        __syncthreads();
        if (s_abort) break;
        // Stage V[0:kc, 0:16] (columns q >= nrhs as zeros), four right-hand
        // sides of one row per thread, all loads in flight together.
        {
            constexpr int kPer = kTmaMaxK * 4 / 256;  // float4 groups per thread at kc = 512
            float4 tmp[kPer];
#pragma unroll
            for (int j = 0; j < kPer; ++j) {
                const int e = threadIdx.x + 256 * j;  // e = qq·kc + c
                const int c = e % kc, qq = e / kc;
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (qq < 4) {
                    const int q0 = 4 * qq;
                    if (q0 + 0 < a.nrhs) v.x = ldcg(V + c + (size_t)(q0 + 0) * N);
                    if (q0 + 1 < a.nrhs) v.y = ldcg(V + c + (size_t)(q0 + 1) * N);
                    if (q0 + 2 < a.nrhs) v.z = ldcg(V + c + (size_t)(q0 + 2) * N);
                    if (q0 + 3 < a.nrhs) v.w = ldcg(V + c + (size_t)(q0 + 3) * N);
                }
                tmp[j] = v;
            }
#pragma unroll
            for (int j = 0; j < kPer; ++j) {
                const int e = threadIdx.x + 256 * j;
                const int c = e % kc, qq = e / kc;
                if (qq < 4) *(float4*)(Vs + c * kTmaVLd + 4 * qq) = tmp[j];
            }
        }
        // Earlier outputs of mode 1 (read before this item writes them).
        float prev[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int e = threadIdx.x + 256 * j;
            const int r = e & (kStrip - 1), q = e >> 6;
            prev[j] = (mode != 0 && q < a.nrhs) ? ldcg(out + r + (size_t)q * N) : 0.f;
        }
        __syncthreads();
        // Every thread waits for the strip (the barrier's completion makes the
        // copy visible to it); a timeout anywhere ends the block, uniformly.
        const int late = __syncthreads_or(tc::mbar_wait(bar, phase, a.timeout_ns) ? 0 : 1);
        if (late) {
            if (threadIdx.x == 0) atomicCAS(a.err, 0, 1);
            break;  // other blocks see the error flag
        }
        phase ^= 1;
        // out = Σ_c M[:, c] V[c, :]: warp w, quarter w/2 of the columns, RHS
        // 8·(w%2) … +7; lane l, rows 2l and 2l+1.
        const int kq = warp >> 1, qg = warp & 1;
        float acc0[8], acc1[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) acc0[q] = acc1[q] = 0.f;
        const int cpart = kc / 4;
#pragma unroll 4
        for (int c = kq * cpart; c < (kq + 1) * cpart; ++c) {
            const float2 m = *(const float2*)(Ms + (size_t)c * kStrip + 2 * lane);
            const float4 v0 = *(const float4*)(Vs + c * kTmaVLd + 8 * qg);
            const float4 v1 = *(const float4*)(Vs + c * kTmaVLd + 8 * qg + 4);
            const float vv[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                acc0[q] = fmaf(m.x, vv[q], acc0[q]);
                acc1[q] = fmaf(m.y, vv[q], acc1[q]);
            }
        }
        __syncthreads();  // every warp is done with Ms: reuse it for the partials
        float* Ps = Ms;   // [kq][q][row]
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            Ps[((size_t)kq * kMaxRhs + 8 * qg + q) * kStrip + 2 * lane] = acc0[q];
            Ps[((size_t)kq * kMaxRhs + 8 * qg + q) * kStrip + 2 * lane + 1] = acc1[q];
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int e = threadIdx.x + 256 * j;
            const int r = e & (kStrip - 1), q = e >> 6;
            if (q >= a.nrhs) continue;
            float sum = 0.f;
#pragma unroll
            for (int w = 0; w < 4; ++w) sum += Ps[((size_t)w * kMaxRhs + q) * kStrip + r];
            out[r + (size_t)q * N] = mode == 0 ? sum : prev[j] - sum;
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

}  // namespace solve
}  // namespace ttg
