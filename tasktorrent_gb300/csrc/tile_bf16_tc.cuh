// tile_bf16_tc.cuh — BF16 trailing update of the mixed Cholesky on the
// 5th-generation tensor cores (tcgen05), run by one block of the persistent
// executor.
//
//   C[m0:m0+128, n0:n0+256] += f · Â[m0:m0+128, :] · B̂[n0:n0+256, :]ᵀ
//
// C is an FP32 working tile (column-major, in HBM).  Â and B̂ are BF16 copies
// of factored panel tiles (L_ik, L_jk), stored K-major (row-major) one slot
// per tile and scaled by a power of two per tile; f = -s_A·s_B undoes the
// scales.  This is the cblas_dgemm(NoTrans, Trans) / cblas_dsyrk trailing
// update of 2d_cholesky.cpp:490-494 in the mixed-precision path.
//
// Data movement and compute:
//   - one thread issues TMA loads (cp.async.bulk.tensor.3d, 64B swizzle) of
//     32-wide K slabs into a 9-slot shared-memory ring guarded by mbarriers;
//   - one thread issues tcgen05.mma.cta_group::1.kind::f16 (M=128, N=256,
//     K=16; BF16 inputs, FP32 accumulator in 256 TMEM columns) and commits
//     each stage back to the producer with tcgen05.commit;
//   - warps 4-7 read the accumulator with tcgen05.ld.32x32b.x32 (warp w reads
//     TMEM lanes 32·(w-4)…) and update C, while the MMAs of the next output
//     block run into the other of two accumulators (512 TMEM columns).
// Every wait is bounded: on timeout the block records an error and drains.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace ttg {
namespace tc {

constexpr int kBM = 128;           // accumulator rows (TMEM lanes)
constexpr int kBN = 256;           // accumulator columns
constexpr int kBK = 32;            // K per slot (one 64-byte swizzle row of BF16)
// The ring holds kSlots slots of one K slab each: A (128 rows) then B (256
// rows) of one BF16 slice.  A plain BF16 K step takes one slot; a split K
// step takes three consecutive slots (hi, mid, lo) and issues all six slice
// products from them, so each slice is loaded once per K step.
constexpr int kSlots = 9;
constexpr int kSlotBytesA = kBM * kBK * 2;        // 8 KB
constexpr int kSlotBytesB = kBN * kBK * 2;        // 16 KB
constexpr int kSlotBytes = kSlotBytesA + kSlotBytesB;
constexpr int kSmemBytes = kSlots * kSlotBytes + 1024;  // 217 KB + alignment slack
constexpr uint32_t kTmemCols = 512;  // two 256-column accumulators (double buffer)

// Per-block state kept in shared memory across tasks.
struct TcShared {
    uint64_t full[kSlots];
    uint64_t empty[kSlots];
    uint64_t accf[2];    // accumulator b complete (tcgen05.commit of the MMA thread)
    uint64_t afree[2];   // accumulator b drained (the epilogue warps)
    uint32_t tmem_base;
    uint32_t produced;   // stages produced (producer thread)
    uint32_t consumed;   // stages consumed (MMA thread)
    uint32_t nacc;       // output blocks accumulated so far (all threads read)
    int failed;          // a bounded wait gave up in this block
    int ep_ok;           // the epilogue's accumulator is complete (warps 4-7)
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ long long tc_globaltimer() {
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for `parity` with a time limit; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = tc_globaltimer();
    for (uint32_t it = 0;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 255) == 255 && tc_globaltimer() - t0 > limit_ns) return false;
    }
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(
            smem_u32(dst)),
        "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
        : "memory");
}

__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Whole warp: allocate kTmemCols TMEM columns, address written to *dst.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(kTmemCols) : "memory");
}

// Instruction descriptor, kind::f16: FP32 accumulator (bits 4-5 = 1), A and B
// BF16 (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N>>3 at
// bits 17-22, M>>4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// The same with FP16 A and B (bits 7-9 and 10-12 = 0).
__host__ __device__ constexpr uint32_t idesc_f16_f32(int M, int N) {
    return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Shared-memory descriptor of a K-major, 64B-swizzled operand whose rows are
// 64 bytes and whose 8-row groups are 512 bytes apart: start address >> 4
// (bits 0-13), leading offset (unused for this layout, 1), stride offset
// 512 >> 4 (bits 32-45), version 1 (bits 46-47), layout SWIZZLE_64B = 4
// (bits 61-63).
__device__ __forceinline__ uint64_t smem_desc_kmajor_sw64(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)1 << 16) | ((uint64_t)(512 >> 4) << 32) | ((uint64_t)1 << 46) |
           ((uint64_t)4 << 61);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Named barrier 1 over the 128 threads of warps 4-7 (the epilogue warpgroup).
__device__ __forceinline__ void epilogue_bar() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, "
        "%17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
}

// Block setup (all threads): barriers and TMEM.  Call once per kernel.
__device__ inline void tc_setup(TcShared* sh) {
    if (threadIdx.x == 0) {
        for (int s = 0; s < kSlots; ++s) {
            mbar_init(&sh->full[s], 1);
            mbar_init(&sh->empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&sh->accf[b], 1);
            mbar_init(&sh->afree[b], 1);
        }
        sh->produced = 0;
        sh->consumed = 0;
        sh->nacc = 0;
        sh->failed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        fence_proxy_async_smem();
    }
    __syncwarp();
    if (threadIdx.x < 32) tmem_alloc(&sh->tmem_base);  // warp 0, converged
    __syncthreads();
    tc_fence_after();
}

// Block teardown (all threads, after the last task).  After a timeout, the
// loads that were issued but never consumed are waited for (bounded) so no
// copy lands in shared memory after the block exits; TMEM is always freed.
__device__ inline void tc_teardown(TcShared* sh, long long limit_ns) {
    if (threadIdx.x == 0 && sh->failed) {
        for (uint32_t p = sh->consumed; p < sh->produced; ++p)
            if (!mbar_wait(&sh->full[p % kSlots], (p / kSlots) & 1, limit_ns)) break;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x < 32) tmem_dealloc(sh->tmem_base);
}

// One 128×256 block of C += f·Â·B̂ᵀ over K = k (multiple of 64).  All
// threads of the block call it; returns false if a wait timed out.
// lower: only elements with (row0 + r) >= (col0 + c) are updated.
// Slice pairs of a split product (slice 0 = hi, 1 = mid, 2 = lo of each
// operand): the six products whose terms reach 2^-16 of hi·hi, smallest
// first — mid·mid, hi·lo, lo·hi, hi·mid, mid·hi, hi·hi.
__device__ __forceinline__ int split_pair_a(int p) { return p == 0 ? 1 : (p == 2 ? 2 : (p == 4 ? 1 : 0)); }
__device__ __forceinline__ int split_pair_b(int p) { return p == 0 ? 1 : (p == 1 ? 2 : (p == 3 ? 1 : 0)); }
// Split FP16 (slice 0 = hi, 1 = lo·2^11): hi·lo, lo·hi into the small
// accumulator (scaled by 2^11), hi·hi last.
__device__ __forceinline__ int f16_pair_a(int p) { return p == 1 ? 1 : 0; }
__device__ __forceinline__ int f16_pair_b(int p) { return p == 0 ? 1 : 0; }

// Number of 128×256 output blocks of an m×n tile (lower: blocks that meet
// the lower triangle of a square tile), and the coordinates of block b.
__device__ __forceinline__ int tc_num_blocks(int m, int n, bool lower) {
    const int bm = (m + kBM - 1) / kBM, bn = (n + kBN - 1) / kBN;
    if (!lower) return bm * bn;
    int cnt = 0;
    for (int j = 0; j < bn; ++j)
        for (int i = 0; i < bm; ++i)
            if (i * kBM + kBM - 1 >= j * kBN) ++cnt;
    return cnt;
}

__device__ __forceinline__ void tc_block_coords(int b, int m, int n, bool lower, int* row0, int* col0) {
    const int bm = (m + kBM - 1) / kBM, bn = (n + kBN - 1) / kBN;
    int cnt = 0;
    for (int j = 0; j < bn; ++j)
        for (int i = 0; i < bm; ++i) {
            if (lower && i * kBM + kBM - 1 < j * kBN) continue;
            if (cnt == b) {
                *row0 = i * kBM;
                *col0 = j * kBN;
                return;
            }
            ++cnt;
        }
    *row0 = 0;
    *col0 = 0;
}

// C[block] += f · Σ A_slotA · B_slotBᵀ for the output blocks b0 .. b0+nblk-1
// of the tile (tc_block_coords order).  split = 1: one BF16 product; split =
// 3: the operands are stored as three BF16 slices (slot + s·stride, s = 0,
// 1, 2) and the six products of split_pair_* accumulate in the same FP32
// TMEM accumulator, which gives FP32-level accuracy.
//
// Roles: thread 0 loads the K slabs of every block into the ring (TMA),
// thread 32 issues the MMAs, warps 2-3 prefetch the C blocks into L2, and
// warps 4-7 (one warpgroup: TMEM lanes 32·(w-4)…) drain the accumulators
// into C.  Plain BF16: consecutive blocks alternate between the two
// 256-column accumulators, so block j's epilogue runs while block j+1's MMAs
// do.  Split: hi·hi accumulates in columns 0-255 and the five smaller
// products in columns 256-511, added in the epilogue — the small terms are
// not rounded against the large accumulator (a K step issues all six
// products), which keeps the update FP32-accurate.  accf[b] says buffer b is
// complete, afree[b] that it has been read.  All threads call it; returns
// false if a wait timed out.
// One instantiation per split (its slot and product counts are constants),
// each compiled out of line: its registers and schedule do not depend on the
// rest of the executor kernel.
template <int SPLIT>
static __device__ __noinline__ bool tc_gemm_blocks_t(TcShared* sh, uint8_t* ring, const CUtensorMap* map, int slotA, int slotB, int b0,
                                                     int nblk, int k, float f, float* C, int ldc, int m, int n, bool lower,
                                                     long long limit_ns, int stride) {
    constexpr int split = SPLIT;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ksteps = k / kBK;
    constexpr int nsl = split;  // slots (slices) per K step: 1, 2 (split FP16) or 3 (split BF16)
    constexpr int npairs = split == 3 ? 6 : (split == 2 ? 3 : 1);
    const int total = nsl * ksteps;      // slots per output block
    const uint32_t base = sh->nacc;
    const bool ok = !sh->failed;
    constexpr bool dbl = split == 1;  // double-buffered accumulators
    auto buf_of = [&](uint32_t gi) { return dbl ? (int)(gi & 1) : 0; };
    auto use_of = [&](uint32_t gi) { return dbl ? (gi >> 1) : gi; };
    if (warp == 2 || warp == 3) {
        // Bring the C blocks into L2 (one 128-byte line per 32 rows of a
        // column) so that the epilogue's reads hit.
        for (int j = 0; j < nblk; ++j) {
            int row0, col0;
            tc_block_coords(b0 + j, m, n, lower, &row0, &col0);
            const int rows = min(kBM, m - row0), lines = (rows + 31) >> 5;
            for (int e = threadIdx.x - 64; e < kBN * lines; e += 64) {
                const int c = e / lines, gc = col0 + c, gr = row0 + 32 * (e % lines);
                if (gc < n && (!lower || row0 + rows - 1 >= gc))
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(__cvta_generic_to_global(C + gr + (size_t)gc * ldc)));
            }
        }
    } else if (threadIdx.x == 0 && ok) {
        // Producer: K slabs of A (128 rows) and B (two boxes of 128 rows).
        fence_proxy_async_global();  // panel tiles were written by other blocks' generic stores
        uint32_t p = sh->produced;
        for (int j = 0; j < nblk && !sh->failed; ++j) {
            int row0, col0;
            tc_block_coords(b0 + j, m, n, lower, &row0, &col0);
            for (int g = 0; g < total; ++g, ++p) {
                const int ks = g / nsl, sl = g % nsl;  // K step, slice
                const int s = p % kSlots;
                if (!mbar_wait(&sh->empty[s], ((p / kSlots) & 1) ^ 1, limit_ns)) {
                    sh->failed = 1;
                    break;
                }
                uint8_t* st = ring + (size_t)s * kSlotBytes;
                mbar_expect_tx(&sh->full[s], kSlotBytes);
                tma_load_3d(st, map, &sh->full[s], ks * kBK, row0, slotA + sl * stride);
                tma_load_3d(st + kSlotBytesA, map, &sh->full[s], ks * kBK, col0, slotB + sl * stride);
                tma_load_3d(st + kSlotBytesA + kSlotBytesB / 2, map, &sh->full[s], ks * kBK, col0 + 128, slotB + sl * stride);
            }
        }
        sh->produced = p;
    } else if (threadIdx.x == 32 && ok) {
        // MMA issuer.
        const uint32_t idesc = split == 2 ? idesc_f16_f32(kBM, kBN) : idesc_bf16_f32(kBM, kBN);
        const uint32_t ring_u32 = smem_u32(ring);
        uint32_t c = sh->consumed;
        bool good = true;
        for (int j = 0; j < nblk && good; ++j) {
            const uint32_t gi = base + j;
            const int buf = buf_of(gi);
            // The accumulator's previous block must have been drained.
            if (!mbar_wait(&sh->afree[buf], (use_of(gi) & 1) ^ 1, limit_ns)) {
                sh->failed = 1;
                good = false;
                break;
            }
            tc_fence_after();
            const uint32_t dacc = sh->tmem_base + (uint32_t)(kBN * buf);
            const uint32_t dsmall = sh->tmem_base + (uint32_t)kBN;  // split: the five smaller products
            for (int ks = 0; ks < ksteps && good; ++ks, c += nsl) {
                // The K step's slots (one per slice) must all be loaded.
                for (int sl = 0; sl < nsl; ++sl) {
                    const uint32_t cs = c + sl;
                    if (!mbar_wait(&sh->full[cs % kSlots], (cs / kSlots) & 1, limit_ns)) {
                        sh->failed = 1;
                        good = false;
                        break;
                    }
                }
                if (!good) break;
                tc_fence_after();
                // The K step's slot addresses in registers (an indexed array of
                // them would live in local memory).
                const uint32_t s0 = ring_u32 + (uint32_t)(c % kSlots) * kSlotBytes;
                const uint32_t s1 = ring_u32 + (uint32_t)((c + 1) % kSlots) * kSlotBytes;
                const uint32_t s2 = ring_u32 + (uint32_t)((c + 2) % kSlots) * kSlotBytes;
                auto slot = [&](int sl) { return sl == 0 ? s0 : (sl == 1 ? s1 : s2); };
                for (int pr = 0; pr < npairs; ++pr) {
                    const uint32_t a0 = slot(split == 3 ? split_pair_a(pr) : (split == 2 ? f16_pair_a(pr) : 0));
                    const uint32_t bb = slot(split == 3 ? split_pair_b(pr) : (split == 2 ? f16_pair_b(pr) : 0)) + kSlotBytesA;
                    // pair npairs-1 is hi·hi (the only one when not split)
                    const bool big = pr == npairs - 1;
                    const uint32_t d = big ? dacc : dsmall;
#pragma unroll
                    for (int kk = 0; kk < kBK / 16; ++kk) {
                        const uint64_t ad = smem_desc_kmajor_sw64(a0 + kk * 32);
                        const uint64_t bd = smem_desc_kmajor_sw64(bb + kk * 32);
                        const bool acc = big ? (ks > 0 || kk > 0) : (ks > 0 || pr > 0 || kk > 0);
                        umma_bf16(d, ad, bd, idesc, acc ? 1u : 0u);
                    }
                }
                for (int sl = 0; sl < nsl; ++sl) umma_commit(&sh->empty[(c + sl) % kSlots]);
            }
            if (good) umma_commit(&sh->accf[buf]);
        }
        sh->consumed = c;
    } else if (warp >= 4) {
        // Epilogue warpgroup: warp w drains TMEM lanes 32·(w-4) (rows of the
        // block) over all 256 columns.
        const int q = warp - 4;
        const int r = 32 * q + lane;
        for (int j = 0; j < nblk; ++j) {
            const uint32_t gi = base + j;
            const int buf = buf_of(gi);
            if (threadIdx.x == 128) {
                bool have = false;
                if (!sh->failed) {
                    have = mbar_wait(&sh->accf[buf], use_of(gi) & 1, limit_ns);
                    if (!have) sh->failed = 1;
                }
                sh->ep_ok = have ? 1 : 0;
            }
            epilogue_bar();
            if (!sh->ep_ok) break;  // the same value in all four warps
            tc_fence_after();
            int row0, col0;
            tc_block_coords(b0 + j, m, n, lower, &row0, &col0);
            const int gr = row0 + r;
#pragma unroll 1
            for (int ch = 0; ch < kBN / 32; ++ch) {
                const int c0 = 32 * ch;
                uint32_t v[32];
                tmem_ld32(sh->tmem_base + ((uint32_t)(32 * q) << 16) + (uint32_t)(kBN * buf + c0), v);
                if (!dbl) {
                    uint32_t w[32];
                    tmem_ld32(sh->tmem_base + ((uint32_t)(32 * q) << 16) + (uint32_t)(kBN + c0), w);
                    const float ws = split == 2 ? 1.0f / 2048.0f : 1.0f;  // split FP16: lo carries 2^11
#pragma unroll
                    for (int jj = 0; jj < 32; ++jj) v[jj] = __float_as_uint(fmaf(__uint_as_float(w[jj]), ws, __uint_as_float(v[jj])));
                }
                if (gr < m) {
                    // All 32 reads first (independent, in flight together), then
                    // the 32 writes: one memory round trip per chunk, not 32.
                    float cv[32];
                    float* pc = C + gr + (size_t)(col0 + c0) * ldc;
#pragma unroll
                    for (int jj = 0; jj < 32; ++jj) {
                        const int gc = col0 + c0 + jj;
                        cv[jj] = (gc < n && (!lower || gr >= gc)) ? __ldcg(pc + (size_t)jj * ldc) : 0.0f;
                    }
#pragma unroll
                    for (int jj = 0; jj < 32; ++jj) {
                        const int gc = col0 + c0 + jj;
                        if (gc < n && (!lower || gr >= gc)) pc[(size_t)jj * ldc] = fmaf(f, __uint_as_float(v[jj]), cv[jj]);
                    }
                }
            }
            tc_fence_before();
            epilogue_bar();  // all four warps have read the accumulator
            if (threadIdx.x == 128) mbar_arrive(&sh->afree[buf]);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) sh->nacc = base + nblk;
    __syncthreads();
    return !sh->failed;
}

__device__ inline bool tc_gemm_blocks(TcShared* sh, uint8_t* ring, const CUtensorMap* map, int slotA, int slotB, int b0, int nblk, int k,
                                      float f, float* C, int ldc, int m, int n, bool lower, long long limit_ns, int split = 1,
                                      int stride = 0) {
    if (split == 3) return tc_gemm_blocks_t<3>(sh, ring, map, slotA, slotB, b0, nblk, k, f, C, ldc, m, n, lower, limit_ns, stride);
    if (split == 2) return tc_gemm_blocks_t<2>(sh, ring, map, slotA, slotB, b0, nblk, k, f, C, ldc, m, n, lower, limit_ns, stride);
    return tc_gemm_blocks_t<1>(sh, ring, map, slotA, slotB, b0, nblk, k, f, C, ldc, m, n, lower, limit_ns, stride);
}

}  // namespace tc
}  // namespace ttg
