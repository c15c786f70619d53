// ttg_solve.cu — triangular solves with a Cholesky plan's factor, the FP64
// residual and GMRES-based iterative refinement (include/ttg_apps.h,
// ttg_chol_plan_solve / ttg_chol_posv).
//
// FP64 plan: X = L⁻ᵀ L⁻¹ B with the FP64 factor (two block sweeps with the
//   inverted diagonal tiles), then one FP64 residual for the backward error.
// Mixed plan (low-precision factor L̃, FP32): GMRES-IR —
//   x0 = M⁻¹ b with M = L̃L̃ᵀ (FP32 sweeps);
//   repeat: r = b − A x — in FP64 (dense FP64 copy of A), or, for a residual
//           that only steers an early FP32 cycle, in double-float from the
//           FP32 high and low copies;
//           stop when the FP64 ‖r‖∞ / (‖A‖∞ ‖x‖∞) ≤ tol for every column;
//           solve A d = r by GMRES left-preconditioned with M (the Krylov
//           basis, the matrix-vector products and M⁻¹ in FP32, or in FP64
//           when FP32 stops making progress; orthogonalisation sums in FP64);
//           x += d in FP64.
// All RHS columns run in lockstep; each column has its own Krylov space and
// Hessenberg matrix (solved on the host; they are tiny).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/ttg.h"
#include "../../include/ttg_apps.h"
#include "solve_kernels.cuh"
#include "sweep_tma.cuh"
#include "ttg_internal.h"
#include "ttg_sliced_api.h"
#include "ttg_solve_api.h"

using namespace ttg;
using namespace ttg::solve;

namespace {

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    ttg_status ensure(size_t count) {
        if (count <= n) return TTG_OK;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc((void**)&p, sizeof(T) * std::max<size_t>(1, count));
        if (e != cudaSuccess) {
            ttg_set_last_cuda_error(e, "cudaMalloc (solve)", __FILE__, __LINE__);
            return TTG_ENOMEM;
        }
        cudaMemset(p, 0, sizeof(T) * std::max<size_t>(1, count));  // no stale NaN patterns
        n = count;
        return TTG_OK;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

}  // namespace

struct ttg_solver {
    ttg_ctx* ctx = nullptr;
    int N = 0, nb = 0;
    bool mixed = false;
    int64_t elems = 0;
    TileLayout lay{};
    DevBuf<int64_t> d_off;
    DevBuf<int> d_bs, d_displ, d_rowblk;
    // Dense copies of the input (rebuilt when the input changes).
    DevBuf<double> A64;
    DevBuf<float> A32;
    DevBuf<float> A32lo;  // fl32(A - A32): the double-float matvec of FP64 Krylov work
    bool dense_valid = false;
    bool lo_valid = false;
    // Digits of A for the FP64-accurate tensor-core products (built from A64
    // when first needed after an input change).
    ttg_sliced* sl = nullptr;
    bool sl_valid = false;
    bool use_sliced = false;  // this solve's products with A are sliced
    double anorm_inf = 0.0;
    // Operands of the sweeps for the current factor: L_ii⁻ᵀ and L_ii⁻¹
    // (compact diagonal tiles at doff) and the transposed off-diagonal tiles
    // (L_ijᵀ at off[i + j·nb], ld bs[j]).
    DevBuf<double> inv64, linv64, lt64;
    DevBuf<float> inv32, linv32, lt32;
    // Folded sweeps (FP32 factor): W_i = L_ii⁻¹·L_i,i-1 (forward) and
    // L_ii⁻ᵀ·L_i+1,iᵀ (backward), compact at woff_f / woff_b (ld bs[i]).
    DevBuf<float> wf32, wb32;
    DevBuf<int64_t> d_woff_f, d_woff_b;
    DevBuf<WdDesc> d_wdesc_f, d_wdesc_b;
    int64_t wsize_f = 0, wsize_b = 0;
    int n_wdesc_f = 0, n_wdesc_b = 0;
    int64_t dsize = 0;  // elements of the compact diagonal
    DevBuf<int64_t> d_doff;
    DevBuf<int> d_strip_pre, d_step_fwd, d_step_bwd;
    DevBuf<int> d_queues;  // the TMA sweep's claim order: forward items, then backward
    DevBuf<int> d_sweep_ctr;  // per sweep direction: claim, ready[nb], applied[strips]
    DevBuf<int> d_err;        // sweep timeout flag (zeroed per solve)
    int n_strips = 0;
    int items_fwd = 0, items_bwd = 0;  // work items of one sweep per direction
    DevBuf<long long> d_trace;         // sweep timeline (TTG_SWEEP_TRACE)
    DevBuf<TransposeDesc> d_tdesc_off, d_tdesc_diag;
    DevBuf<int64_t> d_tsub_off, d_tsub_diag;
    int n_tdesc_off = 0, n_tdesc_diag = 0;
    // Work vectors (N × 16).
    DevBuf<double> B, X, R, D, W, T1, T2, P, Q;  // Q: row sums of |A| by 64-column block
    DevBuf<float> f1, f2, f3;
    DevBuf<float> Pf;  // partials of the FP32 matvec (splits × N × nrhs)
    DevBuf<double> Vd;  // Krylov basis, FP64 variant
    DevBuf<float> Vf;   // Krylov basis, FP32 variant
    DevBuf<double> part, colv, coefA, coefB;
    int sweep_grid64 = 0, sweep_grid32 = 0, sweep_grid_mix = 0;
    // FP32 sweeps with TMA-staged strips (uniform tiles, edge a multiple of
    // 128 and at most 512): the operand maps of both directions, rebuilt
    // when an operand pointer changes.
    int tma_b = 0;  // 0: this layout takes the generic sweep kernel
    SweepMaps tma_maps[2];
    const void* tma_keys[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
};

// 2D FP32 tensor map of an array of b-row column-major tiles: (row, column)
// with the b rows inner; box 64 rows × kTmaCols columns.
static ttg_status encode_strip_map(CUtensorMap* map, const float* base, int64_t elems, int b) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || !fn || q != cudaDriverEntryPointSuccess) {
        ttg_set_last_cuda_error(e, "cudaGetDriverEntryPointByVersion(cuTensorMapEncodeTiled)", __FILE__, __LINE__);
        return TTG_ECUDA;
    }
    auto enc = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    cuuint64_t dims[2] = {(cuuint64_t)b, (cuuint64_t)std::max<int64_t>(1, elems / b)};
    cuuint64_t strides[1] = {(cuuint64_t)b * 4};
    cuuint32_t box[2] = {(cuuint32_t)kStrip, (cuuint32_t)kTmaCols};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        ttg_set_last_cuda_error(cudaErrorInvalidValue, "cuTensorMapEncodeTiled (sweep strips)", __FILE__, __LINE__);
        return TTG_EINVAL;
    }
    return TTG_OK;
}

template <class T, class TM>
static ttg_status sweep_grid(ttg_solver* S, int* grid) {
    const int smem = sweep_smem_bytes<T, TM>();
    TTG_CUDA_CHECK(cudaFuncSetAttribute(sweep_kernel<T, TM>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    int per = 0;
    TTG_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, sweep_kernel<T, TM>, 256, smem));
    *grid = std::max(1, per) * S->ctx->sms;
    return TTG_OK;
}

static ttg_status solver_init(ttg_solver* S) {
    TTG_CUDA_CHECK(cudaSetDevice(S->ctx->device));
    ttg_status st;
    if ((st = sweep_grid<double, double>(S, &S->sweep_grid64)) != TTG_OK) return st;
    if ((st = sweep_grid<float, float>(S, &S->sweep_grid32)) != TTG_OK) return st;
    if ((st = sweep_grid<double, float>(S, &S->sweep_grid_mix)) != TTG_OK) return st;
    TTG_CUDA_CHECK(cudaFuncSetAttribute(sweep_kernel_f32_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, kTmaSmem));
    const int smem = kF64SmemDoubles * (int)sizeof(double);
    TTG_CUDA_CHECK(cudaFuncSetAttribute(invert_diag_tiles<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    TTG_CUDA_CHECK(cudaFuncSetAttribute(invert_diag_tiles<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    return TTG_OK;
}

// Host tables of the sweeps (strips, item counts per step) and of the tile
// transposes.
// The TMA sweep's claim order (folded form), forward items then backward,
// each an item index in step order.  sp: strips before each block row;
// fwd / bwd: items before each step of the two directions.  Step s holds
// D(s), the diagonal strips of its row; Z(s), the Z strips of the next row;
// and its bulk B(s), the updates of the rows after that, nearest row first.
// The order D(0) Z(0), then for s >= 1: B(s-1)'s first row, D(s), Z(s), the
// rest of B(s-1), claims each step's chain items before the bulk of the step
// before it (step order claims them after it: at N = 32768 the next diagonal
// waited ~37 µs behind ~500 bulk items).  Every item still follows all the
// items it reads — D(s): D(s-1), Z(s-1); Z(s): the updates of its row, the
// last in B(s-1)'s first row; B(s-1): D(s-1) and the same strips in B(s-2) —
// so blocks claiming in this order never wait on an unclaimed item.
static void sweep_claim_order(int nb, const std::vector<int>& sp, const std::vector<int>& fwd, const std::vector<int>& bwd,
                              std::vector<int>& order) {
    order.clear();
    order.reserve((size_t)fwd[nb] + bwd[nb]);
    for (int dir = 0; dir < 2; ++dir) {
        const std::vector<int>& steps = dir ? bwd : fwd;
        auto row = [&](int st) { return dir ? nb - 1 - st : st; };
        auto strips = [&](int r) { return sp[r + 1] - sp[r]; };
        auto chain_z = [&](int st) { return st + 1 < nb ? strips(row(st + 1)) : 0; };
        auto first_row = [&](int st) { return st + 2 < nb ? strips(row(st + 2)) : 0; };
        auto push = [&](int a, int n) {
            for (int k = 0; k < n; ++k) order.push_back(a + k);
        };
        auto bulk0 = [&](int st) { return steps[st] + strips(row(st)) + chain_z(st); };
        push(steps[0], strips(row(0)) + chain_z(0));
        for (int st = 1; st <= nb; ++st) {
            const int p = st - 1;  // B(p): first row, [D(st) Z(st)], the rest
            push(bulk0(p), first_row(p));
            if (st < nb) push(steps[st], strips(row(st)) + chain_z(st));
            push(bulk0(p) + first_row(p), steps[p + 1] - bulk0(p) - first_row(p));
        }
    }
}

// Strips before each block row and items before each sweep step (forward,
// backward) for block rows of bs[i] rows; false if a count overflows.
static bool sweep_step_tables(int nb, const int* bs, std::vector<int>& sp, std::vector<int>& fwd, std::vector<int>& bwd) {
    sp.assign(nb + 1, 0);
    for (int i = 0; i < nb; ++i) sp[i + 1] = sp[i] + (bs[i] + kStrip - 1) / kStrip;
    fwd.assign(nb + 1, 0);
    bwd.assign(nb + 1, 0);
    for (int st = 0; st < nb; ++st) {
        const int i = st, ib = nb - 1 - st;
        const int64_t nf = (int64_t)(sp[i + 1] - sp[i]) + (sp[nb] - sp[i + 1]);
        const int64_t nbk = (int64_t)(sp[ib + 1] - sp[ib]) + sp[ib];
        if ((int64_t)fwd[st] + nf > INT32_MAX || (int64_t)bwd[st] + nbk > INT32_MAX) return false;
        fwd[st + 1] = fwd[st] + (int)nf;
        bwd[st + 1] = bwd[st] + (int)nbk;
    }
    return true;
}

static ttg_status solver_tables(ttg_solver* S, const int* bs, const int64_t* off) {
    const int nb = S->nb;
    std::vector<int64_t> doff(nb, 0);
    int64_t d = 0;
    for (int i = 0; i < nb; ++i) {
        doff[i] = d;
        d += (int64_t)bs[i] * bs[i];
    }
    S->dsize = d;
    std::vector<int> sp, fwd, bwd;
    if (!sweep_step_tables(nb, bs, sp, fwd, bwd)) return TTG_EINVAL;
    S->n_strips = sp[nb];
    std::vector<TransposeDesc> to, td;
    std::vector<int64_t> so(1, 0), sd(1, 0);
    for (int j = 0; j < nb; ++j) {
        for (int i = j + 1; i < nb; ++i) {
            const int64_t o = off[i + (size_t)j * nb];
            to.push_back({o, o, bs[i], bs[j]});
            so.push_back(so.back() + (int64_t)((bs[i] + kTrEdge - 1) / kTrEdge) * ((bs[j] + kTrEdge - 1) / kTrEdge));
        }
        td.push_back({doff[j], doff[j], bs[j], bs[j]});
        sd.push_back(sd.back() + (int64_t)((bs[j] + kTrEdge - 1) / kTrEdge) * ((bs[j] + kTrEdge - 1) / kTrEdge));
    }
    S->items_fwd = fwd[nb];
    S->items_bwd = bwd[nb];
    std::vector<int> order;
    sweep_claim_order(nb, sp, fwd, bwd, order);
    if (order.size() != (size_t)S->items_fwd + S->items_bwd) return TTG_EINVAL;
    {
        bool uni = bs[0] % 128 == 0 && bs[0] <= kTmaMaxK;
        for (int i = 1; i < nb; ++i) uni = uni && bs[i] == bs[0];
        S->tma_b = uni ? bs[0] : 0;
    }
    // W products of the folded sweeps: forward W_i (i >= 1) = linv_i · L(i, i-1);
    // backward W_i (i <= nb-2) = inv_i · L(i+1, i)ᵀ (the transposed tile at
    // off[(i+1) + i·nb], ld bs[i]).
    std::vector<int64_t> woff_f(nb, 0), woff_b(nb, 0);
    std::vector<WdDesc> wdf, wdb;
    int64_t wf = 0, wb = 0;
    for (int i = 0; i < nb; ++i) {
        if (i >= 1 && bs[i] > 0 && bs[i - 1] > 0) {
            woff_f[i] = wf;
            wdf.push_back({doff[i], off[i + (size_t)(i - 1) * nb], wf, bs[i], bs[i - 1], bs[i]});
            wf += (int64_t)bs[i] * bs[i - 1];
        }
        if (i + 1 < nb && bs[i] > 0 && bs[i + 1] > 0) {
            woff_b[i] = wb;
            wdb.push_back({doff[i], off[(i + 1) + (size_t)i * nb], wb, bs[i], bs[i + 1], bs[i]});
            wb += (int64_t)bs[i] * bs[i + 1];
        }
    }
    S->wsize_f = wf;
    S->wsize_b = wb;
    S->n_wdesc_f = (int)wdf.size();
    S->n_wdesc_b = (int)wdb.size();
    S->n_tdesc_off = (int)to.size();
    S->n_tdesc_diag = (int)td.size();
    ttg_status st;
    if ((st = S->d_doff.ensure(nb)) != TTG_OK || (st = S->d_strip_pre.ensure(nb + 1)) != TTG_OK ||
        (st = S->d_step_fwd.ensure(nb + 1)) != TTG_OK || (st = S->d_step_bwd.ensure(nb + 1)) != TTG_OK ||
        (st = S->d_queues.ensure(order.size())) != TTG_OK ||
        (st = S->d_sweep_ctr.ensure(2 * (size_t)(2 + 2 * nb + S->n_strips))) != TTG_OK || (st = S->d_err.ensure(1)) != TTG_OK ||
        (st = S->d_woff_f.ensure(nb)) != TTG_OK || (st = S->d_woff_b.ensure(nb)) != TTG_OK ||
        (st = S->d_wdesc_f.ensure(std::max<size_t>(1, wdf.size()))) != TTG_OK ||
        (st = S->d_wdesc_b.ensure(std::max<size_t>(1, wdb.size()))) != TTG_OK ||
        (st = S->d_tdesc_off.ensure(std::max<size_t>(1, to.size()))) != TTG_OK ||
        (st = S->d_tdesc_diag.ensure(td.size())) != TTG_OK || (st = S->d_tsub_off.ensure(so.size())) != TTG_OK ||
        (st = S->d_tsub_diag.ensure(sd.size())) != TTG_OK)
        return st;
    TTG_CUDA_CHECK(cudaMemcpy(S->d_doff.p, doff.data(), sizeof(int64_t) * nb, cudaMemcpyHostToDevice));
    TTG_CUDA_CHECK(cudaMemcpy(S->d_strip_pre.p, sp.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice));
    TTG_CUDA_CHECK(cudaMemcpy(S->d_step_fwd.p, fwd.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice));
    TTG_CUDA_CHECK(cudaMemcpy(S->d_step_bwd.p, bwd.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice));
    TTG_CUDA_CHECK(cudaMemcpy(S->d_queues.p, order.data(), sizeof(int) * order.size(), cudaMemcpyHostToDevice));
    TTG_CUDA_CHECK(cudaMemcpy(S->d_woff_f.p, woff_f.data(), sizeof(int64_t) * nb, cudaMemcpyHostToDevice));
    TTG_CUDA_CHECK(cudaMemcpy(S->d_woff_b.p, woff_b.data(), sizeof(int64_t) * nb, cudaMemcpyHostToDevice));
    if (!wdf.empty()) TTG_CUDA_CHECK(cudaMemcpy(S->d_wdesc_f.p, wdf.data(), sizeof(WdDesc) * wdf.size(), cudaMemcpyHostToDevice));
    if (!wdb.empty()) TTG_CUDA_CHECK(cudaMemcpy(S->d_wdesc_b.p, wdb.data(), sizeof(WdDesc) * wdb.size(), cudaMemcpyHostToDevice));
    if (!to.empty())
        TTG_CUDA_CHECK(cudaMemcpy(S->d_tdesc_off.p, to.data(), sizeof(TransposeDesc) * to.size(), cudaMemcpyHostToDevice));
    TTG_CUDA_CHECK(cudaMemcpy(S->d_tdesc_diag.p, td.data(), sizeof(TransposeDesc) * td.size(), cudaMemcpyHostToDevice));
    TTG_CUDA_CHECK(cudaMemcpy(S->d_tsub_off.p, so.data(), sizeof(int64_t) * so.size(), cudaMemcpyHostToDevice));
    TTG_CUDA_CHECK(cudaMemcpy(S->d_tsub_diag.p, sd.data(), sizeof(int64_t) * sd.size(), cudaMemcpyHostToDevice));
    return TTG_OK;
}

ttg_status ttg_solver_create(ttg_ctx* ctx, int N, int nb, const int* bs, const int64_t* off, bool mixed, ttg_solver** out) {
    *out = nullptr;
    ttg_solver* S = new ttg_solver();
    S->ctx = ctx;
    S->N = N;
    S->nb = nb;
    S->mixed = mixed;
    std::vector<int> displ(nb + 1, 0);
    for (int i = 0; i < nb; ++i) displ[i + 1] = displ[i] + bs[i];
    S->elems = 0;
    for (int j = 0; j < nb; ++j)
        for (int i = j; i < nb; ++i) S->elems += (int64_t)bs[i] * bs[j];
    ttg_status st;
    if ((st = S->d_off.ensure((size_t)nb * nb)) != TTG_OK || (st = S->d_bs.ensure(nb)) != TTG_OK ||
        (st = S->d_displ.ensure(nb + 1)) != TTG_OK) {
        ttg_solver_destroy(S);
        return st;
    }
    cudaMemcpy(S->d_off.p, off, sizeof(int64_t) * nb * nb, cudaMemcpyHostToDevice);
    cudaMemcpy(S->d_bs.p, bs, sizeof(int) * nb, cudaMemcpyHostToDevice);
    cudaMemcpy(S->d_displ.p, displ.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice);
    {
        std::vector<int> rowblk(N);
        for (int i = 0; i < nb; ++i)
            for (int r = displ[i]; r < displ[i + 1]; ++r) rowblk[r] = i;
        if ((st = S->d_rowblk.ensure(std::max(1, N))) != TTG_OK) {
            ttg_solver_destroy(S);
            return st;
        }
        cudaMemcpy(S->d_rowblk.p, rowblk.data(), sizeof(int) * N, cudaMemcpyHostToDevice);
    }
    S->lay.off = S->d_off.p;
    S->lay.bs = S->d_bs.p;
    S->lay.displ = S->d_displ.p;
    S->lay.nb = nb;
    S->lay.N = N;
    if ((st = solver_init(S)) != TTG_OK || (st = solver_tables(S, bs, off)) != TTG_OK) {
        ttg_solver_destroy(S);
        return st;
    }
    *out = S;
    return TTG_OK;
}

void ttg_solver_destroy(ttg_solver* S) {
    if (!S) return;
    cudaSetDevice(S->ctx->device);
    for (auto* b : {&S->A64, &S->inv64, &S->linv64, &S->lt64, &S->B, &S->X, &S->R, &S->D, &S->W, &S->T1, &S->T2, &S->P, &S->Q, &S->Vd, &S->part, &S->colv,
                    &S->coefA, &S->coefB})
        b->release();
    for (auto* b : {&S->A32, &S->A32lo, &S->Pf, &S->wf32, &S->wb32, &S->inv32, &S->linv32, &S->lt32, &S->f1, &S->f2, &S->f3, &S->Vf}) b->release();
    S->d_off.release();
    S->d_bs.release();
    S->d_displ.release();
    S->d_rowblk.release();
    S->d_doff.release();
    S->d_strip_pre.release();
    S->d_step_fwd.release();
    S->d_step_bwd.release();
    S->d_queues.release();
    S->d_sweep_ctr.release();
    S->d_err.release();
    S->d_tdesc_off.release();
    S->d_tdesc_diag.release();
    S->d_tsub_off.release();
    S->d_tsub_diag.release();
    if (S->sl) ttg_sliced_destroy(S->sl);
    delete S;
}

extern "C" ttg_status ttg_split_f64_f32(const double* v, int64_t n, float* hi, float* lo) {
    if (n < 0 || (n > 0 && (!v || !hi || !lo))) return TTG_EINVAL;
    for (int64_t i = 0; i < n; ++i) split_f64_f32(v[i], hi[i], lo[i]);
    return TTG_OK;
}

void ttg_solver_input_changed(ttg_solver* S) {
    if (S) S->dense_valid = S->lo_valid = S->sl_valid = false;
}

// Digits of the dense copy for the sliced products (after ensure_dense).
static ttg_status ensure_sliced(ttg_solver* S, cudaStream_t s) {
    if (S->sl_valid) return TTG_OK;
    ttg_status st;
    if (!S->sl && (st = ttg_sliced_create(S->ctx, S->N, &S->sl)) != TTG_OK) return st;
    if ((st = ttg_sliced_set_matrix(S->sl, S->A64.p, s)) != TTG_OK) return st;
    S->sl_valid = true;
    return TTG_OK;
}

// Dense copies of A (FP64, and FP32 for the mixed path) and ‖A‖∞.
static ttg_status ensure_dense(ttg_solver* S, const double* pristine, cudaStream_t s) {
    if (S->dense_valid) return TTG_OK;
    const size_t NN = (size_t)S->N * S->N;
    ttg_status st = S->A64.ensure(NN);
    if (st != TTG_OK) return st;
    if (S->mixed && ((st = S->A32.ensure(NN)) != TTG_OK || (st = S->A32lo.ensure(NN)) != TTG_OK)) return st;
    // ‖A‖∞ from the row sums by 64-column block (written by the dense build).
    const int nsb = (S->N + kDenseSb - 1) / kDenseSb;
    if ((st = S->T1.ensure(S->N)) != TTG_OK || (st = S->Q.ensure((size_t)nsb * S->N)) != TTG_OK) return st;
    ttg_note_launch();
    dense_sym_from_tiles<<<S->ctx->sms * 8, 256, 0, s>>>(S->lay, S->d_rowblk.p, pristine, S->A64.p, S->mixed ? S->A32.p : nullptr,
                                                        S->mixed ? S->A32lo.p : nullptr, S->Q.p);
    S->lo_valid = S->mixed;
    ttg_note_launch();
    row_abs_final<<<(S->N + 255) / 256, 256, 0, s>>>(S->N, nsb, S->Q.p, S->T1.p);
    TTG_CUDA_CHECK(cudaGetLastError());
    std::vector<double> rs(S->N);
    TTG_CUDA_CHECK(cudaMemcpyAsync(rs.data(), S->T1.p, sizeof(double) * S->N, cudaMemcpyDeviceToHost, s));
    TTG_CUDA_CHECK(cudaStreamSynchronize(s));
    S->anorm_inf = 0.0;
    for (double v : rs) S->anorm_inf = std::max(S->anorm_inf, v);
    S->dense_valid = true;
    return TTG_OK;
}

// Sweep operands of a new factor: L_ii⁻ᵀ (TRSM of the identity), L_ii⁻¹ (its
// transpose) and the transposed off-diagonal tiles.
template <class TM>
static ttg_status prepare_operands(ttg_solver* S, const TM* L, DevBuf<TM>& inv, DevBuf<TM>& linv, DevBuf<TM>& lt,
                                   cudaStream_t s) {
    const int parts = 8;
    const int smem = kF64SmemDoubles * (int)sizeof(double);
    ttg_status st;
    if ((st = inv.ensure(S->dsize)) != TTG_OK || (st = linv.ensure(S->dsize)) != TTG_OK || (st = lt.ensure(S->elems)) != TTG_OK)
        return st;
    ttg_note_launch();
    invert_diag_tiles<TM><<<dim3(S->nb, parts), kThreads, smem, s>>>(S->lay, S->d_doff.p, L, inv.p, parts);
    ttg_note_launch();
    transpose_tiles<TM><<<S->ctx->sms * 8, 256, 0, s>>>(S->d_tdesc_diag.p, S->d_tsub_diag.p, S->n_tdesc_diag, inv.p, linv.p);
    if (S->n_tdesc_off > 0) {
        ttg_note_launch();
        transpose_tiles<TM><<<S->ctx->sms * 8, 256, 0, s>>>(S->d_tdesc_off.p, S->d_tsub_off.p, S->n_tdesc_off, L, lt.p);
    }
    if constexpr (sizeof(TM) == 4) {
        // Folded sweeps: the W products (FP32, 16 parts of 128×128 blocks each).
        if ((st = S->wf32.ensure(std::max<int64_t>(1, S->wsize_f))) != TTG_OK ||
            (st = S->wb32.ensure(std::max<int64_t>(1, S->wsize_b))) != TTG_OK)
            return st;
        if (S->n_wdesc_f > 0) {
            ttg_note_launch();
            wd_gemm_kernel<float><<<dim3(S->n_wdesc_f, 16), kThreads, smem, s>>>(S->d_wdesc_f.p, linv.p, L, S->wf32.p);
        }
        if (S->n_wdesc_b > 0) {
            ttg_note_launch();
            wd_gemm_kernel<float><<<dim3(S->n_wdesc_b, 16), kThreads, smem, s>>>(S->d_wdesc_b.p, inv.p, lt.p, S->wb32.p);
        }
    }
    TTG_CUDA_CHECK(cudaGetLastError());
    return TTG_OK;
}

ttg_status ttg_solver_factor_done(ttg_solver* S, const double* L64, const float* L32, cudaStream_t s) {
    if (S->mixed) return prepare_operands<float>(S, L32, S->inv32, S->linv32, S->lt32, s);
    return prepare_operands<double>(S, L64, S->inv64, S->linv64, S->lt64, s);
}

namespace {

// TTG_SWEEP_TRACE=<file> appends the timeline of every sweep to <file>: one
// line per work item (direction, item, claimed, inputs ready, done in ns of
// the GPU global timer, SM).  A diagnostic: it synchronises after each pair.
const char* sweep_trace_path() {
    static const char* p = getenv("TTG_SWEEP_TRACE");
    return p && *p ? p : nullptr;
}

// R (scratch, overwritten) -> Y = L⁻¹ R -> X = L⁻ᵀ Y (Y overwritten): the
// forward and the backward sweep, one launch each.
template <class T, class TM>
ttg_status sweeps(ttg_solver* S, const TM* L, const TM* LT, const TM* Linv, const TM* invT, T* R, T* Y, T* X, int nrhs, int grid,
                  cudaStream_t s) {
    const size_t region = 2 + 2 * S->nb + S->n_strips;
    TTG_CUDA_CHECK(cudaMemsetAsync(S->d_sweep_ctr.p, 0, sizeof(int) * 2 * region, s));
    SweepArgs a;
    a.off = S->d_off.p;
    a.doff = S->d_doff.p;
    a.bs = S->d_bs.p;
    a.displ = S->d_displ.p;
    a.strip_pre = S->d_strip_pre.p;
    a.nb = S->nb;
    a.N = S->N;
    a.nrhs = nrhs;
    a.err = S->d_err.p;
    a.timeout_ns = (long long)(std::max(1.0, S->ctx->timeout_s) * 1e9);
    a.trace = nullptr;
    // FP32 vectors with an FP32 factor sweep in the folded form.  The fold
    // moves the cancellation of Vin_i against the previous row's update after
    // the multiplication by L_ii⁻¹, which amplifies rounding by κ(L_ii): the
    // double-float sweeps of the FP64 Krylov variant (used for ill-conditioned
    // matrices) stay unfolded (α = 1e-8, N = 32768: 57 iterations unfolded,
    // 150 folded).
    constexpr bool fold = sizeof(TM) == 4 && sizeof(T) == 4;
    a.fold = fold ? 1 : 0;
    const size_t n_trace = 4 * ((size_t)S->items_fwd + S->items_bwd);
    if (sweep_trace_path()) {
        ttg_status st = S->d_trace.ensure(n_trace);
        if (st != TTG_OK) return st;
    }
    const int smem = sweep_smem_bytes<T, TM>();
    constexpr bool f32 = sizeof(T) == 4 && sizeof(TM) == 4;
    const bool tma = f32 && S->tma_b > 0;
    if constexpr (f32) {
        if (tma) {
            // Operand maps of the two directions (forward: L, L_ii⁻¹, W_f;
            // backward: Lᵀ tiles, L_ii⁻ᵀ, W_b), rebuilt when a pointer changes.
            const void* keys[2][3] = {{L, Linv, S->wf32.p}, {LT, invT, S->wb32.p}};
            const int64_t n3[3] = {S->elems, S->dsize, 0};
            for (int dir = 0; dir < 2; ++dir) {
                if (std::equal(keys[dir], keys[dir] + 3, S->tma_keys[dir])) continue;
                SweepMaps& m = S->tma_maps[dir];
                m.b = S->tma_b;
                ttg_status st;
                if ((st = encode_strip_map(&m.mu, (const float*)keys[dir][0], n3[0], m.b)) != TTG_OK ||
                    (st = encode_strip_map(&m.md, (const float*)keys[dir][1], n3[1], m.b)) != TTG_OK ||
                    (st = encode_strip_map(&m.wd, (const float*)keys[dir][2], std::max<int64_t>(dir ? S->wsize_b : S->wsize_f, m.b),
                                           m.b)) != TTG_OK)
                    return st;
                std::copy(keys[dir], keys[dir] + 3, S->tma_keys[dir]);
            }
        }
    }
    for (int dir = 0; dir < 2; ++dir) {
        int* ctr = S->d_sweep_ctr.p + dir * region;
        a.claim = ctr;
        a.ready = ctr + 2;
        a.applied = ctr + 2 + S->nb;
        a.zready = ctr + 2 + S->nb + S->n_strips;
        a.woff = dir ? S->d_woff_b.p : S->d_woff_f.p;
        a.backward = dir;
        a.step_start = dir ? S->d_step_bwd.p : S->d_step_fwd.p;
        a.order = S->d_queues.p + (dir ? S->items_fwd : 0);
        if (sweep_trace_path()) a.trace = S->d_trace.p + (dir ? 4 * (size_t)S->items_fwd : 0);
        const TM* W = nullptr;
        if constexpr (fold) W = dir ? S->wb32.p : S->wf32.p;
        if constexpr (f32) {
            if (tma) {
                ttg_note_launch();
                if (dir == 0) sweep_kernel_f32_tma<<<S->ctx->sms, 256, kTmaSmem, s>>>(a, S->tma_maps[0], (float*)R, (float*)Y);
                else sweep_kernel_f32_tma<<<S->ctx->sms, 256, kTmaSmem, s>>>(a, S->tma_maps[1], (float*)Y, (float*)X);
                TTG_CUDA_CHECK(cudaGetLastError());
                continue;
            }
        }
        if (dir == 0) {
            ttg_note_launch();
            sweep_kernel<T, TM><<<grid, 256, smem, s>>>(a, L, Linv, W, R, Y);
        }
        else {
            ttg_note_launch();
            sweep_kernel<T, TM><<<grid, 256, smem, s>>>(a, LT, invT, W, Y, X);
        }
        TTG_CUDA_CHECK(cudaGetLastError());
    }
    if (const char* path = sweep_trace_path()) {
        std::vector<long long> h(n_trace);
        TTG_CUDA_CHECK(cudaMemcpyAsync(h.data(), S->d_trace.p, sizeof(long long) * n_trace, cudaMemcpyDeviceToHost, s));
        TTG_CUDA_CHECK(cudaStreamSynchronize(s));
        if (FILE* f = fopen(path, "a")) {
            for (int dir = 0; dir < 2; ++dir) {
                const size_t base = dir ? 4 * (size_t)S->items_fwd : 0;
                const int n = dir ? S->items_bwd : S->items_fwd;
                for (int it = 0; it < n; ++it) {
                    const long long* r = h.data() + base + 4 * (size_t)it;
                    fprintf(f, "%d,%d,%lld,%lld,%lld,%lld\n", dir, it, r[0], r[1], r[2], r[3]);
                }
            }
            fclose(f);
        }
    }
    return TTG_OK;
}

// Y = A X (mode 0) or Y = B − A X (mode 2) with the dense copy.  FP32: the
// register-blocked kernel, K split so that the grid fills two blocks per SM.
template <class T>
ttg_status matmul(ttg_solver* S, const T* A, const T* X, const T* B, T* Y, T* P, int nrhs, int mode, cudaStream_t s) {
    if constexpr (sizeof(T) == 4) {
        const int rowblocks = (S->N + kMmRows - 1) / kMmRows;
        const int splits = std::max(1, std::min(2 * S->ctx->sms / rowblocks, S->N / kMmChunk));
        ttg_status st = S->Pf.ensure((size_t)splits * S->N * nrhs);
        if (st != TTG_OK) return st;
        dim3 grid(rowblocks, splits);
        ttg_note_launch();
        dense_matmul_f32_partial<<<grid, 256, 0, s>>>(S->N, (const float*)A, (const float*)X, nrhs, S->Pf.p, splits);
        ttg_note_launch();
        reduce_partials<float><<<S->ctx->sms * 4, 256, 0, s>>>(S->N, nrhs, S->Pf.p, splits, (const float*)B, (float*)Y, mode);
        TTG_CUDA_CHECK(cudaGetLastError());
        return TTG_OK;
    }
    const int splits = 4;
    dim3 grid((S->N + 127) / 128, splits);
    ttg_note_launch();
    dense_matmul_partial<T><<<grid, 256, 0, s>>>(S->N, A, X, nrhs, P, splits);
    ttg_note_launch();
    reduce_partials<T><<<S->ctx->sms * 4, 256, 0, s>>>(S->N, nrhs, P, splits, B, Y, mode);
    TTG_CUDA_CHECK(cudaGetLastError());
    return TTG_OK;
}

constexpr int kDfMaxSplits = 32;  // K splits of the double-float product (partials in S->P)

// Y = A X (mode 0) or Y = B - A X (mode 2) in double-float arithmetic from
// the two FP32 halves of the dense copy (built on first use): the FP64 Krylov
// variant's operator and the early residuals of the refinement.
ttg_status matmul_df(ttg_solver* S, const double* X, double* Y, int nrhs, cudaStream_t s, const double* B = nullptr,
                     int mode = 0) {
    const size_t NN = (size_t)S->N * S->N;
    ttg_status st;
    if (!S->lo_valid) {
        if ((st = S->A32lo.ensure(NN)) != TTG_OK) return st;
        ttg_note_launch();
        split_low_half<<<S->ctx->sms * 8, 256, 0, s>>>((int64_t)NN, S->A64.p, S->A32lo.p);
        TTG_CUDA_CHECK(cudaGetLastError());
        S->lo_valid = true;
    }
    // K splits so that the grid fills whole waves of the SMs (16 blocks each).
    const int rblocks = (S->N + 255) / 256;
    const int splits = std::max(1, std::min(kDfMaxSplits, (S->ctx->sms * 16 + rblocks - 1) / rblocks));
    dim3 grid(rblocks, splits);
    ttg_note_launch();
    dense_matmul_df_partial<<<grid, 256, 0, s>>>(S->N, S->A32.p, S->A32lo.p, X, nrhs, S->P.p, splits);
    ttg_note_launch();
    reduce_partials<double><<<S->ctx->sms * 4, 256, 0, s>>>(S->N, nrhs, S->P.p, splits, B, Y, mode);
    TTG_CUDA_CHECK(cudaGetLastError());
    return TTG_OK;
}

// Per-column reduction to host: kind 0 dot(X, Y), kind 1 max|X|.
template <class T>
ttg_status colreduce(ttg_solver* S, const T* X, const T* Y, int nrhs, int kind, double* host, cudaStream_t s) {
    const int blocks = 128;
    ttg_note_launch();
    column_reduce_partial<T><<<blocks, 256, 0, s>>>(S->N, nrhs, X, Y, kind, S->part.p);
    ttg_note_launch();
    column_reduce_final<<<1, 32, 0, s>>>(nrhs, blocks, S->part.p, kind, S->colv.p);
    TTG_CUDA_CHECK(cudaGetLastError());
    TTG_CUDA_CHECK(cudaMemcpyAsync(host, S->colv.p, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s));
    TTG_CUDA_CHECK(cudaStreamSynchronize(s));
    return TTG_OK;
}

// Y[:,q] = a[q] X[:,q] + b[q] Y[:,q] (b = nullptr: Y = a X).
template <class TX, class TY>
ttg_status axpby(ttg_solver* S, const std::vector<double>& a, const TX* X, const std::vector<double>* b, TY* Y, int nrhs,
                 cudaStream_t s) {
    TTG_CUDA_CHECK(cudaMemcpyAsync(S->coefA.p, a.data(), sizeof(double) * nrhs, cudaMemcpyHostToDevice, s));
    if (b) TTG_CUDA_CHECK(cudaMemcpyAsync(S->coefB.p, b->data(), sizeof(double) * nrhs, cudaMemcpyHostToDevice, s));
    ttg_note_launch();
    column_axpby<TX, TY><<<S->ctx->sms * 4, 256, 0, s>>>(S->N, nrhs, S->coefA.p, X, b ? S->coefB.p : nullptr, Y);
    TTG_CUDA_CHECK(cudaGetLastError());
    return TTG_OK;
}

// Backward errors ‖R_q‖∞ / (‖A‖∞ ‖X_q‖∞) of the current X (R = B − A X).
ttg_status backward_errors(ttg_solver* S, int nrhs, cudaStream_t s, std::vector<double>& be, std::vector<double>& rnorm,
                           bool df = false) {
    ttg_status st = df              ? matmul_df(S, S->X.p, S->R.p, nrhs, s, S->B.p, 2)
                    : S->use_sliced ? ttg_sliced_matmul_run(S->sl, S->X.p, nrhs, S->B.p, S->R.p, 2, s)
                                    : matmul<double>(S, S->A64.p, S->X.p, S->B.p, S->R.p, S->P.p, nrhs, 2, s);
    if (st != TTG_OK) return st;
    std::vector<double> xn(nrhs);
    rnorm.assign(nrhs, 0.0);
    if ((st = colreduce<double>(S, S->R.p, nullptr, nrhs, 1, rnorm.data(), s)) != TTG_OK) return st;
    if ((st = colreduce<double>(S, S->X.p, nullptr, nrhs, 1, xn.data(), s)) != TTG_OK) return st;
    be.assign(nrhs, 0.0);
    for (int q = 0; q < nrhs; ++q) {
        be[q] = xn[q] > 0 ? rnorm[q] / (S->anorm_inf * xn[q]) : (rnorm[q] > 0 ? INFINITY : 0.0);
        if (!(be[q] == be[q])) be[q] = INFINITY;  // NaN never counts as converged
    }
    return TTG_OK;
}

// One GMRES(m) cycle on A d = r, preconditioned on the left by M = L̃L̃ᵀ,
// in precision TG (float or double).  r is in S->R (FP64), d goes to S->D.
// Returns the number of iterations.
template <class TG>
ttg_status gmres_cycle(ttg_solver* S, const float* L32, int nrhs, int m, double inner_tol, cudaStream_t s, int* iters) {
    const int N = S->N;
    const size_t blk = (size_t)N * nrhs;
    TG* V;
    TG *t1, *t2, *t3;
    ttg_status st;
    if (sizeof(TG) == 4) {
        if ((st = S->Vf.ensure(blk * (m + 1))) != TTG_OK) return st;
        V = (TG*)S->Vf.p;
        t1 = (TG*)S->f1.p;
        t2 = (TG*)S->f2.p;
        t3 = (TG*)S->f3.p;
    } else {
        if ((st = S->Vd.ensure(blk * (m + 1))) != TTG_OK) return st;
        V = (TG*)S->Vd.p;
        t1 = (TG*)S->T1.p;
        t2 = (TG*)S->T2.p;
        t3 = nullptr;  // matmul_df keeps its partials in S->P
    }
    const TG* A = sizeof(TG) == 4 ? (const TG*)S->A32.p : (const TG*)S->A64.p;
    const int grid = sizeof(TG) == 4 ? S->sweep_grid32 : S->sweep_grid_mix;
    // Scale r per column by 1/‖r‖∞ (keeps FP32 in range), z0 = M⁻¹ r̂.
    std::vector<double> rn(nrhs), inv(nrhs), one(nrhs, 1.0);
    if ((st = colreduce<double>(S, S->R.p, nullptr, nrhs, 1, rn.data(), s)) != TTG_OK) return st;
    for (int q = 0; q < nrhs; ++q) inv[q] = rn[q] > 0 ? 1.0 / rn[q] : 0.0;
    if ((st = axpby<double, TG>(S, inv, S->R.p, nullptr, t1, nrhs, s)) != TTG_OK) return st;
    if ((st = sweeps<TG, float>(S, L32, S->lt32.p, S->linv32.p, S->inv32.p, t1, t2, V, nrhs, grid, s)) != TTG_OK) return st;
    std::vector<double> beta(nrhs);
    if ((st = colreduce<TG>(S, V, V, nrhs, 0, beta.data(), s)) != TTG_OK) return st;
    std::vector<double> scale(nrhs);
    for (int q = 0; q < nrhs; ++q) {
        beta[q] = std::sqrt(beta[q]);
        scale[q] = beta[q] > 0 ? 1.0 / beta[q] : 0.0;
    }
    if ((st = axpby<TG, TG>(S, scale, V, nullptr, V, nrhs, s)) != TTG_OK) return st;
    // Hessenberg H (m+1)×m per column, Givens (c, s), g.
    std::vector<double> H((size_t)nrhs * (m + 1) * m, 0.0), cs((size_t)nrhs * m), sn((size_t)nrhs * m),
        g((size_t)nrhs * (m + 1), 0.0);
    for (int q = 0; q < nrhs; ++q) g[(size_t)q * (m + 1)] = beta[q];
    auto h = [&](int q, int i, int j) -> double& { return H[((size_t)q * (m + 1) + i) * m + j]; };
    int k = 0;
    for (; k < m; ++k) {
        TG* vk = V + blk * k;
        TG* w = V + blk * (k + 1);
        // w = M⁻¹ (A v_k); FP64 Krylov vectors take A v_k in double-float
        // arithmetic (FP32 instruction rate, ~2^-46 accurate).
        if constexpr (sizeof(TG) == 8) {
            if (S->use_sliced) {
                if ((st = ttg_sliced_matmul_run(S->sl, (const double*)vk, nrhs, nullptr, (double*)t1, 0, s)) != TTG_OK) return st;
            } else if ((st = matmul_df(S, (const double*)vk, (double*)t1, nrhs, s)) != TTG_OK) {
                return st;
            }
        } else {
            if ((st = matmul<TG>(S, A, vk, nullptr, t1, t3, nrhs, 0, s)) != TTG_OK) return st;
        }
        if ((st = sweeps<TG, float>(S, L32, S->lt32.p, S->linv32.p, S->inv32.p, t1, t2, w, nrhs, grid, s)) != TTG_OK)
            return st;
        // Modified Gram-Schmidt.
        for (int j = 0; j <= k; ++j) {
            std::vector<double> d(nrhs), neg(nrhs);
            if ((st = colreduce<TG>(S, w, V + blk * j, nrhs, 0, d.data(), s)) != TTG_OK) return st;
            for (int q = 0; q < nrhs; ++q) {
                h(q, j, k) = d[q];
                neg[q] = -d[q];
            }
            if ((st = axpby<TG, TG>(S, neg, V + blk * j, &one, w, nrhs, s)) != TTG_OK) return st;
        }
        std::vector<double> nw(nrhs), sc(nrhs);
        if ((st = colreduce<TG>(S, w, w, nrhs, 0, nw.data(), s)) != TTG_OK) return st;
        bool done = true;
        for (int q = 0; q < nrhs; ++q) {
            const double hn = std::sqrt(nw[q]);
            h(q, k + 1, k) = hn;
            sc[q] = hn > 0 ? 1.0 / hn : 0.0;
            // Apply previous rotations to column k, then a new one.
            for (int i = 0; i < k; ++i) {
                const double a = h(q, i, k), b = h(q, i + 1, k);
                h(q, i, k) = cs[(size_t)q * m + i] * a + sn[(size_t)q * m + i] * b;
                h(q, i + 1, k) = -sn[(size_t)q * m + i] * a + cs[(size_t)q * m + i] * b;
            }
            const double a = h(q, k, k), b = h(q, k + 1, k);
            const double r = std::hypot(a, b);
            const double c = r > 0 ? a / r : 1.0, sv = r > 0 ? b / r : 0.0;
            cs[(size_t)q * m + k] = c;
            sn[(size_t)q * m + k] = sv;
            h(q, k, k) = r;
            h(q, k + 1, k) = 0.0;
            const double gk = g[(size_t)q * (m + 1) + k];
            g[(size_t)q * (m + 1) + k] = c * gk;
            g[(size_t)q * (m + 1) + k + 1] = -sv * gk;
            if (beta[q] > 0 && std::fabs(g[(size_t)q * (m + 1) + k + 1]) > inner_tol * beta[q]) done = false;
        }
        if ((st = axpby<TG, TG>(S, sc, w, nullptr, w, nrhs, s)) != TTG_OK) return st;
        if (done) {
            ++k;
            break;
        }
    }
    // y = H⁻¹ g per column; d = V y (times ‖r‖∞ undoes the scaling).
    std::vector<double> y((size_t)nrhs * k, 0.0);
    for (int q = 0; q < nrhs; ++q)
        for (int i = k - 1; i >= 0; --i) {
            double v = g[(size_t)q * (m + 1) + i];
            for (int j = i + 1; j < k; ++j) v -= h(q, i, j) * y[(size_t)q * k + j];
            y[(size_t)q * k + i] = h(q, i, i) != 0 ? v / h(q, i, i) : 0.0;
        }
    TTG_CUDA_CHECK(cudaMemsetAsync(S->D.p, 0, sizeof(double) * blk, s));
    for (int j = 0; j < k; ++j) {
        std::vector<double> c(nrhs);
        for (int q = 0; q < nrhs; ++q) c[q] = y[(size_t)q * k + j] * rn[q];
        if ((st = axpby<TG, double>(S, c, V + blk * j, &one, S->D.p, nrhs, s)) != TTG_OK) return st;
    }
    *iters = k;
    return TTG_OK;
}

}  // namespace

// TTG_SOLVE_VERBOSE=1 prints the time of each phase (host clock, after a
// stream synchronisation).
static bool solve_verbose() {
    static const bool v = getenv("TTG_SOLVE_VERBOSE") && atoi(getenv("TTG_SOLVE_VERBOSE")) > 0;
    return v;
}

namespace {
struct PhaseClock {
    cudaStream_t s;
    bool on;
    std::chrono::steady_clock::time_point t;
    PhaseClock(cudaStream_t s_, bool on_) : s(s_), on(on_), t(std::chrono::steady_clock::now()) {}
    void mark(const char* what) {
        if (!on) return;
        cudaStreamSynchronize(s);
        const auto n = std::chrono::steady_clock::now();
        fprintf(stderr, "[ttg solve] %-28s %9.3f ms\n", what, std::chrono::duration<double, std::milli>(n - t).count());
        t = n;
    }
};
}  // namespace

ttg_status ttg_solver_solve(ttg_solver* S, const double* pristine, const double* L64, const float* L32, const double* d_B,
                            double* d_X, const ttg_solve_opts* o, ttg_solve_report* rep, cudaStream_t s, bool* weak_first_step) {
    PhaseClock clk(s, solve_verbose());
    if (weak_first_step) *weak_first_step = false;
    const int nrhs = o->nrhs;
    if (nrhs < 1 || nrhs > kMaxRhs || !d_B || !d_X) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(S->ctx->device));
    const size_t blk = (size_t)S->N * nrhs;
    ttg_status st;
    for (auto* b : {&S->B, &S->X, &S->R, &S->D, &S->W, &S->T1, &S->T2})
        if ((st = b->ensure(blk)) != TTG_OK) return st;
    if ((st = S->P.ensure(blk * std::max(4, kDfMaxSplits))) != TTG_OK) return st;
    for (auto* b : {&S->f1, &S->f2, &S->f3})
        if ((st = b->ensure(blk * 4)) != TTG_OK) return st;  // also the FP32 matmul partials
    if ((st = S->part.ensure(128 * kMaxRhs)) != TTG_OK || (st = S->colv.ensure(kMaxRhs)) != TTG_OK ||
        (st = S->coefA.ensure(kMaxRhs)) != TTG_OK || (st = S->coefB.ensure(kMaxRhs)) != TTG_OK)
        return st;
    TTG_CUDA_CHECK(cudaMemsetAsync(S->d_err.p, 0, sizeof(int), s));
    clk.mark("buffers");
    if ((st = ensure_dense(S, pristine, s)) != TTG_OK) return st;
    clk.mark("dense copies of A");
    S->use_sliced = o->residual == 2 || (o->residual == 0 && S->N >= 256);
    if (S->use_sliced) {
        if ((st = ensure_sliced(S, s)) != TTG_OK || (st = ttg_sliced_reset_err(S->sl, s)) != TTG_OK) return st;
        clk.mark("digits of A");
    }
    TTG_CUDA_CHECK(cudaMemcpyAsync(S->B.p, d_B, sizeof(double) * blk, cudaMemcpyDeviceToDevice, s));
    const double tol = o->tol > 0 ? o->tol : 1e-14;
    const int max_outer = o->max_outer > 0 ? o->max_outer : 10;
    const int m = o->restart > 0 ? std::min(o->restart, 60) : 20;
    ttg_solve_report r{};
    r.status = TTG_OK;
    std::vector<double> be, rn;
    if (!S->mixed) {
        // FP64 direct: X = L⁻ᵀ L⁻¹ B.
        TTG_CUDA_CHECK(cudaMemcpyAsync(S->R.p, S->B.p, sizeof(double) * blk, cudaMemcpyDeviceToDevice, s));
        if ((st = sweeps<double, double>(S, L64, S->lt64.p, S->linv64.p, S->inv64.p, S->R.p, S->T1.p, S->X.p, nrhs,
                                         S->sweep_grid64, s)) != TTG_OK)
            return st;
        clk.mark("FP64 sweeps");
        if ((st = backward_errors(S, nrhs, s, be, rn)) != TTG_OK) return st;
        clk.mark("FP64 residual");
        r.gmres_prec = 64;
    } else {
        // x0 = M⁻¹ b (FP32 sweeps).
        std::vector<double> one(nrhs, 1.0);
        if ((st = axpby<double, float>(S, one, S->B.p, nullptr, S->f1.p, nrhs, s)) != TTG_OK) return st;
        if ((st = sweeps<float, float>(S, L32, S->lt32.p, S->linv32.p, S->inv32.p, S->f1.p, S->f2.p, S->f3.p, nrhs,
                                       S->sweep_grid32, s)) != TTG_OK)
            return st;
        if ((st = axpby<float, double>(S, one, S->f3.p, nullptr, S->X.p, nrhs, s)) != TTG_OK) return st;
        clk.mark("x0 = M^-1 b (FP32 sweeps)");
        int prec = o->gmres_prec == 64 ? 64 : 32;
        double prev = INFINITY;
        bool richardson = o->refine == 0 && prec == 32, after_richardson = false;
        // Relative GMRES tolerance per cycle: FP32 cycles gain ~1e-3 whatever
        // it is (their arithmetic bounds them), and 1e-5 ends them one
        // iteration earlier than 1e-6 at equal refinement steps (N = 32768,
        // alpha 1e-8 .. 1).
        const double inner_tol = o->inner_tol > 0 ? o->inner_tol : 1e-5;
        // Residuals that only steer an intermediate correction are computed
        // in double-float on the FP32 pipes (several times faster than FP64 on
        // this GPU).  A double-float residual is off by about 2^-48 of
        // ‖A‖‖x‖ (measured ~5e-15 in backward-error units at N = 32768), and
        // a correction steered by it cannot end below that, so double-float
        // steers only FP32 Krylov cycles (gain ~1e-3 each) while the backward
        // error is far above it, and the cycle after will be steered in FP64.
        // Convergence is decided, and the reported backward error taken, only
        // from an FP64 residual.
        constexpr double kDfTrust = 1e-11;     // predicted backward error below which FP64 is used at once
        constexpr double kDfFloor = 1e-11;     // smallest double-float value that steers a correction
        constexpr double kDfSafe = 5e-13;      // smallest outcome (value × last cycle's gain) it may steer to
        constexpr double kContraction = 1e-2;  // assumed gain of one cycle, for choosing the next residual
        double expect = INFINITY;              // predicted backward error of the current X
        for (int outer = 0;; ++outer) {
            bool df = !S->use_sliced && S->lo_valid && prec == 32 && expect >= kDfTrust;
            if ((st = backward_errors(S, nrhs, s, be, rn, df)) != TTG_OK) return st;
            double worst = *std::max_element(be.begin(), be.end());
            // A cycle that gains as much as the last one would land near the
            // double-float floor: steer it in FP64.
            const bool lands_low = outer > 0 && worst * std::min(1.0, worst / prev) < kDfSafe;
            if (df && (worst < kDfFloor || worst <= 2 * tol || lands_low)) {
                if (solve_verbose()) fprintf(stderr, "[ttg solve] outer %d double-float estimate %.3e\n", outer, worst);
                df = false;
                if ((st = backward_errors(S, nrhs, s, be, rn)) != TTG_OK) return st;
                worst = *std::max_element(be.begin(), be.end());
            }
            clk.mark(df ? "double-float residual" : S->use_sliced ? "sliced FP64 residual" : "FP64 residual");
            if (solve_verbose()) fprintf(stderr, "[ttg solve] outer %d backward error %.3e%s\n", outer, worst, df ? " (double-float)" : "");
            if (worst <= tol) break;
            expect = worst * kContraction;
            if (outer >= max_outer) {
                // The reported backward error is an FP64 one.
                if (df && (st = backward_errors(S, nrhs, s, be, rn)) != TTG_OK) return st;
                r.status = TTG_ENOCONV;
                break;
            }
            // Classic refinement first (auto mode): x += M⁻¹ r, one pair of
            // FP32 sweeps per step, while each step gains at least 10×; a
            // step that gains less hands over to GMRES for the rest.
            if (richardson && outer > 0 && worst > 0.1 * prev) {
                if (weak_first_step && outer == 1) {
                    if (solve_verbose()) fprintf(stderr, "[ttg solve] first refinement step gained %.3g: new factor\n", prev / worst);
                    *weak_first_step = true;
                    break;
                }
                richardson = false;
                after_richardson = true;
                if (solve_verbose()) fprintf(stderr, "[ttg solve] outer %d: refinement step gained %.3g, GMRES from here\n", outer,
                                             prev / worst);
            }
            if (richardson) {
                std::vector<double> inv(nrhs), ones(nrhs, 1.0);
                for (int q = 0; q < nrhs; ++q) inv[q] = rn[q] > 0 ? 1.0 / rn[q] : 0.0;
                if ((st = axpby<double, float>(S, inv, S->R.p, nullptr, S->f1.p, nrhs, s)) != TTG_OK) return st;
                if ((st = sweeps<float, float>(S, L32, S->lt32.p, S->linv32.p, S->inv32.p, S->f1.p, S->f2.p, S->f3.p, nrhs,
                                               S->sweep_grid32, s)) != TTG_OK)
                    return st;
                if ((st = axpby<float, double>(S, rn, S->f3.p, &ones, S->X.p, nrhs, s)) != TTG_OK) return st;
                clk.mark("refinement step (FP32 sweeps)");
                r.outer = outer + 1;
                prev = worst;
                continue;
            }
            // Switch to FP64 Krylov work when FP32 stops gaining (auto mode;
            // not on the first GMRES cycle after classic steps stalled).
            if (o->gmres_prec == 0 && prec == 32 && outer > 0 && worst > 0.1 * prev && !after_richardson) prec = 64;
            after_richardson = false;
            prev = worst;
            if (df && prec == 64) {  // an FP64 Krylov cycle is steered by an FP64 residual
                if ((st = backward_errors(S, nrhs, s, be, rn)) != TTG_OK) return st;
                clk.mark("FP64 residual");
            }
            int it = 0;
            st = prec == 32 ? gmres_cycle<float>(S, L32, nrhs, m, prec == 32 ? std::max(inner_tol, 1e-6) : inner_tol, s, &it)
                            : gmres_cycle<double>(S, L32, nrhs, m, inner_tol, s, &it);
            if (st != TTG_OK) return st;
            if (solve_verbose()) fprintf(stderr, "[ttg solve] GMRES(FP%d) %d iterations\n", prec, it);
            clk.mark("GMRES cycle");
            // An FP32 cycle that used its whole restart length did not reach
            // its tolerance: the FP32 operators are too coarse for this
            // matrix, so the next cycles use FP64 Krylov vectors (auto mode).
            if (o->gmres_prec == 0 && prec == 32 && it >= m) prec = 64;
            r.inner += it;
            r.outer = outer + 1;
            std::vector<double> ones(nrhs, 1.0);
            if ((st = axpby<double, double>(S, ones, S->D.p, &ones, S->X.p, nrhs, s)) != TTG_OK) return st;
        }
        r.gmres_prec = prec;
    }
    r.bwd_err = be.empty() ? 0.0 : *std::max_element(be.begin(), be.end());
    r.anorm_inf = S->anorm_inf;
    TTG_CUDA_CHECK(cudaMemcpyAsync(d_X, S->X.p, sizeof(double) * blk, cudaMemcpyDeviceToDevice, s));
    int h_err[2] = {0, 0};
    TTG_CUDA_CHECK(cudaMemcpyAsync(&h_err[0], S->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (S->use_sliced) TTG_CUDA_CHECK(cudaMemcpyAsync(&h_err[1], ttg_sliced_err(S->sl), sizeof(int), cudaMemcpyDeviceToHost, s));
    TTG_CUDA_CHECK(cudaStreamSynchronize(s));
    if (h_err[0] || h_err[1]) r.status = TTG_ETIMEOUT;  // a sweep or a product gave up waiting: X is not valid
    if (rep) *rep = r;
    return r.status;
}

// Test hook (no device work): the claim order of the TMA sweeps over nb
// block rows of bs[i] rows — forward items, then backward, each an item
// index in step order — as the solver builds it.  Returns the number of
// items (written when it is at most cap), or -1 for bad sizes.
extern "C" int64_t ttg_internal_sweep_order(int32_t nb, const int32_t* bs, int32_t* out, int64_t cap) {
    if (nb < 1 || !bs) return -1;
    for (int i = 0; i < nb; ++i)
        if (bs[i] < 1) return -1;
    std::vector<int> sp, fwd, bwd, order;
    if (!sweep_step_tables(nb, bs, sp, fwd, bwd)) return -1;
    sweep_claim_order(nb, sp, fwd, bwd, order);
    if (out && (int64_t)order.size() <= cap) std::copy(order.begin(), order.end(), out);
    return (int64_t)order.size();
}
