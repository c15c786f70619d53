// ttg_batch.cu — many independent SPD factor-and-solve systems in one launch
// of the persistent executor (include/ttg_batch.h), and the construction of
// their device task graphs (batch_graph.h, which describes the DAG).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/ttg.h"
#include "../../include/ttg_batch.h"
#include "../../include/ttg_philox.h"
#include "batch_graph.h"
#include "ttg_mixed_api.h"
#include "ttg_internal.h"

namespace {

ttg_op make_op(int kind, int prec, int m, int n, int k, const void* a, int lda, const void* b, int ldb, void* c, int ldc,
               double alpha, double beta, int flags = 0, void* aux = nullptr) {
    ttg_op o{};
    o.kind = kind;
    o.prec = prec;
    o.m = m;
    o.n = n;
    o.k = k;
    o.a = a;
    o.lda = lda;
    o.b = b;
    o.ldb = ldb;
    o.c = c;
    o.ldc = ldc;
    o.alpha = alpha;
    o.beta = beta;
    o.flags = flags;
    o.aux = aux;
    return o;
}

ttg_op nop() { return make_op(TTG_OP_NOP, TTG_PREC_F64, 0, 0, 0, nullptr, 0, nullptr, 0, nullptr, 0, 0.0, 0.0); }

// Right-hand sides: system s, element (q, r) of its nrhs × N row block is
// entry (r, q) of the column-major N × nrhs N(0,1) array of (seed + s, stream 1).
__global__ void batch_rhs_kernel(const int* __restrict__ Ns, const int64_t* __restrict__ vbase, int n_sys, int nrhs, uint32_t seed,
                                 double* B) {
    for (int s = blockIdx.x; s < n_sys; s += gridDim.x) {
        const int N = Ns[s];
        double* Bs = B + vbase[s];
        for (int e = threadIdx.x; e < N * nrhs; e += blockDim.x) {
            const int r = e % N, q = e / N;
            Bs[q + (int64_t)r * nrhs] = ttg_normal_at((uint64_t)e, seed + (uint32_t)s, TTG_STREAM_RHS);
        }
    }
}

// Backward errors, one block (256 threads) per system: max over columns q of
// ‖b_q − A x_q‖∞ / (‖A‖∞ ‖x_q‖∞), A from the packed lower tiles (full
// diagonal tiles).
__global__ void batch_bwd_kernel(const int* __restrict__ Ns, const int* __restrict__ tiles, const int64_t* __restrict__ tbase,
                                 const int64_t* __restrict__ vbase, int n_sys, int nrhs, const double* __restrict__ A,
                                 const double* __restrict__ B, const double* __restrict__ X, double* err) {
    __shared__ double s_r[16][8], s_x[16][8], s_a[8];
    for (int s = blockIdx.x; s < n_sys; s += gridDim.x) {
        const int N = Ns[s], t = tiles[s];
        const int nb = (N + t - 1) / t;
        const double* As = A + tbase[s];
        const double* Bs = B + vbase[s];
        const double* Xs = X + vbase[s];
        auto bs = [&](int i) { return i < nb - 1 ? t : N - (nb - 1) * t; };
        auto off = [&](int i, int j) {
            return (int64_t)t * ((int64_t)j * N - (int64_t)t * j * (j - 1) / 2) + (int64_t)(i - j) * t * bs(j);
        };
        double rmax[16], xmax[16], amax = 0.0;
        for (int q = 0; q < 16; ++q) rmax[q] = xmax[q] = 0.0;
        for (int r = threadIdx.x; r < N; r += blockDim.x) {
            double acc[16];
            for (int q = 0; q < 16; ++q) acc[q] = q < nrhs ? Bs[q + (int64_t)r * nrhs] : 0.0;
            double asum = 0.0;
            const int bi = r / t, li = r - bi * t;
            for (int c = 0; c < N; ++c) {
                const int bj = c / t, lj = c - bj * t;
                const double a = r >= c ? As[off(bi, bj) + li + (int64_t)lj * bs(bi)] : As[off(bj, bi) + lj + (int64_t)li * bs(bj)];
                asum += fabs(a);
                for (int q = 0; q < 16; ++q)
                    if (q < nrhs) acc[q] = fma(-a, Xs[q + (int64_t)c * nrhs], acc[q]);
            }
            amax = fmax(amax, asum);
            for (int q = 0; q < 16; ++q)
                if (q < nrhs) {
                    rmax[q] = fmax(rmax[q], fabs(acc[q]));
                    xmax[q] = fmax(xmax[q], fabs(Xs[q + (int64_t)r * nrhs]));
                    if (acc[q] != acc[q]) rmax[q] = INFINITY;  // a NaN residual never passes
                }
        }
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        for (int o = 16; o > 0; o >>= 1) {
            amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
            for (int q = 0; q < 16; ++q) {
                rmax[q] = fmax(rmax[q], __shfl_xor_sync(0xffffffffu, rmax[q], o));
                xmax[q] = fmax(xmax[q], __shfl_xor_sync(0xffffffffu, xmax[q], o));
            }
        }
        if (lane == 0) {
            s_a[warp] = amax;
            for (int q = 0; q < 16; ++q) {
                s_r[q][warp] = rmax[q];
                s_x[q][warp] = xmax[q];
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const int nw = blockDim.x >> 5;
            double a = 0.0, worst = 0.0;
            for (int w = 0; w < nw; ++w) a = fmax(a, s_a[w]);
            for (int q = 0; q < nrhs; ++q) {
                double rq = 0.0, xq = 0.0;
                for (int w = 0; w < nw; ++w) {
                    rq = fmax(rq, s_r[q][w]);
                    xq = fmax(xq, s_x[q][w]);
                }
                const double be = xq > 0 ? rq / (a * xq) : (rq > 0 ? INFINITY : 0.0);
                worst = (be != be) ? INFINITY : fmax(worst, be);
            }
            err[s] = worst;
        }
        __syncthreads();
    }
}

}  // namespace

namespace ttg {
namespace batch {


// Factor DAG of one system (FP64 in place on W64, or mixed: CONVERT tasks,
// FP32 working tiles, FP64 POTRF scratch); fills the potrf and trsm ids the
// solve depends on.
static void build_factor(Graph& g, const System& S, std::vector<int>& potrf, std::vector<int>& trsm) {
    const int nb = S.nb;
    const bool mx = S.mixed;
    const int prec = mx ? TTG_PREC_MIXED : TTG_PREC_F64;
    auto W = [&](int i, int j) -> void* { return mx ? (void*)(S.W32 + S.off(i, j)) : (void*)(S.W64 + S.off(i, j)); };
    auto T = [&](int i, int j) { return i + j * nb; };
    auto G = [&](int k, int i, int j) { return ((size_t)k * nb + i) * nb + j; };
    potrf.assign(nb, -1);
    trsm.assign((size_t)nb * nb, -1);
    std::vector<int> gemm((size_t)nb * nb * nb, -1), cvt((size_t)nb * nb, -1);
    // Thousands of systems keep every block busy: FP64 tile updates take one
    // part per 128×128 output block and TRSMs one per 128 rows (the
    // single-plan rule splits small FP64 tiles finer, to shorten one
    // factorisation's chain).
    auto c128 = [](int x) { return (x + 127) / 128; };
    auto throughput = [&](ttg_op op) {
        if (op.prec != TTG_PREC_F64) return op;
        if (op.kind == TTG_OP_GEMM_NT) op.parts = std::min(16, c128(op.m) * c128(op.n));
        else if (op.kind == TTG_OP_SYRK_LN) op.parts = std::min(16, c128(op.n) * (c128(op.n) + 1) / 2);
        else if (op.kind == TTG_OP_TRSM_RLTN) op.parts = std::min(8, c128(op.m));
        return op;
    };
    // Tensor-core systems: split-BF16 updates (mixed flags 3) on the panel
    // slots that each TRSM publishes (ldb = its slot, k = its block row);
    // an update's lda/ldb are the slots of L_ik and L_jk.
    const bool tc = mx && S.tc_tables;
    constexpr int kTcSplitBF16 = 3;
    for (int j = 0; j < nb; ++j) {
        ttg_op po = make_op(TTG_OP_POTRF_L, prec, S.bs(j), S.bs(j), 0, nullptr, 0, nullptr, 0, W(j, j), S.bs(j), 1.0, 0.0, 0,
                            mx ? (void*)(S.D64 + (size_t)j * S.tile * S.tile) : nullptr);
        po.parts = S.potrf_parts;
        potrf[j] = g.add(po);
        for (int i = j + 1; i < nb; ++i)
            trsm[T(i, j)] = g.add(tc ? make_op(TTG_OP_TRSM_RLTN, prec, S.bs(i), S.bs(j), i, W(j, j), S.bs(j), nullptr, S.slot(i, j),
                                               W(i, j), S.bs(i), 1.0, 0.0, kTcSplitBF16, S.tc_tables)
                                     : throughput(make_op(TTG_OP_TRSM_RLTN, prec, S.bs(i), S.bs(j), 0, W(j, j), S.bs(j), nullptr,
                                                          0, W(i, j), S.bs(i), 1.0, 0.0, mx ? 1 : 0)));
        for (int k = 0; k < j; ++k)
            for (int i = j; i < nb; ++i) {
                if (tc) {
                    gemm[G(k, i, j)] =
                        g.add(make_op(i == j ? TTG_OP_SYRK_LN : TTG_OP_GEMM_NT, prec, S.bs(i), S.bs(j), S.bs(k), nullptr, S.slot(i, k),
                                      nullptr, S.slot(j, k), W(i, j), S.bs(i), -1.0, 1.0, kTcSplitBF16, S.tc_tables));
                    continue;
                }
                gemm[G(k, i, j)] = g.add(throughput(
                    i == j ? make_op(TTG_OP_SYRK_LN, prec, S.bs(i), S.bs(i), S.bs(k), W(i, k), S.bs(i), nullptr, 0, W(i, i), S.bs(i),
                                     -1.0, 1.0, mx ? 1 : 0)
                           : make_op(TTG_OP_GEMM_NT, prec, S.bs(i), S.bs(j), S.bs(k), W(i, k), S.bs(i), W(j, k), S.bs(j), W(i, j),
                                     S.bs(i), -1.0, 1.0, mx ? 1 : 0)));
            }
    }
    if (mx)
        for (int j = 0; j < nb; ++j)
            for (int i = j; i < nb; ++i)
                cvt[T(i, j)] = g.add(make_op(TTG_OP_CONVERT, TTG_PREC_F64, S.bs(i), S.bs(j), 0, S.A64 + S.off(i, j), S.bs(i), nullptr,
                                             0, W(i, j), S.bs(i), 1.0, 0.0, 2));
    for (int j = 0; j < nb; ++j) {
        for (int i = j + 1; i < nb; ++i) {
            g.edge(potrf[j], trsm[T(i, j)]);
            for (int m = j + 1; m < i; ++m) g.edge(trsm[T(i, j)], gemm[G(j, i, m)]);
            for (int m = i; m < nb; ++m) g.edge(trsm[T(i, j)], gemm[G(j, m, i)]);
        }
        for (int k = 0; k < j; ++k)
            for (int i = j; i < nb; ++i) {
                const int t = gemm[G(k, i, j)];
                if (k < j - 1) g.edge(t, gemm[G(k + 1, i, j)]);
                else if (i == j) g.edge(t, potrf[i]);
                else g.edge(t, trsm[T(i, j)]);
            }
        if (mx)
            for (int i = j; i < nb; ++i) {
                const int first = j == 0 ? (i == 0 ? potrf[0] : trsm[T(i, 0)]) : gemm[G(0, i, j)];
                g.edge(cvt[T(i, j)], first);
            }
    }
}

// Block solve L Lᵀ x = v in place on the row blocks V (ld nrhs) with the
// factor tiles (FP32 when f32).  pre[i]: a task that must precede any access
// to block i (or -1); potrf / trsm: the factor's tasks (empty for a resident
// factor).  Returns the final task of every block.
static std::vector<int> build_solve(Graph& g, const System& S, void* V, bool f32, const std::vector<int>& potrf,
                             const std::vector<int>& trsm, const std::vector<int>& pre) {
    const int nb = S.nb, nr = S.nrhs;
    const int prec = f32 ? TTG_PREC_MIXED : TTG_PREC_F64;
    const size_t es = f32 ? sizeof(float) : sizeof(double);
    const bool dep = !potrf.empty();
    auto Vb = [&](int i) { return (void*)((char*)V + es * (size_t)S.displ(i) * nr); };
    auto F = [&](int i, int j) -> const void* { return f32 ? (const void*)(S.W32 + S.off(i, j)) : (const void*)(S.W64 + S.off(i, j)); };
    auto T = [&](int i, int j) { return i + j * nb; };
    std::vector<int> fs(nb), fu((size_t)nb * nb, -1), bsv(nb), bu((size_t)nb * nb, -1);
    for (int i = 0; i < nb; ++i) {
        for (int j = 0; j < i; ++j)
            fu[T(i, j)] = g.add(make_op(TTG_OP_GEMM_NT, prec, nr, S.bs(i), S.bs(j), Vb(j), nr, F(i, j), S.bs(i), Vb(i), nr, -1.0, 1.0));
        fs[i] = g.add(make_op(TTG_OP_TRSM_RLTN, prec, nr, S.bs(i), 0, F(i, i), S.bs(i), nullptr, 0, Vb(i), nr, 1.0, 0.0));
    }
    for (int i = nb - 1; i >= 0; --i) {
        for (int j = nb - 1; j > i; --j)
            bu[T(i, j)] = g.add(make_op(TTG_OP_GEMM_NN, prec, nr, S.bs(i), S.bs(j), Vb(j), nr, F(j, i), S.bs(j), Vb(i), nr, -1.0, 1.0));
        bsv[i] = g.add(make_op(TTG_OP_TRSM_RLNN, prec, nr, S.bs(i), 0, F(i, i), S.bs(i), nullptr, 0, Vb(i), nr, 1.0, 0.0));
    }
    for (int i = 0; i < nb; ++i) {
        if (pre[i] >= 0) g.edge(pre[i], i == 0 ? fs[0] : fu[T(i, 0)]);
        if (dep) g.edge(potrf[i], fs[i]);
        if (i > 0) g.edge(fu[T(i, i - 1)], fs[i]);
        for (int j = 0; j < i; ++j) {
            const int t = fu[T(i, j)];
            g.edge(fs[j], t);
            if (dep) g.edge(trsm[T(i, j)], t);
            if (j > 0) g.edge(fu[T(i, j - 1)], t);
        }
        if (i == nb - 1) {
            g.edge(fs[i], bsv[i]);
        } else {
            g.edge(fs[nb - 1], bu[T(i, nb - 1)]);  // every forward task is done (see batch_graph.h)
            g.edge(fs[i], bu[T(i, nb - 1)]);
            for (int j = nb - 1; j > i; --j) {
                const int t = bu[T(i, j)];
                g.edge(bsv[j], t);
                if (j < nb - 1) g.edge(bu[T(i, j + 1)], t);
            }
            g.edge(bu[T(i, i + 1)], bsv[i]);
        }
    }
    return bsv;
}

void add_system(Graph& g, const System& S) {
    const int nb = S.nb, nr = S.nrhs;
    std::vector<int> potrf, trsm;
    if (!S.factored) build_factor(g, S, potrf, trsm);
    if (!S.mixed) {
        // FP64: the solve runs in place on X (a copy of B made before the launch).
        build_solve(g, S, S.X, false, potrf, trsm, std::vector<int>(nb, -1));
        return;
    }
    auto vec = [&](auto* base, int i) { return base + (size_t)S.displ(i) * nr; };
    // x0: d = b (FP32), solve, x = d.
    std::vector<int> pre(nb), last(nb);
    for (int i = 0; i < nb; ++i)
        pre[i] = g.add(make_op(TTG_OP_CONVERT, TTG_PREC_F64, nr, S.bs(i), 0, vec(S.B, i), nr, nullptr, 0, vec(S.D32, i), nr, 1.0, 0.0, 2));
    std::vector<int> done = build_solve(g, S, S.D32, true, potrf, trsm, pre);
    for (int i = 0; i < nb; ++i) {
        last[i] = g.add(make_op(TTG_OP_CONVERT, TTG_PREC_F64, nr, S.bs(i), 0, vec(S.D32, i), nr, nullptr, 0, vec(S.X, i), nr, 1.0, 0.0, 1));
        g.edge(done[i], last[i]);
    }
    for (int step = 0; step < S.ir_steps; ++step) {
        const int xb = g.add(nop());  // x is complete
        for (int i = 0; i < nb; ++i) g.edge(last[i], xb);
        const int rb = g.add(nop());  // every row's residual has read x
        std::vector<int> dcv(nb);
        for (int i = 0; i < nb; ++i) {
            // r_i = b_i − Σ_j A_ij x_j, chained over j.
            int prev = g.add(make_op(TTG_OP_CONVERT, TTG_PREC_F64, nr, S.bs(i), 0, vec(S.B, i), nr, nullptr, 0, vec(S.R, i), nr, 1.0, 0.0, 0));
            g.edge(xb, prev);
            for (int j = 0; j < nb; ++j) {
                const bool low = j <= i;
                const double* Aij = S.A64 + (low ? S.off(i, j) : S.off(j, i));
                const int t = g.add(make_op(low ? TTG_OP_GEMM_NT : TTG_OP_GEMM_NN, TTG_PREC_F64, nr, S.bs(i), S.bs(j), vec(S.X, j), nr,
                                            Aij, low ? S.bs(i) : S.bs(j), vec(S.R, i), nr, -1.0, 1.0));
                g.edge(prev, t);
                prev = t;
            }
            g.edge(prev, rb);
            dcv[i] = g.add(make_op(TTG_OP_CONVERT, TTG_PREC_F64, nr, S.bs(i), 0, vec(S.R, i), nr, nullptr, 0, vec(S.D32, i), nr, 1.0, 0.0, 2));
            g.edge(prev, dcv[i]);
        }
        done = build_solve(g, S, S.D32, true, potrf, trsm, dcv);
        for (int i = 0; i < nb; ++i) {
            last[i] = g.add(make_op(TTG_OP_CONVERT, TTG_PREC_F64, nr, S.bs(i), 0, vec(S.D32, i), nr, nullptr, 0, vec(S.X, i), nr, 1.0, 1.0, 1));
            g.edge(done[i], last[i]);
            g.edge(rb, last[i]);
        }
    }
}

ttg_status Graph::finish(bool critical_path) {
    const int n = (int)ops.size();
    init.assign(n, 0);
    ptr.assign(n + 1, 0);
    for (auto& e : edges) {
        ++ptr[e.first + 1];
        ++init[e.second];
    }
    for (int t = 0; t < n; ++t) ptr[t + 1] += ptr[t];
    idx.resize(edges.size());
    {
        std::vector<int64_t> fill(ptr.begin(), ptr.end() - 1);
        for (auto& e : edges) idx[fill[e.first]++] = e.second;
    }
    edges.clear();
    prio.assign(n, 0.0);
    if (critical_path) {
        ttg_graph_desc d = desc();
        return ttg_critical_path_priority(&d, prio.data());
    }
    return TTG_OK;
}

}  // namespace batch
}  // namespace ttg

using namespace ttg::batch;

struct ttg_batch {
    ttg_ctx* ctx = nullptr;
    ttg_batch_args a{};
    std::vector<int32_t> sizes;
    std::vector<System> sys;
    bool mixed = false;
    int64_t tile_elems = 0, vec_elems = 0;
    double* A64 = nullptr;  // FP64 input tiles of all systems (full diagonal tiles)
    double* W64 = nullptr;  // FP64: factor tiles; mixed: FP64 scratch of the diagonal POTRFs
    float* W32 = nullptr;   // mixed: FP32 working tiles
    double *B = nullptr, *X = nullptr, *R = nullptr;
    float* D32 = nullptr;
    // Tensor-core data of the mixed systems whose tiles allow it (split-BF16
    // updates): headers, panel slots, slot and block-row scales, and the
    // list of diagonal tiles whose block-row scales each run computes.
    uint8_t* tc_hdr = nullptr;
    __nv_bfloat16* tc_slots = nullptr;
    float* tc_scales = nullptr;
    TcRowScaleItem* tc_rs = nullptr;
    int n_tc = 0, n_rs = 0;
    Graph g;
    uint64_t gen = 0;  // context graph generation of our upload
    cudaGraphExec_t gexec = nullptr;
    cudaStream_t gstream = nullptr;  // the stream the graph was recorded on
    cudaStream_t own = nullptr;      // used for a NULL stream (the legacy stream cannot be recorded)
    int gworkers = 0;
    bool gen_recorded_run = false;  // the recording counted the executor kernel once already
    double flops = 0.0;
};

namespace {

template <class P>
ttg_status dev_alloc(P** p, size_t count) {
    *p = nullptr;
    if (count == 0) return TTG_OK;
    TTG_CUDA_CHECK(cudaMalloc((void**)p, sizeof(P) * count));
    TTG_CUDA_CHECK(cudaMemset(*p, 0, sizeof(P) * count));
    return TTG_OK;
}

ttg_status batch_upload(ttg_batch* b) {
    ttg_graph_desc d = b->g.desc();
    ttg_status st = ttg_graph_upload(b->ctx, &d);
    if (st != TTG_OK) return st;
    b->gen = ttg_graph_generation(b->ctx);
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    return TTG_OK;
}

// Record the restore copies and the executor run on stream s into a CUDA graph.
ttg_status batch_record(ttg_batch* b, cudaStream_t s) {
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    if (b->mixed) ttg_mixed_set_tc(b->ctx, b->n_tc > 0);  // the launch parameters are recorded with the graph
    TTG_CUDA_CHECK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    ttg_status st = TTG_OK;
    // Block-row scales of the tensor-core systems (from their FP64 inputs).
    if (b->n_rs > 0) st = ttg_mixed_row_scales(b->tc_rs, b->n_rs, s);
    if (!b->mixed) {
        if (cudaMemcpyAsync(b->W64, b->A64, sizeof(double) * b->tile_elems, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(b->X, b->B, sizeof(double) * b->vec_elems, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            st = TTG_ECUDA;
    }
    if (st == TTG_OK) st = ttg_enqueue_run(b->ctx, s);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &graph);
    if (st != TTG_OK || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        if (e != cudaSuccess) ttg_set_last_cuda_error(e, "cudaStreamEndCapture (batch)", __FILE__, __LINE__);
        return st != TTG_OK ? st : TTG_ECUDA;
    }
    e = cudaGraphInstantiate(&b->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        b->gexec = nullptr;
        ttg_set_last_cuda_error(e, "cudaGraphInstantiate (batch)", __FILE__, __LINE__);
        return TTG_ECUDA;
    }
    b->gstream = s;
    b->gworkers = ttg_workers(b->ctx);
    b->gen_recorded_run = false;
    return TTG_OK;
}

}  // namespace

extern "C" ttg_status ttg_batch_create(ttg_ctx* ctx, const ttg_batch_args* args, ttg_batch** out) {
    if (!ctx || !args || !out || args->n_systems < 1 || !args->sizes || args->tile < 1 || args->nrhs < 1 || args->nrhs > 16 ||
        args->ir_steps < 0 || (args->precision != TTG_PREC_F64 && args->precision != TTG_PREC_MIXED))
        return TTG_EINVAL;
    *out = nullptr;
    for (int i = 0; i < args->n_systems; ++i)
        if (args->sizes[i] < 1 || args->sizes[i] > 131072) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(ctx->device));
    ttg_batch* b = new ttg_batch();
    b->ctx = ctx;
    b->a = *args;
    b->sizes.assign(args->sizes, args->sizes + args->n_systems);
    b->a.sizes = b->sizes.data();
    b->mixed = args->precision == TTG_PREC_MIXED;
    b->sys.resize(args->n_systems);
    std::vector<int64_t> tb(args->n_systems), vb(args->n_systems);
    for (int s = 0; s < args->n_systems; ++s) {
        System& S = b->sys[s];
        S.set_size(b->sizes[s], args->tile);
        S.mixed = b->mixed;
        S.nrhs = args->nrhs;
        S.ir_steps = args->ir_steps;
        tb[s] = b->tile_elems;
        vb[s] = b->vec_elems;
        b->tile_elems += (S.elems() + 31) / 32 * 32;  // the next system starts 256-byte aligned
        b->vec_elems += ((int64_t)S.N * args->nrhs + 31) / 32 * 32;
        b->flops += S.flops();
    }
    ttg_status st;
    if ((st = dev_alloc(&b->A64, b->tile_elems)) != TTG_OK || (st = dev_alloc(&b->W64, b->tile_elems)) != TTG_OK ||
        (st = dev_alloc(&b->B, b->vec_elems)) != TTG_OK || (st = dev_alloc(&b->X, b->vec_elems)) != TTG_OK ||
        (b->mixed && ((st = dev_alloc(&b->W32, b->tile_elems)) != TTG_OK || (st = dev_alloc(&b->R, b->vec_elems)) != TTG_OK ||
                      (st = dev_alloc(&b->D32, b->vec_elems)) != TTG_OK))) {
        ttg_batch_destroy(b);
        return st;
    }
    // Tensor-core systems (mixed, tiles a multiple of 128 up to 512, more
    // than one tile row): headers, slots (128-byte aligned per system) and
    // scales, written once here.
    std::vector<size_t> slot_base(args->n_systems, 0), scale_base(args->n_systems, 0), hdr_index(args->n_systems, 0);
    if (b->mixed) {
        size_t slots = 0, scales = 0;
        for (int s = 0; s < args->n_systems; ++s) {
            const System& S = b->sys[s];
            if (!System::tc_fits(S.N, S.tile)) continue;
            hdr_index[s] = (size_t)b->n_tc++;
            slot_base[s] = slots;
            slots += (ttg_mixed_tc_slot_elems(S.tile, S.nb) + 63) / 64 * 64;
            scale_base[s] = scales;
            scales += (size_t)(S.nb * (S.nb + 1) / 2 + S.nb + 31) / 32 * 32;
            b->n_rs += S.nb;
        }
        if (b->n_tc > 0) {
            std::vector<uint8_t> hh(kTcHeaderBytes * (size_t)b->n_tc);
            std::vector<TcRowScaleItem> rs;
            rs.reserve(b->n_rs);
            if ((st = dev_alloc(&b->tc_hdr, kTcHeaderBytes * (size_t)b->n_tc)) != TTG_OK || (st = dev_alloc(&b->tc_slots, slots)) != TTG_OK ||
                (st = dev_alloc(&b->tc_scales, scales)) != TTG_OK || (st = dev_alloc(&b->tc_rs, (size_t)b->n_rs)) != TTG_OK) {
                ttg_batch_destroy(b);
                return st;
            }
            for (int s = 0; s < args->n_systems; ++s) {
                System& S = b->sys[s];
                if (!System::tc_fits(S.N, S.tile)) continue;
                const size_t h = hdr_index[s];
                float* slot_scale = b->tc_scales + scale_base[s];
                float* rowscale = slot_scale + S.nb * (S.nb + 1) / 2;
                st = ttg_mixed_tc_header(hh.data() + kTcHeaderBytes * h, b->tc_hdr + kTcHeaderBytes * h, b->tc_slots + slot_base[s],
                                         slot_scale, rowscale, S.tile, S.nb, &S.tc_tables);
                if (st != TTG_OK) {
                    ttg_batch_destroy(b);
                    return st;
                }
                for (int i = 0; i < S.nb; ++i)
                    rs.push_back(TcRowScaleItem{b->A64 + tb[s] + S.off(i, i), S.bs(i), S.bs(i), rowscale + i});
            }
            cudaError_t e = cudaMemcpy(b->tc_hdr, hh.data(), hh.size(), cudaMemcpyHostToDevice);
            if (e == cudaSuccess) e = cudaMemcpy(b->tc_rs, rs.data(), sizeof(TcRowScaleItem) * rs.size(), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) {
                ttg_set_last_cuda_error(e, "cudaMemcpy (tensor-core tables)", __FILE__, __LINE__);
                ttg_batch_destroy(b);
                return TTG_ECUDA;
            }
        }
    }
    for (int s = 0; s < args->n_systems; ++s) {
        System& S = b->sys[s];
        S.A64 = b->A64 + tb[s];
        S.W64 = b->W64 + tb[s];
        S.B = b->B + vb[s];
        S.X = b->X + vb[s];
        if (b->mixed) {
            S.D64 = b->W64 + tb[s];  // nb·tile² <= the system's tile elements
            S.W32 = b->W32 + tb[s];
            S.R = b->R + vb[s];
            S.D32 = b->D32 + vb[s];
        }
        // Thousands of independent systems keep every block busy: a POTRF
        // team's blocks would mostly wait on the pivot chain, so each
        // diagonal POTRF runs on one block (10,000 systems, N in [32, 2048]:
        // 5,697 systems/s mixed and 3,026 FP64, against 4,756 and 2,836 with
        // teams of n/16).
        S.potrf_parts = 1;
        add_system(b->g, S);
    }
    if ((st = b->g.finish(args->priority == 0)) != TTG_OK) {
        ttg_batch_destroy(b);
        return st;
    }
    if ((st = batch_upload(b)) != TTG_OK) {
        ttg_batch_destroy(b);
        return st;
    }
    *out = b;
    return TTG_OK;
}

extern "C" void ttg_batch_destroy(ttg_batch* b) {
    if (!b) return;
    cudaSetDevice(b->ctx->device);
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->own) cudaStreamDestroy(b->own);
    for (void* p : {(void*)b->A64, (void*)b->W64, (void*)b->W32, (void*)b->B, (void*)b->X, (void*)b->R, (void*)b->D32,
                    (void*)b->tc_hdr, (void*)b->tc_slots, (void*)b->tc_scales, (void*)b->tc_rs})
        if (p) cudaFree(p);
    delete b;
}

extern "C" ttg_status ttg_batch_generate(ttg_batch* b, void* stream) {
    if (!b) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(b->ctx->device));
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<int32_t> bs;
    for (size_t i = 0; i < b->sys.size(); ++i) {
        const System& S = b->sys[i];
        bs.assign(S.nb, 0);
        for (int t = 0; t < S.nb; ++t) bs[t] = S.bs(t);
        ttg_status st = ttg_gen_gram_tiles(b->ctx, S.N, bs.data(), S.nb, b->a.alpha, b->a.seed + (uint32_t)i, S.A64, stream);
        if (st != TTG_OK) return st;
    }
    const int n = (int)b->sys.size();
    std::vector<int> Ns(n);
    std::vector<int64_t> vb(n);
    for (int i = 0; i < n; ++i) {
        Ns[i] = b->sys[i].N;
        vb[i] = b->sys[i].B - b->B;
    }
    int* dN = nullptr;
    int64_t* dV = nullptr;
    cudaError_t e = cudaMalloc((void**)&dN, sizeof(int) * n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&dV, sizeof(int64_t) * n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dN, Ns.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dV, vb.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        ttg_note_launch();
        batch_rhs_kernel<<<std::min(n, 4096), 256, 0, s>>>(dN, dV, n, b->a.nrhs, b->a.seed, b->B);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (dN) cudaFree(dN);
    if (dV) cudaFree(dV);
    if (e != cudaSuccess) {
        ttg_set_last_cuda_error(e, "batch right-hand sides", __FILE__, __LINE__);
        return TTG_ECUDA;
    }
    return TTG_OK;
}

extern "C" ttg_status ttg_batch_set_system(ttg_batch* b, int32_t i, const double* h_A, const double* h_B, void* stream) {
    if (!b || i < 0 || i >= (int)b->sys.size()) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(b->ctx->device));
    cudaStream_t s = (cudaStream_t)stream;
    const System& S = b->sys[i];
    const int nr = b->a.nrhs;
    if (h_A) {
        std::vector<double> t(S.elems());
        for (int j = 0; j < S.nb; ++j)
            for (int ii = j; ii < S.nb; ++ii) {
                double* T = t.data() + S.off(ii, j);
                for (int c = 0; c < S.bs(j); ++c)
                    for (int r = 0; r < S.bs(ii); ++r) {
                        int gr = S.displ(ii) + r, gc = S.displ(j) + c;
                        if (gr < gc) std::swap(gr, gc);  // diagonal tiles: mirror the lower triangle
                        T[r + (size_t)c * S.bs(ii)] = h_A[gr + (size_t)gc * S.N];
                    }
            }
        TTG_CUDA_CHECK(cudaMemcpyAsync(S.A64, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice, s));
        TTG_CUDA_CHECK(cudaStreamSynchronize(s));
    }
    if (h_B) {
        std::vector<double> v((size_t)S.N * nr);
        for (int q = 0; q < nr; ++q)
            for (int r = 0; r < S.N; ++r) v[q + (size_t)r * nr] = h_B[r + (size_t)q * S.N];
        TTG_CUDA_CHECK(cudaMemcpyAsync(S.B, v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice, s));
        TTG_CUDA_CHECK(cudaStreamSynchronize(s));
    }
    return TTG_OK;
}

extern "C" ttg_status ttg_batch_run(ttg_batch* b, void* stream, ttg_batch_report* rep) {
    if (!b) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(b->ctx->device));
    cudaStream_t s = (cudaStream_t)stream;
    if (!s) {
        if (!b->own) TTG_CUDA_CHECK(cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking));
        s = b->own;
    }
    ttg_status st;
    // Another graph (or a worker change) replaced ours in the context: upload
    // again; record the CUDA graph on first use and for a new stream.
    if (ttg_graph_generation(b->ctx) != b->gen && (st = batch_upload(b)) != TTG_OK) return st;
    if (!b->gexec || b->gstream != s || b->gworkers != ttg_workers(b->ctx))
        if ((st = batch_record(b, s)) != TTG_OK) return st;
    TTG_CUDA_CHECK(cudaEventRecord(ttg_event(b->ctx, 0), s));
    TTG_CUDA_CHECK(cudaGraphLaunch(b->gexec, s));
    if (b->gen_recorded_run) ttg_note_launch();  // the executor kernel of the replayed graph
    b->gen_recorded_run = true;
    TTG_CUDA_CHECK(cudaEventRecord(ttg_event(b->ctx, 1), s));
    ttg_mark_launched(b->ctx, s);
    ttg_report r{};
    st = ttg_wait(b->ctx, &r);
    if (rep) {
        rep->run = r;
        rep->tasks = (int64_t)b->g.ops.size();
        rep->flops = b->flops;
    }
    return st;
}

extern "C" ttg_status ttg_batch_get_x(ttg_batch* b, int32_t i, double* h_X) {
    if (!b || !h_X || i < 0 || i >= (int)b->sys.size()) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(b->ctx->device));
    const System& S = b->sys[i];
    const int nr = b->a.nrhs;
    std::vector<double> v((size_t)S.N * nr);
    TTG_CUDA_CHECK(cudaMemcpy(v.data(), S.X, sizeof(double) * v.size(), cudaMemcpyDeviceToHost));
    for (int q = 0; q < nr; ++q)
        for (int r = 0; r < S.N; ++r) h_X[r + (size_t)q * S.N] = v[q + (size_t)r * nr];
    return TTG_OK;
}

extern "C" ttg_status ttg_batch_backward_errors(ttg_batch* b, double* h_err, void* stream) {
    if (!b || !h_err) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(b->ctx->device));
    cudaStream_t s = (cudaStream_t)stream;
    const int n = (int)b->sys.size();
    std::vector<int> Ns(n), tl(n);
    std::vector<int64_t> tb(n), vb(n);
    for (int i = 0; i < n; ++i) {
        Ns[i] = b->sys[i].N;
        tl[i] = b->sys[i].tile;
        tb[i] = b->sys[i].A64 - b->A64;
        vb[i] = b->sys[i].B - b->B;
    }
    int *dN = nullptr, *dT = nullptr;
    int64_t *dTB = nullptr, *dVB = nullptr;
    double* dE = nullptr;
    cudaError_t e = cudaMalloc((void**)&dN, sizeof(int) * n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&dT, sizeof(int) * n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&dTB, sizeof(int64_t) * n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&dVB, sizeof(int64_t) * n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&dE, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dN, Ns.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dT, tl.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dTB, tb.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dVB, vb.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        ttg_note_launch();
        batch_bwd_kernel<<<std::min(n, 8192), 256, 0, s>>>(dN, dT, dTB, dVB, n, b->a.nrhs, b->A64, b->B, b->X, dE);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_err, dE, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    for (void* p : {(void*)dN, (void*)dT, (void*)dTB, (void*)dVB, (void*)dE})
        if (p) cudaFree(p);
    if (e != cudaSuccess) {
        ttg_set_last_cuda_error(e, "batch backward errors", __FILE__, __LINE__);
        return TTG_ECUDA;
    }
    return TTG_OK;
}

extern "C" ttg_status ttg_batch_autotune(ttg_ctx* ctx, const ttg_batch_args* args, const int32_t* tiles, int32_t n_tiles,
                                         const int32_t* workers, int32_t n_workers, int32_t max_sample, int32_t* best_tile,
                                         int32_t* best_workers, double* best_ms_per_system) {
    if (!ctx || !args || !args->sizes || args->n_systems < 1 || !tiles || n_tiles < 1 || !workers || n_workers < 1 ||
        max_sample < 1)
        return TTG_EINVAL;
    // An even sample of the systems (keeps the size mix).
    std::vector<int32_t> sample;
    const int n = args->n_systems;
    const int take = std::min(n, (int)max_sample);
    for (int k = 0; k < take; ++k) sample.push_back(args->sizes[(int64_t)k * n / take]);
    double best = INFINITY;
    int bt = tiles[0], bw = workers[0];
    TTG_CUDA_CHECK(cudaSetDevice(ctx->device));
    ttg_status st = TTG_OK;
    for (int it = 0; it < n_tiles && st == TTG_OK; ++it)
        for (int iw = 0; iw < n_workers && st == TTG_OK; ++iw) {
            if ((st = ttg_set_workers(ctx, workers[iw])) != TTG_OK) break;
            ttg_batch_args a = *args;
            a.sizes = sample.data();
            a.n_systems = (int32_t)sample.size();
            a.tile = tiles[it];
            ttg_batch* b = nullptr;
            if ((st = ttg_batch_create(ctx, &a, &b)) != TTG_OK) break;
            if ((st = ttg_batch_generate(b, nullptr)) == TTG_OK) {
                double ms = 0.0;
                for (int rep = 0; rep < 3 && st == TTG_OK; ++rep) {
                    ttg_batch_report r{};
                    st = ttg_batch_run(b, nullptr, &r);
                    if (rep > 0) ms += r.run.elapsed_ms;
                }
                ms /= 2.0;
                if (st == TTG_OK && ms < best) {
                    best = ms;
                    bt = tiles[it];
                    bw = ttg_workers(ctx);
                }
            }
            ttg_batch_destroy(b);
        }
    if (st != TTG_OK) return st;
    ttg_set_workers(ctx, bw);
    if (best_tile) *best_tile = bt;
    if (best_workers) *best_workers = bw;
    if (best_ms_per_system) *best_ms_per_system = best / (double)sample.size();
    return TTG_OK;
}
