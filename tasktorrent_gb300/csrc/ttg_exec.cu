// ttg_exec.cu — C ABI of the persistent executor (include/ttg.h).
//
// Host side: graph validation and upload, priority levels, queue layout,
// launch/wait and the run report.  Device side: the persistent kernel that
// runs the FP64 tile tasks (tile_f64.cuh) and the mixed-precision tile tasks
// (tile_mixed.cuh) through the executor loop (exec.cuh).
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <vector>

#include "../../include/ttg.h"
#include "exec.cuh"
#include "op_runner.cuh"
#include "tile_f64.cuh"
#include "ttg_internal.h"

namespace ttg {

static_assert(kTeamCounters == kTeamStride, "team counter block size");

// One part of an FP64 tile task on the whole block.  Returns POTRF's info (0 =
// ok).  A POTRF with a team counter block is factored by all its parts.
__device__ int run_op_f64(const ttg_op& op, int part, int parts, double* smem, int* team, int* fin, int* err,
                          long long limit_ns) {
    if (op.kind == TTG_OP_POTRF_L) {
        if (team) return potrf_l_f64_team(op.n, (double*)op.c, op.ldc, smem, TeamCtx{team, limit_ns, err}, nullptr, 0, fin);
        return potrf_l_f64(op.n, (double*)op.c, op.ldc, smem);
    }
    return run_op_plain<double>(op, part, parts, smem);
}

__global__ void __launch_bounds__(kThreads, 1) exec_kernel(ExecParams p) {
    extern __shared__ __align__(128) double smem_f64[];
    executor_loop(p, smem_f64, [&](const ttg_op& op, int part, int parts, double* smem, int* team, int* fin) {
        return run_op_f64(op, part, parts, smem, team, fin, p.err, p.timeout_ns);
    });
}

// Post-run summary: tasks that ran other than once, counters not at zero.
__global__ void summarize_kernel(const int* runs, const int* count, const uint8_t* runnable, int n, int* out) {
    int bad = 0, pending = 0, ran = 0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int r = runs[t];
        ran += r;
        if (runnable[t] ? (r != 1) : (r != 0)) ++bad;
        if (count[t] != 0) ++pending;
    }
    for (int o = 16; o > 0; o >>= 1) {
        bad += __shfl_down_sync(0xffffffffu, bad, o);
        pending += __shfl_down_sync(0xffffffffu, pending, o);
        ran += __shfl_down_sync(0xffffffffu, ran, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out + 0, ran);
        atomicAdd(out + 1, pending);
        atomicAdd(out + 2, bad);
    }
}

// Independent DFMA chains (8 per thread) for the FP64 peak measurement.
__global__ void fp64_peak_kernel(double* out, int iters, double a, double b) {
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

}  // namespace ttg

using namespace ttg;

#define TTG_CUDA_TRY(expr)                                                                          \
    do {                                                                                            \
        cudaError_t _e = (expr);                                                                    \
        if (_e != cudaSuccess) {                                                                    \
            ttg_set_last_cuda_error(_e, #expr, __FILE__, __LINE__);                                 \
            return _e == cudaErrorMemoryAllocation ? TTG_ENOMEM : TTG_ECUDA;                        \
        }                                                                                           \
    } while (0)

static char g_last_cuda[512];

void ttg_set_last_cuda_error(cudaError_t e, const char* expr, const char* file, int line) {
    snprintf(g_last_cuda, sizeof(g_last_cuda), "%s: %s (%s:%d)", cudaGetErrorString(e), expr, file, line);
}

extern "C" const char* ttg_last_cuda_error(void) { return g_last_cuda; }

static std::atomic<long long> g_launches{0};
void ttg_note_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
extern "C" int64_t ttg_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

extern "C" ttg_status ttg_team_item(int32_t P, int32_t idx, int32_t* kind, int32_t* p, int32_t* bi, int32_t* bj) {
    if (P < 1 || idx < 0 || !kind || !p || !bi || !bj) return TTG_EINVAL;
    const ttg::TeamItem t = ttg::team_item(P, idx);
    *kind = t.kind;
    *p = t.p;
    *bi = t.bi;
    *bj = t.bj;
    return TTG_OK;
}

extern "C" const char* ttg_strerror(ttg_status s) {
    switch (s) {
        case TTG_OK: return "ok";
        case TTG_EINVAL: return "invalid argument";
        case TTG_ECUDA: return "CUDA runtime error";
        case TTG_ETIMEOUT: return "executor made no progress within the time limit";
        case TTG_EOVERCOUNT: return "a task received more promises than its indegree";
        case TTG_ENOTPD: return "a diagonal tile is not positive definite";
        case TTG_ENOMEM: return "device allocation failed";
        case TTG_ESTATE: return "call out of order";
        case TTG_EUNDERRUN: return "some tasks never became ready";
        case TTG_ENOCONV: return "iterative refinement did not converge";
        default: return "unknown status";
    }
}

namespace {

template <class T>
ttg_status dev_alloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    TTG_CUDA_TRY(cudaMalloc((void**)p, count * sizeof(T)));
    return TTG_OK;
}

// Grow-only buffer of the device graph (see DevGraph::cap).
template <class T>
ttg_status dev_reserve(DevGraph& g, T** p, size_t count) {
    if (count == 0) count = 1;
    size_t& cap = g.cap[(const void*)p];
    if (*p && cap >= count) return TTG_OK;
    if (*p) cudaFree((void*)*p);
    *p = nullptr;
    cap = 0;
    const size_t want = std::max(count, count + count / 2);
    TTG_CUDA_TRY(cudaMalloc((void**)p, want * sizeof(T)));
    cap = want;
    return TTG_OK;
}

template <class T>
void dev_free(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}

}  // namespace

void ttg_graph_free(ttg_ctx* c) {
    DevGraph& g = c->g;
    dev_free(g.ops);
    dev_free(g.init);
    dev_free(g.count);
    dev_free(g.runs);
    dev_free(g.parts);
    dev_free(g.team_ctr);
    dev_free(g.team_slot);
    g.n_team = 0;
    dev_free(g.part_next);
    dev_free(g.part_done);
    dev_free(g.succ_ptr);
    dev_free(g.succ_idx);
    dev_free(g.level);
    dev_free(g.bind);
    dev_free(g.runnable);
    dev_free(g.qbuf);
    dev_free(g.qinit);
    dev_free(g.q_off);
    dev_free(g.q_head);
    dev_free(g.q_tail);
    dev_free(g.q_tail_init);
    dev_free(g.bq_buf);
    dev_free(g.bq_off);
    dev_free(g.bq_head);
    dev_free(g.bq_tail);
    dev_free(g.trace);
    g = DevGraph();
}

extern "C" ttg_status ttg_create(ttg_ctx** out, const ttg_opts* opts) {
    if (!out) return TTG_EINVAL;
    *out = nullptr;
    ttg_ctx* c = new ttg_ctx();
    c->device = opts ? opts->device : 0;
    c->timeout_s = (opts && opts->timeout_s > 0) ? opts->timeout_s : 10.0;
    c->trace = opts ? opts->trace : 0;
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) {
        ttg_set_last_cuda_error(e, "cudaSetDevice", __FILE__, __LINE__);
        delete c;
        return TTG_ECUDA;
    }
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, c->device);
    if (e != cudaSuccess) {
        ttg_set_last_cuda_error(e, "cudaGetDeviceProperties", __FILE__, __LINE__);
        delete c;
        return TTG_ECUDA;
    }
    c->sms = prop.multiProcessorCount;
    c->workers = (opts && opts->workers > 0) ? opts->workers : c->sms;
    ttg_status st = ttg_ctx_init_device(c);
    if (st != TTG_OK) {
        delete c;
        return st;
    }
    *out = c;
    return TTG_OK;
}

ttg_status ttg_ctx_init_device(ttg_ctx* c) {
    TTG_CUDA_TRY(cudaMalloc((void**)&c->status, sizeof(int) * 8));
    TTG_CUDA_TRY(cudaMallocHost((void**)&c->h_status, sizeof(int) * 8));
    TTG_CUDA_TRY(cudaEventCreate(&c->ev0));
    TTG_CUDA_TRY(cudaEventCreate(&c->ev1));
    const int smem = kPlainSmemDoubles * (int)sizeof(double);
    TTG_CUDA_TRY(cudaFuncSetAttribute(exec_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    // Workers of a bound queue wait for their own block, so every block must
    // be resident: the executor is a cooperative launch and its size is
    // clamped to what the device can hold at once.
    int per_sm = 0;
    TTG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, exec_kernel, kThreads, smem));
    c->max_workers_f64 = std::max(1, per_sm) * c->sms;
    if (c->workers > c->max_workers_f64) c->workers = c->max_workers_f64;
    return ttg_mixed_init(c);
}

extern "C" ttg_status ttg_destroy(ttg_ctx* c) {
    if (!c) return TTG_OK;
    cudaSetDevice(c->device);
    ttg_graph_free(c);
    ttg_mixed_free(c);
    if (c->status) cudaFree(c->status);
    if (c->h_status) cudaFreeHost(c->h_status);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    delete c;
    return TTG_OK;
}

extern "C" int ttg_workers(const ttg_ctx* c) { return c ? c->workers : 0; }

extern "C" ttg_status ttg_set_workers(ttg_ctx* c, int32_t w) {
    if (!c || w < 0) return TTG_EINVAL;
    int maxw = c->max_workers_f64;
    const int mx = ttg_mixed_max_workers(c);
    if (mx > 0) maxw = std::min(maxw, mx);
    const int nw = w == 0 ? maxw : std::min(w, maxw);
    if (nw != c->workers) {
        // The queue layout of an uploaded graph depends on the worker count:
        // the graph must be uploaded again (owners see a new generation).
        c->workers = nw;
        c->uploaded = false;
        c->graph_gen += 1;
    }
    return TTG_OK;
}

extern "C" uint64_t ttg_graph_generation(const ttg_ctx* c) { return c ? c->graph_gen : 0; }

// Blocks that share one task: explicit op.parts, else one per 128×128 output
// block (lower blocks for SYRK) up to 16, TRSM by 128-row slices up to 8;
// POTRF (with team) by n/16 blocks up to 32 for n >= 128; no-op tasks and,
// without team, POTRF are never split.
int ttg_task_parts(const ttg_op& op, bool team) {
    auto cdiv = [](long a, long b) { return (int)((a + b - 1) / b); };
    if (op.kind == TTG_OP_POTRF_L) {
        if (!team || !team_fits(op.n)) return 1;
        if (op.parts > 0) return std::min(op.parts, 64);
        return op.n >= 128 ? std::min(32, op.n / 16) : 1;
    }
    // Tensor-core updates of the mixed path: GEMM kTcBlocksPerPart 128×256
    // output blocks per part, one after the other in the part's block; SYRK
    // (the diagonal tiles, on the factorisation's critical path) one block
    // per part, lower-triangle blocks only.
    if (op.prec == TTG_PREC_MIXED && op.flags >= 2 && (op.kind == TTG_OP_GEMM_NT || op.kind == TTG_OP_SYRK_LN)) {
        const int bm = cdiv(op.m, 128), bn = cdiv(op.n, 256);
        if (op.kind == TTG_OP_GEMM_NT) return std::max(1, cdiv(bm * bn, kTcBlocksPerPart));
        int cnt = 0;
        for (int j = 0; j < bn; ++j)
            for (int i = 0; i < bm; ++i)
                if (i * 128 + 127 >= j * 256) ++cnt;
        return std::max(1, cnt);
    }
    int auto_parts = 1, max_parts = 1;
    switch (op.kind) {
        case TTG_OP_GEMM_NT:
        case TTG_OP_GEMM_NN: {
            // Row-vector products (m <= 16 right-hand-side rows) split their
            // columns by 128 whatever the precision.
            const int e = op.m <= 16 ? 128 : gemm_block_edge(op.m, op.n, op.prec == TTG_PREC_F64);
            max_parts = std::max(1, cdiv(op.m, e) * cdiv(op.n, e));
            auto_parts = std::min(16, max_parts);
            break;
        }
        case TTG_OP_SYRK_LN: {
            const int b = cdiv(op.n, gemm_block_edge(op.n, op.n, op.prec == TTG_PREC_F64));
            max_parts = std::max(1, b * (b + 1) / 2);
            auto_parts = std::min(16, max_parts);
            break;
        }
        case TTG_OP_TRSM_RLTN:
        case TTG_OP_TRSM_RLNN:
            max_parts = std::max(1, cdiv(op.m, 16));
            // Rows per part: 128, or 32 for tiles up to 256 (more SMs on a
            // short critical chain).
            auto_parts = std::min(8, std::max(1, cdiv(op.m, op.n <= 256 && op.prec == TTG_PREC_F64 ? 32 : 128)));
            // The mixed path's FP32 TRSM keeps each part's rows in shared
            // memory: at most 64 rows per part.
            if (op.prec == TTG_PREC_MIXED && op.kind == TTG_OP_TRSM_RLTN) auto_parts = std::min(max_parts, std::max(1, cdiv(op.m, 64)));
            break;
        case TTG_OP_GEADD:
            max_parts = std::max(1, cdiv((long)op.m * op.n, 256));
            auto_parts = std::min(8, std::max(1, cdiv((long)op.m * op.n, 65536)));
            break;
        case TTG_OP_CONVERT:
            // Conversions of whole tiles (batched and serving inputs, refinement
            // vectors): 8192 elements per part, up to 16 parts.
            max_parts = std::max(1, cdiv((long)op.m * op.n, 256));
            auto_parts = std::min(16, std::max(1, cdiv((long)op.m * op.n, 8192)));
            break;
        default:
            return 1;
    }
    if (op.parts > 0) return std::max(1, std::min(op.parts, std::min(64, max_parts)));
    return std::max(1, auto_parts);
}

// Flops per µs per block of a tile update: FP64 DFMA, FP32 FFMA (mixed flags
// 1), or the tensor cores with plain BF16 (2), split BF16 (3: six products)
// and split FP16 (4: three products) operands.
static double mixed_update_rate(const ttg_op& op, bool mixed) {
    if (!mixed) return 7.5e3;
    switch (op.flags) {
        case 2: return 3.0e6;
        case 3: return 5.0e5;
        case 4: return 1.0e6;
        default: return 2.0e5;
    }
}

// Estimated duration (µs) of a task on this executor: its flops over the
// per-block rate of its kernel times the blocks that share it, plus a fixed
// cost for claiming and releasing it.
static double task_cost_us(const ttg_op& op) {
    const double m = op.m, n = op.n, k = op.k;
    const int parts = ttg_task_parts(op, true);
    const bool mixed = op.prec == TTG_PREC_MIXED;
    double flops = 0.0, rate = 1.0, par = parts;  // rate in flops per µs per block
    switch (op.kind) {
        case TTG_OP_POTRF_L:
            flops = n * n * n / 3.0;
            rate = 4.0e3;
            par = std::min(parts, 8) * 0.5 + 0.5;  // team phases are short and synchronised
            break;
        case TTG_OP_TRSM_RLTN:
            flops = m * n * n;
            rate = mixed ? 5.0e4 : 5.0e3;
            break;
        case TTG_OP_SYRK_LN:
            flops = n * n * k;
            rate = mixed_update_rate(op, mixed);
            break;
        case TTG_OP_GEMM_NT:
        case TTG_OP_GEMM_NN:
            flops = 2.0 * m * n * k;
            rate = mixed_update_rate(op, mixed);
            break;
        case TTG_OP_GEADD:
            flops = m * n;
            rate = 5.0e4;
            break;
        case TTG_OP_SPIN:
            return 2.0 + op.alpha * 1e6;
        default:
            break;
    }
    return 2.0 + flops / (rate * std::max(1.0, par));
}

extern "C" ttg_status ttg_critical_path_priority(const ttg_graph_desc* gd, double* out) {
    if (!gd || !out || gd->n_tasks < 0 || (gd->n_tasks > 0 && (!gd->ops || !gd->succ_ptr))) return TTG_EINVAL;
    const int n = gd->n_tasks;
    std::vector<int> indeg(n, 0);
    for (int t = 0; t < n; ++t)
        for (int64_t e = gd->succ_ptr[t]; e < gd->succ_ptr[t + 1]; ++e) {
            const int s = gd->succ_idx[e];
            if (s < 0 || s >= n) return TTG_EINVAL;
            ++indeg[s];
        }
    // Kahn's order, then the longest remaining path in reverse order.
    std::vector<int> order;
    order.reserve(n);
    for (int t = 0; t < n; ++t)
        if (indeg[t] == 0) order.push_back(t);
    for (size_t h = 0; h < order.size(); ++h) {
        const int t = order[h];
        for (int64_t e = gd->succ_ptr[t]; e < gd->succ_ptr[t + 1]; ++e)
            if (--indeg[gd->succ_idx[e]] == 0) order.push_back(gd->succ_idx[e]);
    }
    if ((int)order.size() != n) return TTG_EINVAL;  // a cycle
    for (int h = n - 1; h >= 0; --h) {
        const int t = order[h];
        double best = 0.0;
        for (int64_t e = gd->succ_ptr[t]; e < gd->succ_ptr[t + 1]; ++e) best = std::max(best, out[gd->succ_idx[e]]);
        out[t] = task_cost_us(gd->ops[t]) + best;
    }
    return TTG_OK;
}

// Priority levels: distinct priorities ranked from high to low; more than
// kMaxLevels distinct values are split into kMaxLevels equal-count groups.
static void assign_levels(int n, const double* prio, const std::vector<uint8_t>& runnable, std::vector<uint8_t>& level,
                          int* n_levels) {
    level.assign(n, 0);
    if (!prio) {
        *n_levels = 1;
        return;
    }
    std::vector<double> vals;
    vals.reserve(n);
    for (int t = 0; t < n; ++t)
        if (runnable[t]) vals.push_back(prio[t]);
    std::sort(vals.begin(), vals.end(), std::greater<double>());
    std::vector<double> distinct;
    for (double v : vals)
        if (distinct.empty() || distinct.back() != v) distinct.push_back(v);
    if (distinct.empty()) {
        *n_levels = 1;
        return;
    }
    if ((int)distinct.size() <= kMaxLevels) {
        std::map<double, int> rank;
        for (size_t r = 0; r < distinct.size(); ++r) rank[distinct[r]] = (int)r;
        for (int t = 0; t < n; ++t) level[t] = (uint8_t)(runnable[t] ? rank[prio[t]] : 0);
        *n_levels = (int)distinct.size();
        return;
    }
    // Equal-width split of the range of the runnable priorities: tasks whose
    // priorities differ by more than a 128th of the range never share a
    // level, wherever they sit in the order (an equal-count split leaves the
    // few tasks of a factorisation's last steps in one first-in-first-out
    // level, and their chain waits behind its own updates).
    const double hi = distinct.front(), width = (distinct.front() - distinct.back()) / kMaxLevels;
    for (int t = 0; t < n; ++t) {
        if (!runnable[t]) continue;
        const double q = (hi - prio[t]) / width;
        level[t] = (uint8_t)(q >= kMaxLevels - 1 ? kMaxLevels - 1 : (q > 0 ? (int)q : 0));
    }
    *n_levels = kMaxLevels;
}

extern "C" ttg_status ttg_graph_upload(ttg_ctx* c, const ttg_graph_desc* gd) {
    if (!c || !gd || gd->n_tasks < 0 || (gd->n_tasks > 0 && (!gd->ops || !gd->init_count || !gd->succ_ptr)))
        return TTG_EINVAL;
    TTG_CUDA_TRY(cudaSetDevice(c->device));
    // The buffers are reused below: let a run still in flight finish first.
    if (c->launched && c->stream) TTG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->uploaded = false;
    c->launched = false;
    const int n = gd->n_tasks;
    const int64_t n_edges = n > 0 ? gd->succ_ptr[n] : 0;
    if (n_edges > 0 && !gd->succ_idx) return TTG_EINVAL;
    for (int t = 0; t < n; ++t) {
        if (gd->init_count[t] < 0 || gd->succ_ptr[t] > gd->succ_ptr[t + 1]) return TTG_EINVAL;
        const int k = gd->ops[t].kind;
        if (k < TTG_OP_NOP || k > TTG_OP_SPIN) return TTG_EINVAL;
        if (k == TTG_OP_SPIN && !(gd->ops[t].alpha >= 0.0 && gd->ops[t].alpha <= 1.0)) return TTG_EINVAL;
        if (gd->ops[t].prec != TTG_PREC_F64 && gd->ops[t].prec != TTG_PREC_MIXED) return TTG_EINVAL;
    }
    if (n > 0 && gd->succ_ptr[0] != 0) return TTG_EINVAL;
    for (int64_t e = 0; e < n_edges; ++e)
        if (gd->succ_idx[e] < 0 || gd->succ_idx[e] >= n) return TTG_EINVAL;

    // Host simulation of the counters: which tasks will reach zero, and
    // whether any counter would be decremented below zero.
    std::vector<int> cnt(gd->init_count, gd->init_count + n);
    std::vector<uint8_t> runnable(n, 0);
    std::vector<int> stack;
    for (int t = 0; t < n; ++t)
        if (cnt[t] == 0) {
            runnable[t] = 1;
            stack.push_back(t);
        }
    bool over = false;
    while (!stack.empty()) {
        const int t = stack.back();
        stack.pop_back();
        for (int64_t e = gd->succ_ptr[t]; e < gd->succ_ptr[t + 1]; ++e) {
            const int s = gd->succ_idx[e];
            if (--cnt[s] == 0) {
                runnable[s] = 1;
                stack.push_back(s);
            } else if (cnt[s] < 0) {
                over = true;
            }
        }
    }
    int n_runnable = 0;
    for (int t = 0; t < n; ++t) n_runnable += runnable[t];
    c->pending_host = n - n_runnable;
    c->g_mixed = false;
    for (int t = 0; t < n; ++t)
        if (gd->ops[t].prec == TTG_PREC_MIXED) c->g_mixed = true;
    c->overcount_host = over;

    std::vector<uint8_t> level;
    int n_levels = 1;
    assign_levels(n, gd->priority, runnable, level, &n_levels);
    std::vector<int> parts(n, 1);
    std::vector<int> team_slot(n, -1);
    int n_team = 0;
    for (int t = 0; t < n; ++t) {
        parts[t] = ttg_task_parts(gd->ops[t], true);
        // Every POTRF that fits runs the team code, a team of one included, so
        // the factor does not depend on how many blocks share it.
        if (gd->ops[t].kind == TTG_OP_POTRF_L && team_fits(gd->ops[t].n))
            team_slot[t] = n_team++;
    }

    // Queue layout: level queues sized by runnable unbound tasks per level,
    // bound queues by runnable tasks bound to each worker.
    const int W = c->workers;
    std::vector<int> bind(n, -1);
    if (gd->bind)
        for (int t = 0; t < n; ++t) bind[t] = gd->bind[t] < 0 ? -1 : gd->bind[t];
    std::vector<int> qcount(kMaxLevels, 0), bqcount(W, 0);
    for (int t = 0; t < n; ++t) {
        if (!runnable[t]) continue;
        if (bind[t] >= 0) bqcount[bind[t] % W] += parts[t];  // one slot per part
        else qcount[level[t]] += parts[t];
    }
    std::vector<int> q_off(kMaxLevels + 1, 0), bq_off(W + 1, 0);
    for (int l = 0; l < kMaxLevels; ++l) q_off[l + 1] = q_off[l] + qcount[l];
    for (int w = 0; w < W; ++w) bq_off[w + 1] = bq_off[w] + bqcount[w];
    bool has_bound = bq_off[W] > 0;
    // Initial queue images: initially-ready tasks in index order.
    std::vector<int> qinit(std::max(1, q_off[kMaxLevels]), -1), bqinit(std::max(1, bq_off[W]), -1);
    std::vector<int> tail0(kMaxLevels * 32, 0), btail0(W, 0);
    for (int t = 0; t < n; ++t) {
        if (gd->init_count[t] != 0) continue;
        if (bind[t] >= 0) {
            const int w = bind[t] % W;
            for (int q = 0; q < parts[t]; ++q) bqinit[bq_off[w] + btail0[w]++] = t;
        } else {
            const int l = level[t];
            for (int q = 0; q < parts[t]; ++q) qinit[q_off[l] + tail0[l * 32]++] = t;
        }
    }
    // Available slots of each level at launch: all the initial ones.
    for (int l = 0; l < kMaxLevels; ++l) tail0[l * 32 + 1] = tail0[l * 32];

    DevGraph& g = c->g;
    g.n_tasks = n;
    g.n_runnable = n_runnable;
    g.n_levels = n_levels;
    g.has_bound = has_bound;
    g.q_total = q_off[kMaxLevels];
    g.bq_total = bq_off[W];
    ttg_status st;
#define ALLOC(ptr, cnt)                                    \
    if ((st = dev_reserve(g, &g.ptr, (cnt))) != TTG_OK) {  \
        ttg_graph_free(c);                                 \
        return st;                                         \
    }
    ALLOC(ops, n);
    ALLOC(init, n);
    ALLOC(count, n);
    ALLOC(runs, n);
    ALLOC(parts, n);
    ALLOC(part_next, n);
    ALLOC(part_done, n);
    ALLOC(succ_ptr, n + 1);
    ALLOC(succ_idx, n_edges);
    ALLOC(level, n);
    ALLOC(bind, n);
    ALLOC(runnable, n);
    ALLOC(qbuf, qinit.size());
    ALLOC(qinit, qinit.size());
    ALLOC(q_off, kMaxLevels + 1);
    ALLOC(q_head, kMaxLevels * 32);
    ALLOC(q_tail, kMaxLevels * 32);
    ALLOC(q_tail_init, kMaxLevels * 32);
    ALLOC(bq_buf, bqinit.size() * 2);  // second half: initial image
    ALLOC(bq_off, W + 1);
    ALLOC(bq_head, W * 2);             // head + initial tail
    ALLOC(bq_tail, W);
    if (c->trace) ALLOC(trace, kTraceWords * (size_t)std::max(1, n));
    ALLOC(team_slot, n);
    if (n_team) ALLOC(team_ctr, (size_t)n_team * kTeamStride);
    g.n_team = n_team;
#undef ALLOC
    TTG_CUDA_TRY(cudaMemcpy(g.ops, gd->ops, sizeof(ttg_op) * n, cudaMemcpyHostToDevice));
    TTG_CUDA_TRY(cudaMemcpy(g.init, gd->init_count, sizeof(int) * n, cudaMemcpyHostToDevice));
    TTG_CUDA_TRY(cudaMemcpy(g.succ_ptr, gd->succ_ptr, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice));
    if (n_edges) TTG_CUDA_TRY(cudaMemcpy(g.succ_idx, gd->succ_idx, sizeof(int32_t) * n_edges, cudaMemcpyHostToDevice));
    TTG_CUDA_TRY(cudaMemcpy(g.level, level.data(), n, cudaMemcpyHostToDevice));
    TTG_CUDA_TRY(cudaMemcpy(g.parts, parts.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    TTG_CUDA_TRY(cudaMemcpy(g.team_slot, team_slot.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    TTG_CUDA_TRY(cudaMemcpy(g.bind, bind.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    TTG_CUDA_TRY(cudaMemcpy(g.runnable, runnable.data(), n, cudaMemcpyHostToDevice));
    TTG_CUDA_TRY(cudaMemcpy(g.qinit, qinit.data(), sizeof(int) * qinit.size(), cudaMemcpyHostToDevice));
    TTG_CUDA_TRY(cudaMemcpy(g.q_off, q_off.data(), sizeof(int) * (kMaxLevels + 1), cudaMemcpyHostToDevice));
    TTG_CUDA_TRY(cudaMemcpy(g.q_tail_init, tail0.data(), sizeof(int) * kMaxLevels * 32, cudaMemcpyHostToDevice));
    TTG_CUDA_TRY(cudaMemcpy(g.bq_buf + bqinit.size(), bqinit.data(), sizeof(int) * bqinit.size(), cudaMemcpyHostToDevice));
    TTG_CUDA_TRY(cudaMemcpy(g.bq_off, bq_off.data(), sizeof(int) * (W + 1), cudaMemcpyHostToDevice));
    TTG_CUDA_TRY(cudaMemcpy(g.bq_head + W, btail0.data(), sizeof(int) * W, cudaMemcpyHostToDevice));
    g.bq_image = (int)bqinit.size();
    c->uploaded = true;
    c->graph_gen += 1;
    c->launched = false;
    return TTG_OK;
}

ttg_status ttg_reset_state(ttg_ctx* c, cudaStream_t s) {
    DevGraph& g = c->g;
    const int n = g.n_tasks, W = c->workers;
    TTG_CUDA_TRY(cudaMemcpyAsync(g.count, g.init, sizeof(int) * std::max(1, n), cudaMemcpyDeviceToDevice, s));
    TTG_CUDA_TRY(cudaMemsetAsync(g.runs, 0, sizeof(int) * std::max(1, n), s));
    TTG_CUDA_TRY(cudaMemsetAsync(g.part_next, 0, sizeof(int) * std::max(1, n), s));
    TTG_CUDA_TRY(cudaMemsetAsync(g.part_done, 0, sizeof(int) * std::max(1, n), s));
    TTG_CUDA_TRY(cudaMemcpyAsync(g.qbuf, g.qinit, sizeof(int) * std::max(1, g.q_total), cudaMemcpyDeviceToDevice, s));
    TTG_CUDA_TRY(cudaMemsetAsync(g.q_head, 0, sizeof(int) * kMaxLevels * 32, s));
    TTG_CUDA_TRY(cudaMemcpyAsync(g.q_tail, g.q_tail_init, sizeof(int) * kMaxLevels * 32, cudaMemcpyDeviceToDevice, s));
    TTG_CUDA_TRY(cudaMemcpyAsync(g.bq_buf, g.bq_buf + g.bq_image, sizeof(int) * g.bq_image, cudaMemcpyDeviceToDevice, s));
    TTG_CUDA_TRY(cudaMemsetAsync(g.bq_head, 0, sizeof(int) * W, s));
    TTG_CUDA_TRY(cudaMemcpyAsync(g.bq_tail, g.bq_head + W, sizeof(int) * W, cudaMemcpyDeviceToDevice, s));
    TTG_CUDA_TRY(cudaMemsetAsync(c->status, 0, sizeof(int) * 8, s));
    if (g.trace) TTG_CUDA_TRY(cudaMemsetAsync(g.trace, 0, sizeof(long long) * kTraceWords * std::max(1, n), s));
    if (g.n_team) TTG_CUDA_TRY(cudaMemsetAsync(g.team_ctr, 0, sizeof(int) * (size_t)g.n_team * kTeamStride, s));
    return TTG_OK;
}

static ExecParams ttg_make_params(ttg_ctx* c) {
    DevGraph& g = c->g;
    ExecParams p;
    p.ops = g.ops;
    p.n_tasks = g.n_tasks;
    p.n_runnable = g.n_runnable;
    p.count = g.count;
    p.runs = g.runs;
    p.parts = g.parts;
    p.part_next = g.part_next;
    p.part_done = g.part_done;
    p.succ_ptr = g.succ_ptr;
    p.succ_idx = g.succ_idx;
    p.level = g.level;
    p.bind = g.bind;
    p.n_levels = g.n_levels;
    p.n_workers = c->workers;
    p.qbuf = g.qbuf;
    p.q_off = g.q_off;
    p.q_head = g.q_head;
    p.q_tail = g.q_tail;
    p.bq_buf = g.bq_buf;
    p.bq_off = g.bq_off;
    p.bq_head = g.bq_head;
    p.bq_tail = g.bq_tail;
    p.has_bound = g.has_bound;
    p.done = c->status + 0;
    p.err = c->status + 1;
    p.err_task = c->status + 2;
    p.err_info = c->status + 3;
    p.trace = (long long*)g.trace;
    p.timeout_ns = (long long)(c->timeout_s * 1e9);
    p.team_ctr = g.team_ctr;
    p.team_slot = g.team_slot;
    p.pub = nullptr;  // a closed graph
    p.roots = nullptr;
    p.admit = nullptr;
    return p;
}

// Enqueue a 32-bit store of v at addr on stream s, ordered after the
// stream's earlier work (copies included): cuStreamWriteValue32 of the
// driver API, which needs no SM (the persistent executor holds them all).
ttg_status ttg_stream_write_u32(cudaStream_t s, uint32_t* addr, uint32_t v) {
    typedef CUresult (*write_fn)(CUstream, CUdeviceptr, cuuint32_t, unsigned int);
    static write_fn fn = nullptr;
    if (!fn) {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuStreamWriteValue32", &f, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || !f || q != cudaDriverEntryPointSuccess) {
            ttg_set_last_cuda_error(e, "cudaGetDriverEntryPointByVersion(cuStreamWriteValue32)", __FILE__, __LINE__);
            return TTG_ECUDA;
        }
        fn = (write_fn)f;
    }
    if (fn((CUstream)s, (CUdeviceptr)addr, v, 0) != CUDA_SUCCESS) {
        ttg_set_last_cuda_error(cudaErrorInvalidValue, "cuStreamWriteValue32", __FILE__, __LINE__);
        return TTG_ECUDA;
    }
    return TTG_OK;
}

extern "C" ttg_status ttg_launch(ttg_ctx* c, void* stream) {
    if (!c) return TTG_EINVAL;
    if (!c->uploaded) return TTG_ESTATE;
    TTG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = (cudaStream_t)stream;
    c->stream = s;
    ttg_status st = ttg_reset_state(c, s);
    if (st != TTG_OK) return st;
    TTG_CUDA_TRY(cudaEventRecord(c->ev0, s));
    if (c->g.n_runnable > 0) {
        ExecParams p = ttg_make_params(c);
        st = ttg_launch_executor(c, p, s);
        if (st != TTG_OK) return st;
    }
    TTG_CUDA_TRY(cudaEventRecord(c->ev1, s));
    c->launched = true;
    return TTG_OK;
}

cudaError_t ttg_launch_cooperative(const void* fn, int grid, int block, void** args, size_t smem, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelExC(&cfg, fn, args);
}

ttg_status ttg_launch_executor(ttg_ctx* c, const ExecParams& p, cudaStream_t s) {
    if (c->g_mixed) return ttg_launch_mixed(c, p, s);
    const int smem = kPlainSmemDoubles * (int)sizeof(double);
    void* args[] = {(void*)&p};
    ttg_note_launch();
    TTG_CUDA_TRY(ttg_launch_executor_kernel(c, (const void*)exec_kernel, args, smem, s));
    return TTG_OK;
}

// The executor kernel needs every block resident only when a task is bound
// to a block (its bound queue waits for that block); without bound tasks any
// resident subset makes progress, and a context may launch it as a plain
// kernel so that it shares the GPU with another context's executor.
cudaError_t ttg_launch_executor_kernel(ttg_ctx* c, const void* fn, void** args, size_t smem, cudaStream_t s) {
    if (c->coop || c->g.has_bound) return ttg_launch_cooperative(fn, c->workers, kThreads, args, smem, s);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(c->workers);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    return cudaLaunchKernelExC(&cfg, fn, args);
}

ttg_status ttg_enqueue_run(ttg_ctx* c, cudaStream_t s) {
    if (!c->uploaded) return TTG_ESTATE;
    ttg_status st = ttg_reset_state(c, s);
    if (st != TTG_OK) return st;
    if (c->g.n_runnable > 0) {
        ExecParams p = ttg_make_params(c);
        st = ttg_launch_executor(c, p, s);
    }
    return st;
}

ttg_status ttg_mark_launched(ttg_ctx* c, cudaStream_t s) {
    c->stream = s;
    c->launched = true;
    return TTG_OK;
}

cudaEvent_t ttg_event(ttg_ctx* c, int which) { return which ? c->ev1 : c->ev0; }

extern "C" ttg_status ttg_wait(ttg_ctx* c, ttg_report* rep) {
    if (!c) return TTG_EINVAL;
    if (!c->launched) return TTG_ESTATE;
    TTG_CUDA_TRY(cudaSetDevice(c->device));
    DevGraph& g = c->g;
    // status[4..6] <- ran, pending, bad
    ttg_note_launch();
    summarize_kernel<<<std::max(1, std::min(256, (g.n_tasks + 255) / 256)), 256, 0, c->stream>>>(
        g.runs, g.count, g.runnable, g.n_tasks, c->status + 4);
    TTG_CUDA_TRY(cudaGetLastError());
    TTG_CUDA_TRY(cudaMemcpyAsync(c->h_status, c->status, sizeof(int) * 8, cudaMemcpyDeviceToHost, c->stream));
    TTG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->launched = false;
    const int* h = c->h_status;
    ttg_status st = h[1];
    if (st == TTG_OK && c->overcount_host) st = TTG_EOVERCOUNT;
    if (st == TTG_OK && c->pending_host > 0) st = TTG_EUNDERRUN;
    if (rep) {
        rep->tasks_total = g.n_tasks;
        rep->tasks_run = h[4];
        rep->tasks_pending = h[5];
        rep->bad_runs = h[6];
        rep->status = st;
        rep->error_task = h[1] ? h[2] : -1;
        rep->info = h[3];
        rep->workers = c->workers;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        rep->elapsed_ms = ms;
    }
    c->last_status = st;
    return st;
}

extern "C" ttg_status ttg_run(ttg_ctx* c, void* stream, ttg_report* rep) {
    ttg_status st = ttg_launch(c, stream);
    if (st != TTG_OK) return st;
    return ttg_wait(c, rep);
}

extern "C" ttg_status ttg_task_record(ttg_ctx* c, int32_t* h_runs, int32_t* h_final_count) {
    if (!c || !c->uploaded) return TTG_ESTATE;
    TTG_CUDA_TRY(cudaSetDevice(c->device));
    const int n = c->g.n_tasks;
    if (h_runs) TTG_CUDA_TRY(cudaMemcpy(h_runs, c->g.runs, sizeof(int) * n, cudaMemcpyDeviceToHost));
    if (h_final_count) TTG_CUDA_TRY(cudaMemcpy(h_final_count, c->g.count, sizeof(int) * n, cudaMemcpyDeviceToHost));
    return TTG_OK;
}

static ttg_status read_trace(ttg_ctx* c, std::vector<long long>& tr, long long* t0) {
    if (!c || !c->uploaded || !c->g.trace) return TTG_ESTATE;
    TTG_CUDA_TRY(cudaSetDevice(c->device));
    const int n = c->g.n_tasks;
    tr.resize(kTraceWords * (size_t)n);
    TTG_CUDA_TRY(cudaMemcpy(tr.data(), c->g.trace, sizeof(long long) * kTraceWords * n, cudaMemcpyDeviceToHost));
    bool any = false;
    *t0 = 0;
    for (int t = 0; t < n; ++t)
        if (tr[kTraceWords * t] > 0 && (!any || tr[kTraceWords * t] < *t0)) {
            *t0 = tr[kTraceWords * t];
            any = true;
        }
    return TTG_OK;
}

extern "C" ttg_status ttg_trace(ttg_ctx* c, int64_t* h_start, int64_t* h_end, int32_t* h_worker) {
    std::vector<long long> tr;
    long long t0;
    ttg_status st = read_trace(c, tr, &t0);
    if (st != TTG_OK) return st;
    const int n = c->g.n_tasks;
    for (int t = 0; t < n; ++t) {
        const long long* w = tr.data() + kTraceWords * (size_t)t;
        const bool ran = w[0] > 0;
        if (h_start) h_start[t] = ran ? w[0] - t0 : -1;
        if (h_end) h_end[t] = ran ? w[1] - t0 : -1;
        if (h_worker) h_worker[t] = ran ? (int32_t)w[2] : -1;
    }
    return TTG_OK;
}

extern "C" ttg_status ttg_trace_busy(ttg_ctx* c, int64_t* h_busy_ns) {
    std::vector<long long> tr;
    long long t0;
    ttg_status st = read_trace(c, tr, &t0);
    if (st != TTG_OK) return st;
    for (int t = 0; t < c->g.n_tasks; ++t) h_busy_ns[t] = tr[kTraceWords * (size_t)t + 3];
    return TTG_OK;
}

extern "C" ttg_status ttg_measure_fp64_peak(ttg_ctx* c, double ms, double* tflops) {
    if (!c || !tflops || ms <= 0) return TTG_EINVAL;
    TTG_CUDA_TRY(cudaSetDevice(c->device));
    const int blocks = c->sms * 2, threads = 256;
    double* out = nullptr;
    TTG_CUDA_TRY(cudaMalloc((void**)&out, sizeof(double) * blocks * threads));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // Calibrate the iteration count on a short run, then time the long one.
    int iters = 2000;
    float t = 0.f;
    for (int pass = 0; pass < 2; ++pass) {
        ttg_note_launch();
        fp64_peak_kernel<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
        cudaEventRecord(e0);
        ttg_note_launch();
        fp64_peak_kernel<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&t, e0, e1);
        if (pass == 0) iters = (int)std::max(1000.0, std::min(2e8, iters * ms / std::max(1e-3, (double)t)));
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) {
        ttg_set_last_cuda_error(err, "fp64_peak_kernel", __FILE__, __LINE__);
        return TTG_ECUDA;
    }
    *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (t * 1e-3) / 1e12;
    return TTG_OK;
}

extern "C" int64_t ttg_tile_layout(const int32_t* bs, int32_t nb, int64_t* off) {
    int64_t o = 0;
    for (int j = 0; j < nb; ++j)
        for (int i = j; i < nb; ++i) {
            if (off) off[i + (int64_t)j * nb] = o;
            o += (int64_t)bs[i] * bs[j];
        }
    return o;
}
