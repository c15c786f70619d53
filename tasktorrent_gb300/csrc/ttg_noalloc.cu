// ttg_noalloc.cu — a variant of the persistent executor that allocates no
// device memory (ttg_run_graph_noalloc in include/ttg.h).
//
// Why it exists: some callers cannot call cudaMalloc.  A serving process
// whose memory pool owns all free HBM would see an extra allocation fail or
// fragment the pool; a caller embedded in another framework's operator may be
// forbidden to allocate outside that framework's allocator; and on a busy
// device cudaMalloc/cudaFree can synchronise and stall other streams.  The
// regular path (ttg_graph_upload) allocates the graph, counters and queues
// with cudaMalloc; this one places all of that scratch in one file-scope
// device array of fixed size, reserved by every GPU that loads the library
// until the process exits.
//
// Limits (rejected with TTG_EINVAL, nothing is written): at most
// TTG_NOALLOC_MAX_TASKS tasks, TTG_NOALLOC_MAX_EDGES successor entries,
// TTG_NOALLOC_MAX_QUEUE queue entries (the parts of all runnable tasks) and
// TTG_NOALLOC_MAX_WORKERS workers.
//
// Sharing: every call uses the same array, which keeps the previous call's
// contents; each call rewrites everything the kernel reads (counters, queues,
// status words) before launching.  Calls that overlap on the GPU would race
// on that array; the entry point therefore holds a process-wide lock for its
// whole duration and waits for its stream before returning.
//
// Set-up: the first call on a device looks up the array's device address
// (cudaGetSymbolAddress, with that device current) and the executor's
// occupancy; later calls reuse both.  Make the first call on each device
// before any stream capture begins.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "../../include/ttg.h"
#include "exec.cuh"
#include "tile_f64.cuh"
#include "ttg_internal.h"

namespace {

constexpr size_t kScratchBytes = TTG_NOALLOC_SCRATCH_BYTES;

// The scratch of every no-alloc run on this device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Offsets (bytes) of the arrays inside the scratch; each is 256-aligned.
constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t kT = TTG_NOALLOC_MAX_TASKS, kE = TTG_NOALLOC_MAX_EDGES, kQ = TTG_NOALLOC_MAX_QUEUE,
                 kW = TTG_NOALLOC_MAX_WORKERS;
constexpr size_t oOps = 0;
constexpr size_t oCount = align256(oOps + kT * sizeof(ttg_op));
constexpr size_t oRuns = align256(oCount + kT * 4);
constexpr size_t oParts = align256(oRuns + kT * 4);
constexpr size_t oPartNext = align256(oParts + kT * 4);
constexpr size_t oPartDone = align256(oPartNext + kT * 4);
constexpr size_t oBind = align256(oPartDone + kT * 4);
constexpr size_t oLevel = align256(oBind + kT * 4);
constexpr size_t oRunnable = align256(oLevel + kT);
constexpr size_t oSuccPtr = align256(oRunnable + kT);
constexpr size_t oSuccIdx = align256(oSuccPtr + (kT + 1) * 8);
constexpr size_t oQbuf = align256(oSuccIdx + kE * 4);          // level queues, then bound queues
constexpr size_t oQoff = align256(oQbuf + kQ * 4);
constexpr size_t oQhead = align256(oQoff + (ttg::kMaxLevels + 1) * 4);
constexpr size_t oQtail = align256(oQhead + ttg::kMaxLevels * 32 * 4);
constexpr size_t oBqoff = align256(oQtail + ttg::kMaxLevels * 32 * 4);
constexpr size_t oBqhead = align256(oBqoff + (kW + 1) * 4);
constexpr size_t oBqtail = align256(oBqhead + kW * 4);
// Status of a run: the executor's words, the first start / last end of the
// blocks (GPU global timer, ns) and the run report counts.
struct RunStatus {
    int done, err, err_task, err_info;
    int pad[12];
    unsigned long long start, end;
    unsigned long long ran, pending, bad;
};
constexpr size_t oStatus = align256(oBqtail + kW * 4);
constexpr size_t kUsed = align256(oStatus + sizeof(RunStatus));
static_assert(kUsed <= kScratchBytes, "no-alloc scratch layout exceeds the array");

__device__ int run_op_f64_noalloc(const ttg_op& op, int part, int parts, double* smem) {
    using namespace ttg;
    switch (op.kind) {
        case TTG_OP_POTRF_L:
            return potrf_l_f64(op.n, (double*)op.c, op.ldc, smem);
        case TTG_OP_TRSM_RLTN:
            trsm_rltn_f64(op.m, op.n, op.alpha, (const double*)op.a, op.lda, (double*)op.c, op.ldc, smem, part, parts);
            return 0;
        case TTG_OP_SYRK_LN:
            gemm_tile_auto<double, false, true>(op.n, op.n, op.k, op.alpha, (const double*)op.a, op.lda, (const double*)op.a, op.lda,
                                  op.beta, (double*)op.c, op.ldc, smem, part, parts);
            return 0;
        case TTG_OP_GEMM_NT:
            gemm_tile_auto<double, false, false>(op.m, op.n, op.k, op.alpha, (const double*)op.a, op.lda, (const double*)op.b, op.ldb,
                                   op.beta, (double*)op.c, op.ldc, smem, part, parts);
            return 0;
        case TTG_OP_GEMM_NN:
            gemm_tile_auto<double, true, false>(op.m, op.n, op.k, op.alpha, (const double*)op.a, op.lda, (const double*)op.b, op.ldb,
                                  op.beta, (double*)op.c, op.ldc, smem, part, parts);
            return 0;
        case TTG_OP_GEADD:
            geadd_f64(op.m, op.n, op.alpha, (const double*)op.a, op.lda, op.beta, (double*)op.c, op.ldc, part, parts);
            return 0;
        default:
            return 0;
    }
}

// The executor over scratch-resident state; also stamps the run's first
// start and last end (GPU global timer) into the status words.
__global__ void __launch_bounds__(ttg::kThreads, 1) exec_kernel_noalloc(ttg::ExecParams p, RunStatus* st) {
    extern __shared__ __align__(128) double smem_na[];
    if (threadIdx.x == 0) atomicMin(&st->start, (unsigned long long)ttg::globaltimer());
    ttg::executor_loop(p, smem_na, [](const ttg_op& op, int part, int parts, double* smem, int*, int*) {
        return run_op_f64_noalloc(op, part, parts, smem);
    });
    if (threadIdx.x == 0) atomicMax(&st->end, (unsigned long long)ttg::globaltimer());
}

// Run report: runs, runs other than once, counters not at zero.
__global__ void summarize_noalloc(const int* runs, const int* count, const uint8_t* runnable, int n, RunStatus* st) {
    int bad = 0, pending = 0, ran = 0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        ran += runs[t];
        if (runnable[t] ? (runs[t] != 1) : (runs[t] != 0)) ++bad;
        if (count[t] != 0) ++pending;
    }
    atomicAdd(&st->ran, (unsigned long long)ran);
    atomicAdd(&st->pending, (unsigned long long)pending);
    atomicAdd(&st->bad, (unsigned long long)bad);
}

struct DeviceSetup {
    bool ready = false;
    unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch
    int sms = 0;
    int max_workers = 0;
};

std::mutex g_lock;
DeviceSetup g_setup[64];

// Host staging of everything copied into the scratch (static: no heap).
ttg_op h_ops[kT];
int h_count[kT], h_parts[kT], h_bind[kT], h_sim[kT], h_stack[kT];
uint8_t h_level[kT], h_runnable[kT];
int h_qbuf[kQ], h_qoff[ttg::kMaxLevels + 1], h_qtail[ttg::kMaxLevels * 32], h_bqoff[kW + 1], h_bqtail[kW];
int h_qfill[ttg::kMaxLevels], h_bqfill[kW];
RunStatus h_status;
double h_sorted[kT];
double h_cut[ttg::kMaxLevels];

ttg_status setup_device(int device, DeviceSetup& d) {
    if (d.ready) return TTG_OK;
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) {
        ttg_set_last_cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
        return TTG_ECUDA;
    }
    int sms = 0, per_sm = 0;
    TTG_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    TTG_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, exec_kernel_noalloc, ttg::kThreads,
                                                                 ttg::kF64SmemDoubles * (int)sizeof(double)));
    d.scratch = (unsigned char*)ptr;
    d.sms = sms;
    d.max_workers = std::max(1, per_sm) * sms;
    d.ready = true;
    return TTG_OK;
}

// Priority levels without heap use: rank of each runnable task's priority
// among the distinct values (descending) if there are at most kMaxLevels
// (128) of them, else kMaxLevels equal-count groups of the sorted values.
void levels_static(int n, const double* prio, int* n_levels) {
    for (int t = 0; t < n; ++t) h_level[t] = 0;
    *n_levels = 1;
    if (!prio) return;
    int m = 0;
    for (int t = 0; t < n; ++t)
        if (h_runnable[t]) h_sorted[m++] = prio[t];
    if (m == 0) return;
    auto desc = [](double a, double b) { return a > b; };
    std::sort(h_sorted, h_sorted + m, desc);
    int distinct = 1;
    for (int i = 1; i < m; ++i) distinct += h_sorted[i] != h_sorted[i - 1];
    if (distinct > ttg::kMaxLevels) {
        // Group cuts from the sorted values: here m >= distinct > kMaxLevels,
        // so every index (l+1)·m/kMaxLevels − 1 lies in [0, m).
        for (int l = 0; l < ttg::kMaxLevels; ++l)
            h_cut[l] = h_sorted[std::max(0, std::min(m - 1, (int)((long)(l + 1) * m / ttg::kMaxLevels) - 1))];
    } else {
        std::unique(h_sorted, h_sorted + m);
    }
    for (int t = 0; t < n; ++t) {
        if (!h_runnable[t]) continue;
        int l = 0;
        if (distinct <= ttg::kMaxLevels) {
            l = (int)(std::lower_bound(h_sorted, h_sorted + distinct, prio[t], desc) - h_sorted);
        } else {
            while (l < ttg::kMaxLevels - 1 && prio[t] < h_cut[l]) ++l;
        }
        h_level[t] = (uint8_t)l;
    }
    *n_levels = std::min(distinct, ttg::kMaxLevels);
}

}  // namespace

extern "C" ttg_status ttg_run_graph_noalloc(int device, const ttg_graph_desc* gd, int workers, double timeout_s,
                                            void* stream, ttg_report* rep) {
    if (!gd || gd->n_tasks < 0 || device < 0 || device >= 64) return TTG_EINVAL;
    const int n = gd->n_tasks;
    if (n > (int)kT) return TTG_EINVAL;
    if (n > 0 && (!gd->ops || !gd->init_count || !gd->succ_ptr)) return TTG_EINVAL;
    const int64_t n_edges = n > 0 ? gd->succ_ptr[n] : 0;
    if (n > 0 && gd->succ_ptr[0] != 0) return TTG_EINVAL;
    if (n_edges < 0 || n_edges > (int64_t)kE || (n_edges > 0 && !gd->succ_idx)) return TTG_EINVAL;
    for (int t = 0; t < n; ++t) {
        if (gd->init_count[t] < 0 || gd->succ_ptr[t] > gd->succ_ptr[t + 1]) return TTG_EINVAL;
        if (gd->ops[t].kind < TTG_OP_NOP || gd->ops[t].kind > TTG_OP_GEADD) return TTG_EINVAL;
        // The FP64 tile kernels only: a mixed-precision op's tiles are FP32
        // or BF16 and would be read as doubles.
        if (gd->ops[t].kind != TTG_OP_NOP && gd->ops[t].prec != TTG_PREC_F64) return TTG_EINVAL;
    }
    for (int64_t e = 0; e < n_edges; ++e)
        if (gd->succ_idx[e] < 0 || gd->succ_idx[e] >= n) return TTG_EINVAL;

    std::lock_guard<std::mutex> guard(g_lock);
    TTG_CUDA_CHECK(cudaSetDevice(device));
    DeviceSetup& d = g_setup[device];
    ttg_status st = setup_device(device, d);
    if (st != TTG_OK) return st;
    const int W = workers > 0 ? std::min(workers, d.max_workers) : std::min(d.sms, d.max_workers);
    if (W > (int)kW) return TTG_EINVAL;

    // Host simulation of the counters (which tasks will run; overcount).
    int top = 0;
    bool over = false;
    for (int t = 0; t < n; ++t) {
        h_sim[t] = gd->init_count[t];
        h_runnable[t] = 0;
        if (h_sim[t] == 0) {
            h_runnable[t] = 1;
            h_stack[top++] = t;
        }
    }
    while (top > 0) {
        const int t = h_stack[--top];
        for (int64_t e = gd->succ_ptr[t]; e < gd->succ_ptr[t + 1]; ++e) {
            const int s = gd->succ_idx[e];
            if (--h_sim[s] == 0) {
                h_runnable[s] = 1;
                h_stack[top++] = s;
            } else if (h_sim[s] < 0) {
                over = true;
            }
        }
    }
    int n_runnable = 0;
    for (int t = 0; t < n; ++t) n_runnable += h_runnable[t];
    int n_levels = 1;
    levels_static(n, gd->priority, &n_levels);

    // Queue layout: level queues then bound queues, one slot per part.
    long q_total = 0;
    for (int l = 0; l < ttg::kMaxLevels; ++l) h_qfill[l] = 0;
    for (int w = 0; w < W; ++w) h_bqfill[w] = 0;
    for (int t = 0; t < n; ++t) {
        h_ops[t] = gd->ops[t];
        h_parts[t] = ttg_task_parts(gd->ops[t]);
        h_bind[t] = (gd->bind && gd->bind[t] >= 0) ? gd->bind[t] : -1;
        h_count[t] = gd->init_count[t];
        if (!h_runnable[t]) continue;
        const int slots = h_parts[t];
        if (h_bind[t] >= 0) h_bqfill[h_bind[t] % W] += slots;
        else h_qfill[h_level[t]] += slots;
        q_total += slots;
    }
    if (q_total > (long)kQ) return TTG_EINVAL;
    h_qoff[0] = 0;
    for (int l = 0; l < ttg::kMaxLevels; ++l) h_qoff[l + 1] = h_qoff[l] + h_qfill[l];
    h_bqoff[0] = 0;
    for (int w = 0; w < W; ++w) h_bqoff[w + 1] = h_bqoff[w] + h_bqfill[w];
    const int q_levels = h_qoff[ttg::kMaxLevels];
    for (long i = 0; i < q_total; ++i) h_qbuf[i] = -1;
    for (int i = 0; i < ttg::kMaxLevels * 32; ++i) h_qtail[i] = 0;
    for (int w = 0; w < W; ++w) h_bqtail[w] = 0;
    for (int t = 0; t < n; ++t) {
        if (gd->init_count[t] != 0) continue;
        if (h_bind[t] >= 0) {
            const int w = h_bind[t] % W;
            for (int q = 0; q < h_parts[t]; ++q) h_qbuf[q_levels + h_bqoff[w] + h_bqtail[w]++] = t;
        } else {
            const int l = h_level[t];
            for (int q = 0; q < h_parts[t]; ++q) h_qbuf[h_qoff[l] + h_qtail[l * 32]++] = t;
        }
    }
    for (int l = 0; l < ttg::kMaxLevels; ++l) h_qtail[l * 32 + 1] = h_qtail[l * 32];  // available at launch
    std::memset(&h_status, 0, sizeof(h_status));
    h_status.start = ~0ULL;

    // Fill the scratch, launch and read the status back.  Every array the
    // kernel reads is rewritten here.
    unsigned char* S = d.scratch;
    cudaStream_t s = (cudaStream_t)stream;
    RunStatus* dst = (RunStatus*)(S + oStatus);
    auto enqueue = [&]() -> ttg_status {
        if (n > 0) {
            TTG_CUDA_CHECK(cudaMemcpyAsync(S + oOps, h_ops, sizeof(ttg_op) * n, cudaMemcpyHostToDevice, s));
            TTG_CUDA_CHECK(cudaMemcpyAsync(S + oCount, h_count, 4 * n, cudaMemcpyHostToDevice, s));
            TTG_CUDA_CHECK(cudaMemsetAsync(S + oRuns, 0, 4 * n, s));
            TTG_CUDA_CHECK(cudaMemcpyAsync(S + oParts, h_parts, 4 * n, cudaMemcpyHostToDevice, s));
            TTG_CUDA_CHECK(cudaMemsetAsync(S + oPartNext, 0, 4 * n, s));
            TTG_CUDA_CHECK(cudaMemsetAsync(S + oPartDone, 0, 4 * n, s));
            TTG_CUDA_CHECK(cudaMemcpyAsync(S + oBind, h_bind, 4 * n, cudaMemcpyHostToDevice, s));
            TTG_CUDA_CHECK(cudaMemcpyAsync(S + oLevel, h_level, n, cudaMemcpyHostToDevice, s));
            TTG_CUDA_CHECK(cudaMemcpyAsync(S + oRunnable, h_runnable, n, cudaMemcpyHostToDevice, s));
            TTG_CUDA_CHECK(cudaMemcpyAsync(S + oSuccPtr, gd->succ_ptr, 8 * (n + 1), cudaMemcpyHostToDevice, s));
        }
        if (n_edges > 0) TTG_CUDA_CHECK(cudaMemcpyAsync(S + oSuccIdx, gd->succ_idx, 4 * n_edges, cudaMemcpyHostToDevice, s));
        if (q_total > 0) TTG_CUDA_CHECK(cudaMemcpyAsync(S + oQbuf, h_qbuf, 4 * q_total, cudaMemcpyHostToDevice, s));
        TTG_CUDA_CHECK(cudaMemcpyAsync(S + oQoff, h_qoff, 4 * (ttg::kMaxLevels + 1), cudaMemcpyHostToDevice, s));
        TTG_CUDA_CHECK(cudaMemsetAsync(S + oQhead, 0, 4 * ttg::kMaxLevels * 32, s));
        TTG_CUDA_CHECK(cudaMemcpyAsync(S + oQtail, h_qtail, 4 * ttg::kMaxLevels * 32, cudaMemcpyHostToDevice, s));
        TTG_CUDA_CHECK(cudaMemcpyAsync(S + oBqoff, h_bqoff, 4 * (W + 1), cudaMemcpyHostToDevice, s));
        TTG_CUDA_CHECK(cudaMemsetAsync(S + oBqhead, 0, 4 * W, s));
        TTG_CUDA_CHECK(cudaMemcpyAsync(S + oBqtail, h_bqtail, 4 * W, cudaMemcpyHostToDevice, s));
        TTG_CUDA_CHECK(cudaMemcpyAsync(S + oStatus, &h_status, sizeof(h_status), cudaMemcpyHostToDevice, s));

        if (n_runnable > 0) {
            ttg::ExecParams p;
            p.ops = (const ttg_op*)(S + oOps);
            p.n_tasks = n;
            p.n_runnable = n_runnable;
            p.count = (int*)(S + oCount);
            p.runs = (int*)(S + oRuns);
            p.parts = (const int*)(S + oParts);
            p.part_next = (int*)(S + oPartNext);
            p.part_done = (int*)(S + oPartDone);
            p.succ_ptr = (const int64_t*)(S + oSuccPtr);
            p.succ_idx = (const int32_t*)(S + oSuccIdx);
            p.level = (const uint8_t*)(S + oLevel);
            p.bind = (const int32_t*)(S + oBind);
            p.n_levels = n_levels;
            p.n_workers = W;
            p.qbuf = (int*)(S + oQbuf);
            p.q_off = (const int*)(S + oQoff);
            p.q_head = (int*)(S + oQhead);
            p.q_tail = (int*)(S + oQtail);
            p.bq_buf = (int*)(S + oQbuf) + q_levels;
            p.bq_off = (const int*)(S + oBqoff);
            p.bq_head = (int*)(S + oBqhead);
            p.bq_tail = (int*)(S + oBqtail);
            p.has_bound = h_bqoff[W] > 0;
            p.done = &dst->done;
            p.err = &dst->err;
            p.err_task = &dst->err_task;
            p.err_info = &dst->err_info;
            p.trace = nullptr;
            p.timeout_ns = (long long)((timeout_s > 0 ? timeout_s : 10.0) * 1e9);
            p.pub = nullptr;  // a closed graph
            p.roots = nullptr;
            p.admit = nullptr;
            p.team_ctr = nullptr;  // POTRF tasks run on one block here
            p.team_slot = nullptr;
            void* args[] = {(void*)&p, (void*)&dst};
            TTG_CUDA_CHECK(cudaLaunchCooperativeKernel((const void*)exec_kernel_noalloc, dim3(W), dim3(ttg::kThreads), args,
                                                       ttg::kF64SmemDoubles * sizeof(double), s));
        }
        if (n > 0) {
            summarize_noalloc<<<std::max(1, std::min(64, (n + 255) / 256)), 256, 0, s>>>(
                (const int*)(S + oRuns), (const int*)(S + oCount), (const uint8_t*)(S + oRunnable), n, dst);
            TTG_CUDA_CHECK(cudaGetLastError());
        }
        TTG_CUDA_CHECK(cudaMemcpyAsync(&h_status, dst, sizeof(h_status), cudaMemcpyDeviceToHost, s));
        return TTG_OK;
    };
    const ttg_status enq = enqueue();
    // Whatever was enqueued finishes before the lock is released, also when
    // a step failed: the next call rewrites the shared scratch.
    const cudaError_t se = cudaStreamSynchronize(s);
    if (enq != TTG_OK) return enq;
    TTG_CUDA_CHECK(se);

    const int err = h_status.err;
    ttg_status result = err;
    if (result == TTG_OK && over) result = TTG_EOVERCOUNT;
    if (result == TTG_OK && n_runnable < n) result = TTG_EUNDERRUN;
    if (rep) {
        rep->tasks_total = n;
        rep->tasks_run = (int64_t)h_status.ran;
        rep->tasks_pending = (int64_t)h_status.pending;
        rep->bad_runs = (int64_t)h_status.bad;
        rep->status = result;
        rep->error_task = err ? h_status.err_task : -1;
        rep->info = h_status.err_info;
        rep->workers = W;
        rep->elapsed_ms =
            (n_runnable > 0 && h_status.end >= h_status.start) ? (float)((h_status.end - h_status.start) * 1e-6) : 0.f;
    }
    return result;
}
