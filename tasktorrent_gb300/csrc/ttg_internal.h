// ttg_internal.h — context and device-graph state shared by the .cu files of
// libttg.so.  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <unordered_map>

#include "../../include/ttg.h"

namespace ttg {
struct ExecParams;
}

struct DevGraph {
    int n_tasks = 0;
    int n_runnable = 0;
    int n_levels = 1;
    int has_bound = 0;
    int q_total = 0;
    int bq_total = 0;
    int bq_image = 0;
    ttg_op* ops = nullptr;
    int* init = nullptr;
    int* count = nullptr;
    int* runs = nullptr;
    int* parts = nullptr;
    int* part_next = nullptr;
    int* part_done = nullptr;
    int64_t* succ_ptr = nullptr;
    int32_t* succ_idx = nullptr;
    uint8_t* level = nullptr;
    int* bind = nullptr;
    uint8_t* runnable = nullptr;
    int* qbuf = nullptr;
    int* qinit = nullptr;
    int* q_off = nullptr;
    int* q_head = nullptr;
    int* q_tail = nullptr;
    int* q_tail_init = nullptr;
    int* bq_buf = nullptr;
    int* bq_off = nullptr;
    int* bq_head = nullptr;
    int* bq_tail = nullptr;
    long long* trace = nullptr;
    int n_team = 0;             // POTRF tasks factored by a team of blocks
    int* team_ctr = nullptr;    // kTeamStride words per team task
    int* team_slot = nullptr;   // per task: team counter block or -1
    // Capacity (elements) of each buffer above, keyed by the field's address:
    // a new upload reuses buffers that are large enough, so uploading a graph
    // frees nothing (cudaFree would wait for the whole device).
    std::unordered_map<const void*, size_t> cap;
};

struct ttg_ctx {
    int device = 0;
    int sms = 0;
    int workers = 0;
    int max_workers_f64 = 0;  // co-resident blocks of the FP64 executor
    double timeout_s = 10.0;
    int trace = 0;
    bool uploaded = false;
    bool launched = false;
    bool g_mixed = false;     // the uploaded graph has mixed-precision tasks
    bool coop = true;         // cooperative launches (off: graphs without bound tasks may
                              // start while other kernels hold part of the GPU)
    uint64_t graph_gen = 0;   // incremented by every successful upload
    int pending_host = 0;     // tasks that will never become ready
    bool overcount_host = false;
    ttg_status last_status = TTG_OK;
    DevGraph g;
    int* status = nullptr;    // device: done, err, err_task, err_info, ran, pending, bad, spare
    int* h_status = nullptr;  // pinned host copy
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaStream_t stream = nullptr;
    void* mixed = nullptr;    // mixed-path resources (ttg_mixed.cu)
};

void ttg_set_last_cuda_error(cudaError_t e, const char* expr, const char* file, int line);
// Count one kernel launch of this library (ttg_kernel_launches).
void ttg_note_launch(int n = 1);
ttg_status ttg_ctx_init_device(ttg_ctx* c);
ttg_status ttg_reset_state(ttg_ctx* c, cudaStream_t s);
ttg_status ttg_launch_executor(ttg_ctx* c, const ttg::ExecParams& p, cudaStream_t s);
// A cooperative launch (every block resident) through cudaLaunchKernelEx, so
// that it can also be recorded into a CUDA graph.
cudaError_t ttg_launch_cooperative(const void* fn, int grid, int block, void** args, size_t smem, cudaStream_t s);
// Enqueue the counter/queue reset and the executor launch of the uploaded
// graph on s (no events): the body of a recorded CUDA graph.
ttg_status ttg_enqueue_run(ttg_ctx* c, cudaStream_t s);
// Cooperative, or plain when c->coop is off and the graph has no bound tasks.
cudaError_t ttg_launch_executor_kernel(ttg_ctx* c, const void* fn, void** args, size_t smem, cudaStream_t s);
// After a recorded graph holding ttg_enqueue_run was launched on s between
// the context's events: let ttg_wait collect the run.
ttg_status ttg_mark_launched(ttg_ctx* c, cudaStream_t s);
cudaEvent_t ttg_event(ttg_ctx* c, int which);
void ttg_graph_free(ttg_ctx* c);
// Blocks that share one task.  team: a POTRF may be split over a team of
// blocks (needs a team counter block at run time).
int ttg_task_parts(const ttg_op& op, bool team = false);
// A 32-bit store of v at addr (device memory) enqueued on stream s after its
// earlier work, copies included (cuStreamWriteValue32: no SM needed).
ttg_status ttg_stream_write_u32(cudaStream_t s, uint32_t* addr, uint32_t v);

// Lower tiles of the miniapp matrix 1/((i-j)^2+1) (ttg_gen.cu).
ttg_status ttg_gen_miniapp_tiles(ttg_ctx* c, const int32_t* h_bs, int32_t nb, double* d_tiles, void* stream);

// Lower tiles (uniform tile, a multiple of 64 or >= n, the last ragged) of
// A = G·Gᵀ/n + αI as ttg_gen_gram_tiles, enqueued on s without waiting
// (stream-ordered scratch).
ttg_status ttg_gen_gram_async(ttg_ctx* c, int n, int tile, double alpha, uint32_t seed, double* d_tiles, cudaStream_t s);
// Right-hand sides as an nrhs × n row block (ld nrhs), entry (r, q) of the
// column-major N(0,1) array of (seed, stream 1); enqueued on s.
ttg_status ttg_gen_rhs_rows_async(int n, int nrhs, uint32_t seed, double* d_B, cudaStream_t s);
// Load the two generators' kernels now.  With lazy module loading the first
// launch of a kernel waits for the device to be idle, which never happens
// while a persistent executor waits for work: load them before one starts.
ttg_status ttg_gen_preload();

// Block-GEMM inputs in tile layout (ttg_gen.cu).
ttg_status ttg_gen_gemm_tiles(ttg_ctx* c, int32_t N, int32_t b, int32_t inputs, uint32_t seed, double* d_A, double* d_B,
                              void* stream);

// Mixed-precision path (ttg_mixed.cu).
ttg_status ttg_mixed_init(ttg_ctx* c);
void ttg_mixed_free(ttg_ctx* c);
ttg_status ttg_launch_mixed(ttg_ctx* c, const ttg::ExecParams& p, cudaStream_t s);
int ttg_mixed_max_workers(const ttg_ctx* c);

#define TTG_CUDA_CHECK(expr)                                                            \
    do {                                                                                \
        cudaError_t _e = (expr);                                                        \
        if (_e != cudaSuccess) {                                                        \
            ttg_set_last_cuda_error(_e, #expr, __FILE__, __LINE__);                     \
            return _e == cudaErrorMemoryAllocation ? TTG_ENOMEM : TTG_ECUDA;            \
        }                                                                               \
    } while (0)
