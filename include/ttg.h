/*
 * ttg.h — C ABI of the GB300 task-graph executor (libttg.so).
 *
 * This is the boundary between the host-side drop-in of TaskTorrent's
 * ttor::Taskflow<K> / ttor::Threadpool_shared (C++ headers under
 * tasktorrent_gb300/tasktorrent/) and the CUDA runtime.  In the reference the
 * same boundary is the call from Taskflow into the thread pool:
 *
 *   Taskflow::fulfill_promise -> Threadpool_shared::insert(Task*, where, binding)
 *     (tasktorrent/src/taskflow.hpp:241-296, threadpool_shared.cpp:200-224)
 *   Threadpool_shared::join()  (threadpool_shared.cpp:234-241)
 *
 * Here the host records the task graph once (task kind + operand tiles, the
 * indegree, priority and binding of every task, and the successor lists that
 * fulfill() produces), uploads it, and one persistent kernel runs it: its
 * blocks pop ready tasks from device queues, run the tile kernel, and
 * decrement successor counters with atomics.
 *
 * Conventions: every function returns a ttg_status (0 = success) and never
 * aborts; pointers named d_* are device pointers, h_* host pointers; matrices
 * and tiles are column-major.  A ttg_ctx is not thread-safe: use one per host
 * thread.  Device buffers passed in are owned by the caller; the context owns
 * the uploaded graph, the queues, the counters and the trace buffer.
 */
#ifndef TTG_H
#define TTG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int ttg_status;
enum {
    TTG_OK = 0,
    TTG_EINVAL = 1,     /* bad argument                                            */
    TTG_ECUDA = 2,      /* a CUDA runtime call failed                              */
    TTG_ETIMEOUT = 3,   /* the executor made no progress within the time limit     */
    TTG_EOVERCOUNT = 4, /* a task received more promises than its indegree         */
    TTG_ENOTPD = 5,     /* a diagonal tile is not positive definite                */
    TTG_ENOMEM = 6,     /* device allocation failed                                */
    TTG_ESTATE = 7,     /* call out of order (e.g. launch before upload)           */
    TTG_EUNDERRUN = 8,  /* some tasks never became ready (indegree too large)      */
    TTG_ENOCONV = 9     /* iterative refinement did not reach the requested error  */
};

const char* ttg_strerror(ttg_status s);

/* Text of the last CUDA runtime error behind a TTG_ECUDA / TTG_ENOMEM status
 * (the failing call and its source location), or an empty string. */
const char* ttg_last_cuda_error(void);

/* Kernels this library has launched in the process so far (executor runs,
 * solver, generator and conversion kernels; a replayed CUDA graph counts its
 * kernels again).  Differences bracket a region of work. */
int64_t ttg_kernel_launches(void);

/* Item idx of the team POTRF dataflow of a P×P-block diagonal tile (the
 * order the team's blocks claim items in): *kind 0 = F(p) (panel block
 * (p,p-1), last update and factor of the diagonal block p), 1 = R(p, bi)
 * (panel block (bi,p)), 2 = T(p, bi, bj) (update of block (bi,bj) by panel
 * p), -1 past the last item.  Host computation of the device's table, for
 * checking the order (every item once, every wait on an earlier claim). */
ttg_status ttg_team_item(int32_t P, int32_t idx, int32_t* kind, int32_t* p, int32_t* bi, int32_t* bj);

/* ------------------------------------------------------------------ tasks */

/* Tile operation of one task.  The reference task bodies call BLAS/LAPACK on
 * tiles (miniapp/dense_cholesky/2d_cholesky.cpp:319,404-405,490-494;
 * miniapp/gemm/2d_gemm.cpp:157); each kind below is one of those calls. */
enum {
    TTG_OP_NOP = 0,       /* no device work (pure dependency task)                  */
    TTG_OP_POTRF_L = 1,   /* c[n×n] <- lower Cholesky factor, in place (LAPACKE_dpotrf 'L') */
    TTG_OP_TRSM_RLTN = 2, /* c[m×n] <- alpha c · a⁻ᵀ, a[n×n] lower non-unit (cblas_dtrsm R,L,T,N) */
    TTG_OP_SYRK_LN = 3,   /* lower(c[n×n]) <- alpha a·aᵀ + beta c, a[n×k] (cblas_dsyrk L,N) */
    TTG_OP_GEMM_NT = 4,   /* c[m×n] <- alpha a·bᵀ + beta c, a[m×k], b[n×k] (cblas_dgemm N,T) */
    TTG_OP_GEMM_NN = 5,   /* c[m×n] <- alpha a·b + beta c, a[m×k], b[k×n]  (cblas_dgemm N,N) */
    TTG_OP_GEADD = 6,     /* c[m×n] <- alpha a + beta c  (tile accumulation)          */
    TTG_OP_TRSM_RLNN = 7, /* c[m×n] <- alpha c · a⁻¹, a[n×n] lower non-unit (cblas_dtrsm R,L,N,N):
                             the backward step of a block solve with row-vector RHS */
    TTG_OP_CONVERT = 8,   /* c[m×n] <- alpha a + beta c with a and c of either precision:
                             flags bit 0 = a is float, bit 1 = c is float; bit 2 (mixed-precision
                             plans' input tasks) = first wait until word 1 + k of the uint32
                             array aux equals its word 0 (the tile column has arrived) */
    TTG_OP_SPIN = 9       /* the block spins for alpha seconds (0 <= alpha <= 1): the
                             task body of the scheduler micro-benchmarks
                             (miniapp/mini_benchmarks/shared/ttor_wait.cpp, ttor_deps.cpp,
                             spin_for_seconds in mini_benchmarks/common.hpp:21-28) */
};

/* Arithmetic of one task. */
enum {
    TTG_PREC_F64 = 0,      /* a, b, c are double                                         */
    TTG_PREC_MIXED = 1     /* mixed-precision tile path, see ttg_mixed_tile below        */
};

typedef struct ttg_op {
    int32_t kind;      /* TTG_OP_*                           */
    int32_t prec;      /* TTG_PREC_*                         */
    int32_t m, n, k;   /* dimensions as in the BLAS call      */
    int32_t lda, ldb, ldc;
    int32_t parts;     /* blocks that share the task: 0 = chosen by the executor
                          (one per 128×128 output block, up to 16; TRSM by
                          128-row slices; POTRF: a team of n/16 blocks up to
                          32 for n >= 128, else 1), else that many (POTRF:
                          up to 64; the factor is the same for any count)   */
    int32_t flags;     /* reserved, 0                         */
    double alpha, beta;
    const void* a;     /* device pointers                     */
    const void* b;
    void* c;
    void* aux;         /* per-kind extra data (mixed path)    */
} ttg_op;

/* A task graph in compressed form.  Task t is ready when its counter reaches
 * zero; init_count[t] is its indegree minus the promises made before launch
 * (the reference's seeding from the main thread, 2d_cholesky.cpp:613-615). */
typedef struct ttg_graph_desc {
    int32_t n_tasks;
    const ttg_op* ops;          /* [n_tasks] host array                                    */
    const int32_t* init_count;  /* [n_tasks]                                               */
    const double* priority;     /* [n_tasks] or NULL; higher runs first (set_priority)     */
    const int32_t* bind;        /* [n_tasks] or NULL; -1 = stealable, w >= 0 = run only on
                                   worker w mod workers (set_mapping + set_binding)        */
    const int64_t* succ_ptr;    /* [n_tasks+1] CSR offsets into succ_idx                   */
    const int32_t* succ_idx;    /* successors; one entry per fulfill_promise call          */
} ttg_graph_desc;

/* ---------------------------------------------------------------- context */

typedef struct ttg_opts {
    int device;          /* CUDA device ordinal                                     */
    int workers;         /* persistent blocks; 0 = one per SM                         */
    double timeout_s;    /* no-progress limit of the executor; 0 = 10 s              */
    int trace;           /* record per-task start/end times and worker               */
} ttg_opts;

typedef struct ttg_report {
    int64_t tasks_total;    /* tasks in the graph                                    */
    int64_t tasks_run;      /* tasks the device completed                            */
    int64_t tasks_pending;  /* counters that did not reach zero                      */
    int64_t bad_runs;       /* tasks that ran other than exactly once                */
    int32_t status;         /* ttg_status of the run                                 */
    int32_t error_task;     /* first task that reported an error, or -1              */
    int32_t info;           /* POTRF: 1-based failing column inside error_task        */
    int32_t workers;        /* blocks used                                           */
    float elapsed_ms;       /* launch to completion (CUDA events on the stream)       */
} ttg_report;

typedef struct ttg_ctx ttg_ctx;

ttg_status ttg_create(ttg_ctx** ctx, const ttg_opts* opts);
ttg_status ttg_destroy(ttg_ctx* ctx);

/* Upload a task graph (replaces any previous one).  Copies everything. */
ttg_status ttg_graph_upload(ttg_ctx* ctx, const ttg_graph_desc* g);

/* Reset the counters and queues and launch the persistent executor on
 * `stream` (a cudaStream_t; NULL = legacy default stream).  Asynchronous. */
ttg_status ttg_launch(ttg_ctx* ctx, void* stream);

/* Wait for the launched run and fill `rep` (may be NULL). */
ttg_status ttg_wait(ttg_ctx* ctx, ttg_report* rep);

/* ttg_launch + ttg_wait. */
ttg_status ttg_run(ttg_ctx* ctx, void* stream, ttg_report* rep);

/* Per-task record of the last run: how often each task ran and its counter at
 * the end (both int32[n_tasks], host). */
ttg_status ttg_task_record(ttg_ctx* ctx, int32_t* h_runs, int32_t* h_final_count);

/* Per-task trace of the last run (opts.trace): start/end in ns of the GPU
 * global timer relative to the earliest start, and the worker (block) id. */
ttg_status ttg_trace(ttg_ctx* ctx, int64_t* h_start_ns, int64_t* h_end_ns, int32_t* h_worker);

/* Extension: priorities for a graph from the longest path (in estimated
 * device time: flops over the per-block rate of each task kind, shared by the
 * task's parts) from each task to the end of the graph.  out[n_tasks]; higher
 * runs first, as ttg_graph_desc.priority.  TTG_EINVAL for a cyclic graph. */
ttg_status ttg_critical_path_priority(const ttg_graph_desc* g, double* out);

/* Per-task busy time of the last run (opts.trace): the durations of all its
 * parts added up, in ns.  A task shared by P blocks that ran together shows
 * about P times its span. */
ttg_status ttg_trace_busy(ttg_ctx* ctx, int64_t* h_busy_ns);

/* Number of persistent workers the context launches. */
int ttg_workers(const ttg_ctx* ctx);

/* Extension: change the number of persistent blocks of a context (1 ..
 * the resident maximum; 0 = the maximum).  A change drops the uploaded graph
 * (its queues are laid out per worker): upload again before the next launch
 * (the graph generation changes, so plans do so by themselves). */
ttg_status ttg_set_workers(ttg_ctx* ctx, int32_t workers);

/* Identifier of the graph currently uploaded to the context (changes with
 * every successful ttg_graph_upload): a host-side owner of a graph compares
 * it to decide whether to upload again before relaunching. */
uint64_t ttg_graph_generation(const ttg_ctx* ctx);

/* Measured FP64 FMA throughput of the device (TFLOP/s): every block of the
 * device runs independent DFMA chains for about `ms` milliseconds.  The
 * roofline denominator of the FP64 tile kernels. */
ttg_status ttg_measure_fp64_peak(ttg_ctx* ctx, double ms, double* tflops);

/* ---------------------------------------------------- run without allocation */

/* No counterpart in the reference: an addition for callers that cannot call
 * cudaMalloc — a service whose memory pool already owns the free device
 * memory, an operator hosted by another framework that may only allocate
 * through that framework, or a caller that cannot afford the device-wide
 * synchronisation an allocation can cause.  ttg_run_graph_noalloc uploads the
 * graph and runs the FP64 executor with all of its scratch (the graph copy,
 * counters, queues, status words) in one fixed device array of
 * TTG_NOALLOC_SCRATCH_BYTES that every GPU loading libttg.so reserves until
 * the process exits; it calls no device allocation routine.
 *
 * Limits: n_tasks <= TTG_NOALLOC_MAX_TASKS, successor entries <=
 * TTG_NOALLOC_MAX_EDGES, queue entries (parts of the runnable tasks, see
 * ttg_op.parts) <= TTG_NOALLOC_MAX_QUEUE, workers <= TTG_NOALLOC_MAX_WORKERS;
 * larger graphs are rejected with TTG_EINVAL before anything is written.
 * Only TTG_PREC_F64 tasks.  The tiles in the ops are the caller's (inputs and
 * outputs); `workers` 0 = one per SM; `timeout_s` 0 = 10 s.
 *
 * Every call shares the array and finds the previous call's contents in it:
 * each call rewrites all of it that the kernel reads.  Calls that overlapped
 * on the GPU would race on it, so calls are serialised by a process-wide lock
 * and each call waits for `stream` before returning.  The first call on a
 * device also looks up the array's device address (with that device
 * current); make that first call before any stream capture begins. */
#define TTG_NOALLOC_MAX_TASKS 16384
#define TTG_NOALLOC_MAX_EDGES 131072
#define TTG_NOALLOC_MAX_QUEUE 262144
#define TTG_NOALLOC_MAX_WORKERS 1024
#define TTG_NOALLOC_SCRATCH_BYTES (4u << 20)
ttg_status ttg_run_graph_noalloc(int device, const ttg_graph_desc* g, int workers, double timeout_s, void* stream,
                                 ttg_report* rep);

/* ------------------------------------------------------------ generators */
/* Seeded inputs of the workloads (include/ttg_philox.h), built on the device. */

/* Lower tiles of A = G·Gᵀ/N + alpha·I, G the quantised Gaussian of (seed).
 * Tiles are stored back to back, tile (i,j), i >= j, at d_tiles + off[i,j],
 * column-major with leading dimension bs[i]; off/bs as in ttg_tile_layout. */
ttg_status ttg_gen_gram_tiles(ttg_ctx* ctx, int32_t n, const int32_t* h_block_sizes, int32_t num_blocks,
                              double alpha, uint32_t seed, double* d_tiles, void* stream);

/* Dense N×N column-major U[-1,1] matrix from (seed, stream id). */
ttg_status ttg_gen_uniform(ttg_ctx* ctx, int64_t count, uint32_t seed, uint32_t stream_id, double* d_out, void* stream);

/* Dense column-major N(0,1) matrix from (seed, stream id). */
ttg_status ttg_gen_normal(ttg_ctx* ctx, int64_t count, uint32_t seed, uint32_t stream_id, double* d_out, void* stream);

/* Offsets (in elements) of the packed lower-tile layout: off[i + j*nb] for
 * i >= j, and the total element count. */
int64_t ttg_tile_layout(const int32_t* h_block_sizes, int32_t num_blocks, int64_t* h_off);

#ifdef __cplusplus
}
#endif

#endif /* TTG_H */
