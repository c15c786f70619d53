/*
 * ttg_apps.h — C ABI of the two workloads of the reference's miniapps, built
 * on the Taskflow<K> drop-in and the persistent executor (libttg.so).
 *
 *   Cholesky plan: the task graph of miniapp/dense_cholesky/2d_cholesky.cpp at
 *     one rank (potrf/trsm/gemm flows, optional accu flow, priorities, uneven
 *     block sizes) on lower tiles resident in device memory.
 *   GEMM plan: the task graph of miniapp/gemm/2d_gemm.cpp at one rank
 *     (send_Aij, send_Bij, gemm_Cikj chained over k) on resident tiles.
 *
 * A plan is created once (tiles allocated, graph captured and uploaded) and
 * then factorised / multiplied any number of times; each run restores the
 * input tiles first.  All functions return a ttg_status and never abort.
 */
#ifndef TTG_APPS_H
#define TTG_APPS_H

#include "ttg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Arguments of 2d_cholesky (2d_cholesky.cpp:705-719) at one rank, plus the
 * GB300 additions (matrix, alpha, seed, precision, workers). */
typedef struct ttg_chol_args {
    int32_t n_threads;        /* --n_threads: mapping modulus of the task graph     */
    int32_t verb;             /* --verb                                            */
    int32_t block_size;       /* --block_size                                      */
    int32_t num_blocks;       /* --num_blocks                                      */
    int32_t kind;             /* --kind: 0 none, 1 row, 2 critical path, 3 cp+row;
                                 4 (extension): longest remaining path in
                                 estimated device time (ttg_critical_path_priority);
                                 5 (extension): look-ahead — POTRF, then TRSM and
                                 the next panel column's updates, then the rest;
                                 6 (extension): the tasks of the tiles within
                                 two of the diagonal above all others (by
                                 column), the rest as kind 2                    */
    int32_t accumulate;       /* --accumulate                                      */
    int32_t upper_block_size; /* --upper_block_size (-1 = block_size)              */
    int32_t matrix;           /* 0: 1/((i-j)^2+1) (the miniapp's); 1: G·Gᵀ/N + αI    */
    double alpha;
    uint32_t seed;
    int32_t precision;        /* TTG_PREC_F64 or TTG_PREC_MIXED                     */
    int32_t mixed_kind;       /* mixed path: 0 = BF16 tensor-core updates, 1 = FP32
                                 updates, 2 = split-BF16 tensor-core updates (three
                                 BF16 slices per operand, six products, FP32-level
                                 accuracy), 3 = split-FP16 tensor-core updates (two
                                 FP16 slices, three products, ~2^-22 accuracy; in
                                 ttg_chol_posv* a first refinement step that gains
                                 < 10x replaces it by the split-BF16 factor); 0, 2
                                 and 3 need uniform tiles, a multiple of 128        */
} ttg_chol_args;

typedef struct ttg_chol_plan ttg_chol_plan;

ttg_status ttg_chol_plan_create(ttg_ctx* ctx, const ttg_chol_args* args, ttg_chol_plan** plan);
ttg_status ttg_chol_plan_destroy(ttg_chol_plan* plan);

/* Matrix order and block sizes (h_bs may be NULL). */
int32_t ttg_chol_plan_n(const ttg_chol_plan* plan, int32_t* h_bs);
/* Number of device tasks of the captured graph and the capture time (s). */
int32_t ttg_chol_plan_tasks(const ttg_chol_plan* plan, double* capture_s);

/* Input: regenerate it on the device from args (matrix/alpha/seed). */
ttg_status ttg_chol_plan_generate(ttg_chol_plan* plan, void* stream);
/* Input: dense N×N column-major symmetric matrix in host memory (lower part
 * read).  Copies into the pristine tiles. */
ttg_status ttg_chol_plan_set_matrix(ttg_chol_plan* plan, const double* h_A, void* stream);

/* Restore the working tiles from the pristine input (device copy). */
ttg_status ttg_chol_plan_restore(ttg_chol_plan* plan, void* stream);
/* Run the captured task graph once: an FP64 plan on the working tiles (no
 * restore), a mixed plan on the pristine input (converted to FP32). */
ttg_status ttg_chol_plan_factor(ttg_chol_plan* plan, void* stream, ttg_report* rep);

/* End-to-end: host matrix in (pinned or pageable), factor, host factor out.
 * h_L receives the dense N×N lower factor (upper part zeroed). */
ttg_status ttg_chol_factor_host(ttg_chol_plan* plan, const double* h_A, double* h_L, void* stream, ttg_report* rep);

/* End-to-end with host buffers in the plan's packed lower-tile layout
 * (ttg_tile_layout order; host memory, pinned for full bandwidth): h_tiles_in
 * -> factor -> h_tiles_out (may alias).  One copy each way. */
ttg_status ttg_chol_factor_host_tiles(ttg_chol_plan* plan, const double* h_tiles_in, double* h_tiles_out, void* stream,
                                      ttg_report* rep);
/* Copy the packed tiles to host: which = 0 working tiles (the factor after a
 * run), 1 the pristine input. */
ttg_status ttg_chol_plan_copy_tiles(ttg_chol_plan* plan, int32_t which, double* h_dst);
/* Number of doubles of the packed lower-tile layout. */
int64_t ttg_chol_plan_tile_elems(const ttg_chol_plan* plan);

/* The factor as a dense N×N column-major lower-triangular host array. */
ttg_status ttg_chol_plan_get_factor(ttg_chol_plan* plan, double* h_L);
/* The input as a dense N×N column-major symmetric host array. */
ttg_status ttg_chol_plan_get_input(ttg_chol_plan* plan, double* h_A);

/* Device pointers of the working tiles (lower, packed) and their offsets.
 * An FP64 plan factors these tiles in place; a mixed plan factors its input
 * (ttg_chol_plan_set_matrix / _generate) and uses them as FP64 scratch. */
double* ttg_chol_plan_tiles(ttg_chol_plan* plan, const int64_t** h_off);

/* DAG record of the last run in the oracle's CSV format. */
ttg_status ttg_chol_plan_dump_dag(ttg_chol_plan* plan, const char* prefix);
/* Capture the Cholesky task graph on the host only (no device, no tiles)
 * and write its DAG record — the graph a plan with these arguments runs. */
ttg_status ttg_chol_dag_dump(const ttg_chol_args* args, const char* prefix);

/* Mixed plans: how the last factorisation was obtained (see
 * ttg_solve_report.remedy); -1 for a NULL plan. */
int32_t ttg_chol_plan_remedy(const ttg_chol_plan* plan);

/* Per-kind device busy time (ms) of the last run (needs ctx trace). */
ttg_status ttg_chol_plan_kind_times(ttg_chol_plan* plan, double* potrf_ms, double* trsm_ms, double* gemm_ms, double* accu_ms);
/* Per-task record of the last factorisation run on a context created with
 * opts.trace: one CSV line "name,start_ns,end_ns,worker,busy_ns" per device
 * task: the task name of the captured Taskflow (e.g. "POTRF_3"), first start
 * and release times relative to the earliest start, the releasing worker, and
 * the task's part durations added up.  The timeline view of the reference's Logger output
 * (tasktorrent/src/util.hpp Logger, written by 2d_cholesky with -log). */
ttg_status ttg_chol_plan_trace_dump(ttg_chol_plan* plan, const char* path);
/* The last factorisation in the reference's trace formats, as 2d_cholesky
 * writes them with --log and --depslog (2d_cholesky.cpp:630-644; read by
 * tools/ttor_logging.py:11-25): log_path gets the Logger CSV, one line
 * "<thread>>run><task>,<start s>,<end s>" per task (util.cpp Logger output;
 * the thread is the executor block, "Wk_Chol_0_<block>"), deps_path the
 * DepsLogger CSV, one line "<task>,<successor>" per dependency.  Either path
 * may be NULL.  The log needs a context created with opts.trace. */
ttg_status ttg_chol_plan_write_log(ttg_chol_plan* plan, const char* log_path, const char* deps_path);

/* ------------------------------------------------------------------ solve */

/* Solve A X = B with the plan's factor.  FP64 plan: X = L⁻ᵀL⁻¹B (block
 * sweeps with inverted diagonal tiles).  Mixed plan: GMRES-based iterative
 * refinement preconditioned by the low-precision factor, with the residual
 * r = B − A X and the update X += D in FP64, until the backward error
 * ‖b − A x‖∞ / (‖A‖∞ ‖x‖∞) of every column is ≤ tol. */
typedef struct ttg_solve_opts {
    int32_t nrhs;       /* right-hand sides, 1..16                                     */
    double tol;         /* target backward error (0 = 1e-14)                           */
    int32_t max_outer;  /* refinement steps (0 = 10)                                   */
    int32_t restart;    /* GMRES iterations per step (0 = 20, at most 60)              */
    int32_t gmres_prec; /* 0 auto (FP32 Krylov work, FP64 once FP32 stalls), 32, 64    */
    double inner_tol;   /* relative GMRES tolerance per step (0 = 1e-5)                */
    int32_t residual;   /* products with A in the refinement: 0 auto (sliced for N >= 256),
                           1 FP64 FMA (and double-float steering of early FP32 steps),
                           2 sliced: FP64-accurate on the BF16 tensor cores
                           (ttg_sliced_matmul), also for the FP64 Krylov operator    */
    int32_t refine;     /* mixed plans: 0 auto — classic steps x += M⁻¹ r while each
                           gains 10×, then GMRES; 1 GMRES from the first step        */
} ttg_solve_opts;

typedef struct ttg_solve_report {
    int32_t status;     /* TTG_OK or TTG_ENOCONV                                       */
    int32_t outer;      /* refinement steps taken                                      */
    int32_t inner;      /* GMRES iterations, all steps                                 */
    int32_t gmres_prec; /* precision of the last GMRES cycle (32 or 64)                */
    double bwd_err;     /* max over columns of ‖b − A x‖∞ / (‖A‖∞ ‖x‖∞), FP64          */
    double anorm_inf;   /* ‖A‖∞                                                        */
    double factor_ms;   /* factorisation (device events; 0 for ttg_chol_plan_solve)     */
    double solve_ms;    /* solve and refinement (host clock)                           */
    int32_t remedy;     /* mixed factor: 0 BF16 updates, 5 split-FP16 updates; after a
                           loss of definiteness 4 split-BF16 updates, 2 FP32 updates,
                           3 FP32 updates on A + 16·2^-24·diag(A), 1 BF16 updates on
                           A + 8·2^-8·diag(A); 4 also after a split-FP16 factor whose
                           first refinement step gained < 10x (ttg_chol_posv*)     */
    double h2d_ms;      /* ttg_chol_posv_host / ttg_chol_solve_host: host-to-device copies
                           of the tiles and B (device events; 0 elsewhere)             */
    double d2h_ms;      /* ... the device-to-host copy of X                             */
    double compute_ms;  /* ... from the end of the input copies to the start of the
                           output copy: factorisation, solve, refinement (events)      */
    double total_ms;    /* ... whole call, host clock                                   */
} ttg_solve_report;

/* d_B, d_X: device N×nrhs column-major (ld N). */
ttg_status ttg_chol_plan_solve(ttg_chol_plan* plan, const double* d_B, double* d_X, const ttg_solve_opts* opts,
                               ttg_solve_report* rep, void* stream);
/* Time to solution on the resident input: restore, factor, solve. */
ttg_status ttg_chol_posv(ttg_chol_plan* plan, const double* d_B, double* d_X, const ttg_solve_opts* opts,
                         ttg_solve_report* rep, void* stream);
/* Solve with the resident factor (no factorisation), host B in, host X out. */
ttg_status ttg_chol_solve_host(ttg_chol_plan* plan, const double* h_B, double* h_X, const ttg_solve_opts* opts,
                               ttg_solve_report* rep, void* stream);
/* End to end with host buffers: h_tiles (packed lower tiles of A, or NULL to
 * keep the resident input), h_B in, h_X out (N×nrhs column-major). */
ttg_status ttg_chol_posv_host(ttg_chol_plan* plan, const double* h_tiles, const double* h_B, double* h_X,
                              const ttg_solve_opts* opts, ttg_solve_report* rep, void* stream);
/* The FP32 high/low split of FP64 values that the mixed solver's dense
 * copies use (hi = fl32(v), lo = fl32(v - hi), bit for bit), computed on the
 * host by the same source as the device kernels: n values of v -> hi, lo. */
ttg_status ttg_split_f64_f32(const double* v, int64_t n, float* hi, float* lo);

/* Y = Aᵀ·X (mode 0) or Y = B − Aᵀ·X (mode 2) with FP64 accuracy on the BF16
 * tensor cores; for the symmetric matrices of the solver Aᵀ·X = A·X.  d_A:
 * dense N×N column-major FP64; d_X, d_B, d_Y: N×nrhs column-major (ld N),
 * nrhs 1..16; all device pointers.  Each column of A is scaled by its largest
 * magnitude and cut into eight signed base-256 digits (BF16 integers), each
 * column of X likewise; the digit products are summed exactly (integer
 * partial sums below 2^24 in the FP32 accumulator, int64 across K), and only
 * the final combination of the eight digit groups and the scaling round in
 * FP64 (Ozaki, Ogita, Oishi, Rump, Numer. Algorithms 59, 2012).  Allocates
 * its workspace (16·N² bytes of digits) for the call.  Replaces the
 * cblas_dgemv/dgemm products of the solve check, 2d_cholesky.cpp:646-689. */
ttg_status ttg_sliced_matmul(ttg_ctx* ctx, int32_t N, const double* d_A, int32_t nrhs, const double* d_X, const double* d_B,
                             double* d_Y, int32_t mode, void* stream);

/* Arguments of 2d_gemm (2d_gemm.cpp:243-253) at one rank. */
typedef struct ttg_gemm_args {
    int32_t n_threads;
    int32_t verb;
    int32_t block_size;
    int32_t matrix_size;
    int32_t inputs;           /* 0: val_global (gemm_shared.hpp:74-76); 1: U[-1,1] from seed */
    uint32_t seed;
} ttg_gemm_args;

typedef struct ttg_gemm_plan ttg_gemm_plan;

ttg_status ttg_gemm_plan_create(ttg_ctx* ctx, const ttg_gemm_args* args, ttg_gemm_plan** plan);
ttg_status ttg_gemm_plan_destroy(ttg_gemm_plan* plan);
int32_t ttg_gemm_plan_tasks(const ttg_gemm_plan* plan, double* capture_s);
/* Zero C and run the task graph once. */
ttg_status ttg_gemm_plan_run(ttg_gemm_plan* plan, void* stream, ttg_report* rep);
/* End-to-end: host A and B in, C = A·B out (dense N×N column-major). */
ttg_status ttg_gemm_host(ttg_gemm_plan* plan, const double* h_A, const double* h_B, double* h_C, void* stream, ttg_report* rep);
ttg_status ttg_gemm_plan_get_C(ttg_gemm_plan* plan, double* h_C);
ttg_status ttg_gemm_plan_dump_dag(ttg_gemm_plan* plan, const char* prefix);
/* Capture the block GEMM task graph on the host only and write its DAG record. */
ttg_status ttg_gemm_dag_dump(const ttg_gemm_args* args, const char* prefix);

#ifdef __cplusplus
}
#endif

#endif
