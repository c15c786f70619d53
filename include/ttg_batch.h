/* ttg_batch.h — many independent SPD factor-and-solve systems in one launch
 * of the persistent executor (GB300 extension; the reference runs one tiled
 * Cholesky per miniapp invocation, 2d_cholesky.cpp:281-616).
 *
 * Every system i gets the tiled Cholesky DAG of the reference's 2d_cholesky
 * (potrf / trsm / gemm flows with their indegrees, accumulate = false) over
 * its own tiles, followed by the block triangular solves of its right-hand
 * sides; the DAGs of all systems are concatenated into one device graph and
 * run by one launch, recorded once into a CUDA graph and replayed.
 *   TTG_PREC_F64:   FP64 factor and FP64 solve.
 *   TTG_PREC_MIXED: FP32 working tiles (FP64 diagonal POTRF, FP32 TRSM and
 *                   updates), an FP32 solve, then ir_steps rounds of iterative
 *                   refinement inside the same launch: r = b − A·x with the
 *                   FP64 input tiles, d = (L̃L̃ᵀ)⁻¹ r in FP32, x += d in FP64.
 * Right-hand sides are stored as nrhs × N_i row blocks (ld nrhs), so the
 * solve tasks are the row-vector TRSM_RLTN / GEMM_NT / GEMM_NN / TRSM_RLNN
 * operations of the executor. */
#ifndef TTG_BATCH_H
#define TTG_BATCH_H

#include <stdint.h>

#include "ttg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ttg_batch ttg_batch;

typedef struct ttg_batch_args {
    int32_t n_systems;
    const int32_t* sizes;  /* N_i (host, n_systems entries, each 1..131072)               */
    int32_t tile;          /* tile size (>= 1); each system has ceil(N_i / tile) tiles,
                              the last one ragged                                          */
    int32_t precision;     /* TTG_PREC_F64, or TTG_PREC_MIXED: FP32 factor with FP64
                              diagonal POTRFs, split-BF16 tensor-core updates for systems
                              with tile 128..512 and N > tile, FP32 ones otherwise       */
    int32_t nrhs;          /* right-hand sides per system, 1..16                          */
    int32_t ir_steps;      /* TTG_PREC_MIXED: refinement rounds inside the launch (>= 0) */
    uint32_t seed;         /* system i: A_i = G_i·G_iᵀ/N_i + alpha·I with the quantised
                              Gaussian G_i of seed + i (ttg_gen_gram_tiles), b_i iid
                              N(0,1) from (seed + i, stream 1)                            */
    double alpha;
    int32_t priority;      /* 0: longest remaining path (ttg_critical_path_priority);
                              1: none (FIFO)                                             */
} ttg_batch_args;

typedef struct ttg_batch_report {
    ttg_report run;  /* the executor run; run.elapsed_ms is the replayed CUDA graph
                        (restore copies + executor run)                              */
    int64_t tasks;   /* tasks in the device graph                                    */
    double flops;    /* Σ N_i³/3 (the factorisations' algorithmic work)              */
} ttg_batch_report;

/* Allocates the tiles and vectors of every system and uploads the graph to
 * ctx (replacing the context's graph; ttg_batch_run uploads it again if
 * another graph took its place). */
ttg_status ttg_batch_create(ttg_ctx* ctx, const ttg_batch_args* args, ttg_batch** out);
void ttg_batch_destroy(ttg_batch* b);

/* Generate A_i and b_i of every system as described at seed/alpha. */
ttg_status ttg_batch_generate(ttg_batch* b, void* stream);

/* Set system i from host data: A (N_i × N_i column-major, lower triangle
 * read) and B (N_i × nrhs column-major), or NULL to keep either. */
ttg_status ttg_batch_set_system(ttg_batch* b, int32_t i, const double* h_A, const double* h_B, void* stream);

/* Factor and solve every system: one replay of the recorded CUDA graph
 * (restore the working tiles and vectors from the inputs, run the executor),
 * then wait.  Safe to call repeatedly; each run starts from the inputs.
 * stream: a created stream (the graph is recorded on it), or NULL for the
 * batch's own stream. */
ttg_status ttg_batch_run(ttg_batch* b, void* stream, ttg_batch_report* rep);

/* Solution of system i (N_i × nrhs column-major) after a run. */
ttg_status ttg_batch_get_x(ttg_batch* b, int32_t i, double* h_X);

/* Per system, max over its columns of ‖b − A x‖∞ / (‖A‖∞ ‖x‖∞) with the FP64
 * input A (h_err: n_systems entries). */
ttg_status ttg_batch_backward_errors(ttg_batch* b, double* h_err, void* stream);

/* Autotuner: time the batch (a sample of at most max_sample systems, taken
 * evenly over the list) for every tile size in tiles[0..n_tiles) and every
 * worker count in workers[0..n_workers) (0 = all resident blocks), two runs
 * each after a warm-up, and return the fastest pair and its time per system
 * (ms).  ctx's worker count is left at the best value. */
ttg_status ttg_batch_autotune(ttg_ctx* ctx, const ttg_batch_args* args, const int32_t* tiles, int32_t n_tiles,
                              const int32_t* workers, int32_t n_workers, int32_t max_sample, int32_t* best_tile,
                              int32_t* best_workers, double* best_ms_per_system);

#ifdef __cplusplus
}
#endif

#endif /* TTG_BATCH_H */
