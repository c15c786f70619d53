/* ttg_serve.h — a request loop for factor-and-solve requests of mixed sizes
 * (GB300 extension; the reference has no serving layer).
 *
 * Requests arrive as a Poisson stream (simulated in real time: each request
 * has an arrival time, and its latency runs from that time to the moment the
 * loop sees its result).  A request either factors and solves a new SPD
 * system A = G·Gᵀ/N + α·I (ttg_gen_gram_tiles, N log-uniform), or solves a
 * new right-hand side with the resident factor of an earlier request.
 * Continuous batching: the GPU is shared by `lanes` executors (each with
 * sms/lanes persistent blocks, launched on its own stream); whenever a lane
 * is free, the waiting requests that fit the HBM budget form its next launch
 * (the concatenated DAGs of ttg_batch.h), so requests that arrive while
 * others run start as soon as a lane and memory free up, and work of several
 * launches overlaps on the device.  Factors stay resident until the budget
 * needs their memory (least recently used first); a follow-up whose factor
 * was evicted factors its matrix again (counted as a miss).
 * Every request's backward error ‖b − A x‖∞ / (‖A‖∞ ‖x‖∞) is measured on the
 * device; a mixed request above tol runs again with twice the refinement
 * rounds.  Each request's result is the same alone and in the mix: its DAG
 * and arithmetic do not depend on what shares the launch. */
#ifndef TTG_SERVE_H
#define TTG_SERVE_H

#include <stdint.h>

#include "ttg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ttg_serve ttg_serve;

typedef struct ttg_serve_args {
    int32_t n_requests;
    double rate;            /* Poisson arrival rate (requests/s)                            */
    int32_t n_min, n_max;   /* N log-uniform in [n_min, n_max]                              */
    double alpha;
    uint32_t seed;          /* request i: arrival, size and kind from (seed, i); its matrix
                               from seed + (i, or the request whose factor it reuses); its
                               right-hand sides from (seed + i, stream 1)                   */
    double followup_frac;   /* share of follow-up right-hand sides on an earlier factor     */
    int32_t precision;      /* TTG_PREC_F64: FP64 factor + solve; TTG_PREC_MIXED: FP32
                               factor (FP64 diagonal POTRF; split-BF16 tensor-core updates
                               when the tile is 128..512 and N > tile) + FP64-residual
                               refinement                                                   */
    int32_t ir_steps;       /* mixed: refinement rounds of a first attempt                  */
    int32_t nrhs;           /* right-hand sides per request, 1..16                          */
    int32_t lanes;          /* executors sharing the GPU (>= 1)                              */
    int32_t max_batch;      /* requests per launch                                          */
    double hbm_budget_gb;   /* resident factors + requests in flight                        */
    double tol;             /* backward-error target                                        */
    int32_t keep_results;   /* keep every solution for ttg_serve_get_x                      */
    int32_t admission;      /* 0: a lane takes waiting requests when its launch ends (one
                               launch per batch of requests); 1 (mixed only, else
                               TTG_EINVAL): open lanes — each
                               lane's executor keeps running and takes a request's tasks as
                               soon as they are published, between other tasks; the lanes
                               leave half the SMs to the input generators and backward
                               errors (env TTG_SERVE_SPARE_SMS sets the count).  On the
                               synthetic stream mode 0 is faster (the generators need the
                               whole GPU between launches)                                  */
} ttg_serve_args;

typedef struct ttg_serve_report {
    int32_t completed, factorisations, followups, followup_misses, evictions, launches, retries, unconverged;
    double wall_s;                             /* first arrival to last completion           */
    double p50_ms, p99_ms, mean_ms, max_ms;    /* request latency                            */
    double solves_per_s;                       /* completed requests / wall_s                */
    double tflops;                             /* Σ factorisation N³/3 / wall_s               */
    double worst_bwd_err;
    double peak_gb;                            /* peak of resident + in-flight memory          */
} ttg_serve_report;

/* Tile size the loop uses for a system of size N. */
int32_t ttg_serve_tile(int32_t n);

ttg_status ttg_serve_create(int device, const ttg_serve_args* args, ttg_serve** out);
void ttg_serve_destroy(ttg_serve* s);

/* Run the whole stream; h_latency_ms (n_requests entries, or NULL) gets each
 * request's latency. */
ttg_status ttg_serve_run(ttg_serve* s, ttg_serve_report* rep, double* h_latency_ms);

/* Request i as generated: its size, tile, matrix seed, right-hand-side seed,
 * arrival time (s), the request whose factor it reuses (-1 for a new system),
 * and after a run its backward error and the refinement rounds of its last
 * attempt.  Any output pointer may be NULL. */
ttg_status ttg_serve_request(const ttg_serve* s, int32_t i, int32_t* n, int32_t* tile, uint32_t* seed_a, uint32_t* seed_b,
                             double* arrival_s, int32_t* followup_of, double* bwd_err, int32_t* ir_steps);

/* Solution of request i (N × nrhs column-major) after a run with keep_results. */
ttg_status ttg_serve_get_x(const ttg_serve* s, int32_t i, double* h_X);

#ifdef __cplusplus
}
#endif

#endif /* TTG_SERVE_H */
