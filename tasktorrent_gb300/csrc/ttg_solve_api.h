// ttg_solve_api.h — solver state attached to a Cholesky plan (ttg_solve.cu),
// used by apps.cpp.  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ttg.h"
#include "../../include/ttg_apps.h"

struct ttg_solver;

ttg_status ttg_solver_create(ttg_ctx* ctx, int N, int nb, const int* bs, const int64_t* off, bool mixed, ttg_solver** out);
void ttg_solver_destroy(ttg_solver* S);
// The plan's input changed: rebuild the dense copies on the next solve.
void ttg_solver_input_changed(ttg_solver* S);
// A new factor is in L64 (FP64 plan) or L32 (mixed plan): invert its diagonal tiles.
ttg_status ttg_solver_factor_done(ttg_solver* S, const double* L64, const float* L32, cudaStream_t s);
// Solve with the current factor (see ttg_chol_plan_solve).  With
// weak_first_step set, a mixed solve whose first classic refinement step
// gains less than 10× stops there and sets *weak_first_step (the caller
// replaces the factor by a more accurate one and solves again).
ttg_status ttg_solver_solve(ttg_solver* S, const double* pristine, const double* L64, const float* L32, const double* d_B,
                            double* d_X, const ttg_solve_opts* o, ttg_solve_report* rep, cudaStream_t s,
                            bool* weak_first_step = nullptr);
