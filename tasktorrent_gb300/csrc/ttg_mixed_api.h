// ttg_mixed_api.h — host interface of the mixed-precision Cholesky path,
// used by the Cholesky plan (apps.cpp).  Not part of the public ABI.
#pragma once
#include <stdint.h>

#include "../../include/ttg.h"

struct ttg_mixed_state;

ttg_status ttg_mixed_state_create(ttg_ctx* ctx, int N, int nb, const int* bs, const int64_t* off, double* tiles, int kind,
                                  ttg_mixed_state** out);
void ttg_mixed_state_destroy(ttg_mixed_state* m);
// Record the mixed-precision tile operation of a task into the running task.
void ttg_mixed_record_potrf(ttg_mixed_state* m, int j);
void ttg_mixed_record_trsm(ttg_mixed_state* m, int i, int j);
void ttg_mixed_record_update(ttg_mixed_state* m, int k, int i, int j);
// Convert the FP64 input tiles to the working precision before a run.
ttg_status ttg_mixed_prepare(ttg_mixed_state* m, void* stream);
// FP64 tiles holding the low-precision factor after a run.
const double* ttg_mixed_factor_tiles(ttg_mixed_state* m);
