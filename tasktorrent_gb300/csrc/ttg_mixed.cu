// ttg_mixed.cu — mixed-precision tile path of the executor.
#include <cuda_runtime.h>

#include "../../include/ttg.h"
#include "exec.cuh"
#include "ttg_internal.h"

ttg_status ttg_mixed_init(ttg_ctx* c) {
    (void)c;
    return TTG_OK;
}

void ttg_mixed_free(ttg_ctx* c) { (void)c; }

ttg_status ttg_launch_mixed(ttg_ctx* c, const ttg::ExecParams& p, cudaStream_t s) {
    (void)c;
    (void)p;
    (void)s;
    return TTG_EINVAL;
}

#include <stdexcept>

#include "ttg_mixed_api.h"

struct ttg_mixed_state {
    int unused;
};

ttg_status ttg_mixed_state_create(ttg_ctx*, int, int, const int*, const int64_t*, double*, int, ttg_mixed_state** out) {
    *out = nullptr;
    return TTG_EINVAL;
}
void ttg_mixed_state_destroy(ttg_mixed_state* m) { delete m; }
void ttg_mixed_record_potrf(ttg_mixed_state*, int) { throw std::logic_error("mixed path not built"); }
void ttg_mixed_record_trsm(ttg_mixed_state*, int, int) { throw std::logic_error("mixed path not built"); }
void ttg_mixed_record_update(ttg_mixed_state*, int, int, int) { throw std::logic_error("mixed path not built"); }
ttg_status ttg_mixed_prepare(ttg_mixed_state*, void*) { return TTG_EINVAL; }
const double* ttg_mixed_factor_tiles(ttg_mixed_state*) { return nullptr; }
