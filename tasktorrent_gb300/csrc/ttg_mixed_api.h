// ttg_mixed_api.h — host interface of the mixed-precision Cholesky path,
// used by the Cholesky plan (apps.cpp).  Not part of the public ABI.
//
// Working data of one mixed factorisation: an FP32 copy of the packed lower
// tiles (the trailing updates accumulate there in FP32), BF16 copies of the
// factored panel tiles with one power-of-two scale per tile (operands of the
// tensor-core updates), and the FP64 tiles of the plan used as scratch for the
// FP64 diagonal POTRF.
#pragma once
#include <cuda_bf16.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/ttg.h"

struct ttg_mixed_state;

// Trailing-update arithmetic of a mixed graph: FP32 on the CUDA cores, BF16
// on the tensor cores, or split BF16 (three BF16 slices per operand, six
// products, FP32-level accuracy) on the tensor cores.
// Split FP16: two FP16 slices (hi, and the remainder scaled by 2^11), three
// products, ~22-bit updates.
enum { TTG_UPD_FP32 = 0, TTG_UPD_BF16 = 1, TTG_UPD_BF16X3 = 2, TTG_UPD_F16X2 = 3 };

// kind: 0 = tensor-core updates available (BF16 and split BF16), 1 = FP32 updates only.
ttg_status ttg_mixed_state_create(ttg_ctx* ctx, int N, int nb, const int* bs, const int64_t* off, double* tiles64, int kind,
                                  ttg_mixed_state** out);
void ttg_mixed_state_destroy(ttg_mixed_state* m);
// Whether the state has the tensor-core variants (kind 0).
bool ttg_mixed_has_tc(const ttg_mixed_state* m);
// Tile operations of the three task kinds with update arithmetic upd
// (TTG_UPD_*; the tensor-core ones need a kind 0 state, else FP32).
ttg_op ttg_mixed_potrf_op(ttg_mixed_state* m, int j, int upd);
ttg_op ttg_mixed_trsm_op(ttg_mixed_state* m, int i, int j, int upd);
ttg_op ttg_mixed_update_op(ttg_mixed_state* m, int k, int i, int j, int upd);
// Convert the FP64 input tiles src (the plan's input, same layout as
// tiles64, which the factorisation only uses as FP64 scratch) to the FP32
// working tiles, adding shift·|a_ii| to every diagonal entry (shift 0: none),
// for a run with update arithmetic upd.
// in_graph: the run's graph converts the input itself (input tasks of
// ttg_mixed_input_op, no shift); only the block-row scales are computed here.
ttg_status ttg_mixed_prepare(ttg_mixed_state* m, void* stream, double shift, int upd, const double* src, bool in_graph = false);

// Input tasks of a graph that converts its own input, one per tile column j:
// FP64 src tiles of the column (contiguous in the packed layout) -> FP32
// working tiles, after column j has arrived.  Arrival is signalled through
// the gate words (ttg_mixed_gate): word 0 holds the run's generation, word
// 1 + j the generation whose column j is in device memory; an input task
// waits (bounded) until they are equal.
ttg_op ttg_mixed_input_op(ttg_mixed_state* m, int j, const double* src);
uint32_t* ttg_mixed_gate(ttg_mixed_state* m);
// Open a run: a new generation in gate word 0 (enqueued on stream).
// converted: the input was converted by ttg_mixed_prepare, the input tasks
// only pass (word 0 carries a flag bit); else each waits for its column
// word to receive the generation.  Returns the generation.
uint32_t ttg_mixed_gate_begin(ttg_mixed_state* m, void* stream, bool converted);
// The low-precision factor as FP64 tiles (converted into tiles64).
const double* ttg_mixed_factor_tiles(ttg_mixed_state* m);
// The FP32 factor tiles (same layout as tiles64).
const float* ttg_mixed_factor32(ttg_mixed_state* m);

// Tensor-core updates for the systems of a batch or a serving lane (uniform
// tiles b, a multiple of 128 up to 512, except a ragged last tile row): each
// system has kTcHeaderBytes of header (its tensor map and tables, 128-byte
// aligned) and ttg_mixed_tc_slot_elems BF16 values of panel slots (three
// slices of one b×b slot per lower tile (i, j), slot j·nb − j(j−1)/2 + i − j),
// n_slots slot scales and nb block-row scales, all in device memory the
// caller owns.  The ops of such a system carry the device tables as aux
// (TRSM: ldb = slot, k = block row; GEMM/SYRK: lda, ldb = slots).
constexpr size_t kTcHeaderBytes = 256;
size_t ttg_mixed_tc_slot_elems(int b, int nb);
// Fill the host copy of a header (copied by the caller to dev_hdr); *tables
// receives the device address of its tables.
ttg_status ttg_mixed_tc_header(void* host_hdr, void* dev_hdr, __nv_bfloat16* slots, float* slot_scale, const float* rowscale, int b,
                               int nb, void** tables);
// Block-row scales (2^e >= sqrt(max |diag|) of each diagonal tile) of a list
// of tiles, before a launch that publishes slots scaled by them.
struct TcRowScaleItem {
    const double* diag;  // the diagonal tile (FP64 input)
    int bs, ld;
    float* out;
};
ttg_status ttg_mixed_row_scales(const TcRowScaleItem* d_items, int n, void* stream);
// Load the row-scale kernel now (before a persistent executor starts: with
// lazy module loading a first launch waits for the device to be idle).
ttg_status ttg_mixed_row_scales_preload();
// Whether the mixed executor of ctx sets up the tensor cores (TMEM, barriers).
void ttg_mixed_set_tc(ttg_ctx* ctx, bool on);
