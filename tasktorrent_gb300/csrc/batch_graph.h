// batch_graph.h — device task graphs of independent SPD factor-and-solve
// systems, shared by the batched path (ttg_batch.cu) and the serving loop
// (ttg_serve.cu).  Host code only.
//
// Per system it is the DAG of the reference's 2d_cholesky flows with
// accumulate = false (2d_cholesky.cpp:316-551):
//   potrf(j)      indegree 1                 -> trsm(i,j), i > j
//   trsm(i,j)     indegree 1 + (j > 0)        -> gemm{j,i,m} (j<m<i), gemm{j,m,i} (m>=i)
//   gemm{k,i,j}   indegree (i==j ? 1 : 2) + (k > 0)
//                 -> gemm{k+1,i,j} if k < j-1, else potrf(i) if i == j, else trsm(i,j)
// followed by the block solves of its right-hand sides (row blocks, ld nrhs):
//   forward   fs(i) = TRSM_RLTN on block i after fu(i,i-1) and potrf(i);
//             fu(i,j) = GEMM_NT  X_i -= X_j·L_ijᵀ, chained over j = 0..i-1;
//   backward  bs(i) = TRSM_RLNN on block i after bu(i,i+1) (or fs(nb-1));
//             bu(i,j) = GEMM_NN  X_i -= X_j·L_ji, chained over j = nb-1..i+1.
// fs(nb-1) depends, through the forward chains, on every forward task, so no
// backward update overwrites a block that a forward update still reads.
// Every block's updates are chained in a fixed order, so each system's
// result is the same whatever else shares the launch.
// Mixed systems convert the FP64 input tiles to FP32 working tiles with
// CONVERT tasks, factor them (FP64 diagonal POTRF through an FP64 scratch
// tile, FP32 TRSM and updates), solve in FP32, and run ir_steps rounds of
// refinement: r = b − A·x (FP64 input tiles, row-vector GEMMs chained over
// the tile row), d = (L̃L̃ᵀ)⁻¹ r in FP32, x += d.
// A system whose factor is already in its tiles (a resident factor) gets the
// solve and refinement tasks only.
#pragma once
#include <stdint.h>

#include <utility>
#include <vector>

#include "../../include/ttg.h"

namespace ttg {
namespace batch {

struct System {
    int N = 0, nb = 0, tile = 0;
    bool mixed = false;      // FP32 factor + refinement, else FP64 factor + solve
    bool factored = false;   // the tiles already hold the factor: solve only
    int ir_steps = 0;        // mixed: refinement rounds
    int nrhs = 1;
    int potrf_parts = 0;     // blocks per diagonal POTRF (0: the executor's team rule)
    // Mixed systems with tensor-core updates (split BF16): the device tables
    // of ttg_mixed_tc_header (null: FP32 updates on the CUDA cores).
    void* tc_tables = nullptr;
    // Device arrays of the system.
    double* A64 = nullptr;   // FP64 input tiles (packed lower, full diagonal tiles)
    double* W64 = nullptr;   // FP64: factor tiles
    double* D64 = nullptr;   // mixed: FP64 scratch of the diagonal POTRFs, tile² per block row
    float* W32 = nullptr;    // mixed: FP32 factor tiles
    double* B = nullptr;     // nrhs × N row blocks (ld nrhs)
    double* X = nullptr;
    double* R = nullptr;     // mixed: residual
    float* D32 = nullptr;    // mixed: FP32 correction
    void set_size(int n, int t) {
        N = n;
        tile = t < n ? t : n;
        nb = (N + tile - 1) / tile;
    }
    int bs(int i) const { return i < nb - 1 ? tile : N - (nb - 1) * tile; }
    // Tensor-core panel slot of lower tile (i, j): column-major over the lower tiles.
    int slot(int i, int j) const { return j * nb - j * (j - 1) / 2 + (i - j); }
    // Tensor-core updates apply: tiles a multiple of 128 up to 512, and updates to do.
    static bool tc_fits(int n, int t) { return t % 128 == 0 && t <= 512 && n > t; }
    int displ(int i) const { return i * tile; }
    // Packed lower tiles, column by column: tile (i, j), i >= j.  Tile
    // columns c < j are full width (c < nb - 1) with N − c·tile rows.
    int64_t off(int i, int j) const {
        return (int64_t)tile * ((int64_t)j * N - (int64_t)tile * j * (j - 1) / 2) + (int64_t)(i - j) * tile * bs(j);
    }
    int64_t elems() const { return off(nb - 1, nb - 1) + (int64_t)bs(nb - 1) * bs(nb - 1); }
    double flops() const { return (double)N * N * N / 3.0; }
};

// A device graph under construction.
struct Graph {
    std::vector<ttg_op> ops;
    std::vector<std::pair<int32_t, int32_t>> edges;
    // Finished form (finish()).
    std::vector<int32_t> init;
    std::vector<int64_t> ptr;
    std::vector<int32_t> idx;
    std::vector<double> prio;
    int add(const ttg_op& op) {
        ops.push_back(op);
        return (int)ops.size() - 1;
    }
    void edge(int a, int b) { edges.emplace_back(a, b); }
    void clear() {
        ops.clear();
        edges.clear();
        init.clear();
        ptr.clear();
        idx.clear();
        prio.clear();
    }
    // Indegrees, CSR successors and priorities (critical path, or none).
    ttg_status finish(bool critical_path);
    ttg_graph_desc desc() {
        ttg_graph_desc d{};
        d.n_tasks = (int32_t)ops.size();
        d.ops = ops.data();
        d.init_count = init.data();
        d.priority = prio.data();
        d.succ_ptr = ptr.data();
        d.succ_idx = idx.data();
        return d;
    }
};

// Append the tasks of one system.
void add_system(Graph& g, const System& S);

}  // namespace batch
}  // namespace ttg
