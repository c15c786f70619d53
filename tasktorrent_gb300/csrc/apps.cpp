// apps.cpp — the two miniapp workloads written against the Taskflow<K>
// drop-in (include/ttg_apps.h).
//
// The task graphs are the reference's, at one rank (nprows = npcols = 1):
//   Cholesky: miniapp/dense_cholesky/2d_cholesky.cpp — block sizes (:63-104),
//     thread map (:125-130), priorities (:158-204), names (:206-217), potrf
//     (:316-361), trsm (:398-464), gemm/syrk (:469-551), accu (:556-608),
//     seeding potrf(0) (:613-615).  With one rank every active-message send is
//     skipped (dest == rank), so only the local fulfill loops remain.
//   GEMM: miniapp/gemm/2d_gemm.cpp — send_Aij (:98-120), send_Bij (:122-144),
//     gemm_Cikj (:151-168), seeding every (i,j) (:174-181).
// The flows, indegrees, keys and names must equal the reference's for the
// graph to be the same graph; the task bodies call the ttor::gpu spellings of
// the same BLAS/LAPACK routines on device tiles.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "../../include/ttg.h"
#include "../../include/ttg_apps.h"
#include "../../include/ttg_philox.h"
#include "../tasktorrent/tasktorrent.hpp"
#include "ttg_internal.h"
#include "ttg_mixed_api.h"
#include "ttg_solve_api.h"

using namespace ttor;
typedef std::array<int, 2> Key2;  // the reference's int2 (CUDA headers own that name)
typedef std::array<int, 3> Key3;  // the reference's int3

namespace {

// Block sizes of 2d_cholesky.cpp:63-104 (uniform unless upper > block).
bool cholesky_block_sizes(int block_size, int num_blocks, int upper, std::vector<int>& bs) {
    const int N = block_size * num_blocks;
    if (upper < 0) upper = block_size;
    if (upper < block_size || upper > 2 * block_size) return false;
    const int lower = 2 * block_size - upper;
    std::mt19937 gen(2020);
    std::uniform_int_distribution<> distrib(lower, upper);
    bs.assign(num_blocks, block_size);
    int n = 0;
    for (int i = 0; i < num_blocks - 1; ++i) {
        const int b = std::min(N - n, distrib(gen));
        n += b;
        bs[i] = b;
    }
    bs[num_blocks - 1] = N - n;
    return true;
}

}  // namespace

struct ttg_chol_plan {
    ttg_ctx* ctx = nullptr;
    ttg_chol_args args{};
    int N = 0, nb = 0;
    std::vector<int> bs, displ;
    std::vector<int64_t> off;
    int64_t elems = 0;
    double* tiles = nullptr;     // working tiles (factorised in place)
    double* pristine = nullptr;  // input copy
    std::unique_ptr<Threadpool_shared> tp;    // the plan's graph (FP64, or mixed with BF16 updates when available)
    std::unique_ptr<Threadpool_shared> tp32;  // mixed plans with tensor cores: the same graph with FP32 updates
    std::unique_ptr<Threadpool_shared> tpx3;  // ... and with split-BF16 updates (mixed_kind 0 and 3)
    int remedy = 0;                           // last mixed factorisation: 0 none, 1 diagonal shift, 2 FP32 updates
    std::vector<int> kind_of_dev;  // per device task: 0 potrf, 1 trsm, 2 gemm, 3 accu, -1 other
    std::vector<double*> tmp;      // accumulate-flow temporaries (device)
    ttg_mixed_state* mixed = nullptr;
    ttg_solver* solver = nullptr;
    double* d_b = nullptr;         // device B and X of ttg_chol_posv_host
    size_t host_b_elems = 0;
    cudaEvent_t host_ev[4] = {};   // phase events of the host-buffer entry points
    // Mixed plans: the first attempt's graph converts its input column by
    // column (input tasks gated on arrival), so a host input can stream in
    // while the factorisation runs.
    bool input_tasks = false;
    bool streaming = false;        // this factorisation's input is still arriving
    cudaStream_t copy_s = nullptr; // host input copies
    cudaEvent_t copy_ev[3] = {};   // start on the caller's stream, diagonal tiles in, all in
    long factor_gen = 0;   // incremented by every successful factorisation
    long solver_gen = -1;  // factorisation the solver's inverted tiles belong to
    // Frees whatever was allocated, so every early return of
    // ttg_chol_plan_create (through the owning unique_ptr) releases the
    // device tiles as ttg_chol_plan_destroy does.
    ~ttg_chol_plan() {
        if (ctx) cudaSetDevice(ctx->device);
        tp.reset();
        tp32.reset();
        tpx3.reset();
        for (double* t : tmp) cudaFree(t);
        if (tiles) cudaFree(tiles);
        if (pristine) cudaFree(pristine);
        if (mixed) ttg_mixed_state_destroy(mixed);
        if (solver) ttg_solver_destroy(solver);
        if (d_b) cudaFree(d_b);
        for (cudaEvent_t e : host_ev)
            if (e) cudaEventDestroy(e);
        for (cudaEvent_t e : copy_ev)
            if (e) cudaEventDestroy(e);
        if (copy_s) cudaStreamDestroy(copy_s);
    }
};

static ttg_status chol_build_graph(ttg_chol_plan* P, bool dry, int upd, std::unique_ptr<Threadpool_shared>& tp_out) {
    const ttg_chol_args& a = P->args;
    const int nb = P->nb, n_threads = a.n_threads;
    const bool accumulate = a.accumulate != 0;
    // kind 4 (extension): capture with the kind-3 priorities, then replace
    // them by the longest remaining path of each device task.  kind 5
    // (extension): look-ahead — three levels, the POTRFs, then the TRSMs and
    // the updates of the next panel column (GEMM (k, i, k+1)), then the other
    // updates; within a level tasks run in the order they become ready.
    // kind 6 (extension): the critical chain above everything else — the
    // tasks of the tiles within two of the diagonal (POTRF(j), TRSM(j+1, j),
    // TRSM(j+2, j) and every update of the tiles (j, j), (j+1, j), (j+2, j))
    // at 9nb + 9(nb-j), the other TRSMs and updates of column j at kind 2's
    // 9(nb-j)-2 — so a chain task never queues behind the bulk of a column
    // (kind 2 ranks the next diagonal tile's update below the current
    // column's TRSMs).  2nb distinct values: 128 levels for 64 tile columns.
    const int pk = a.kind == 4 ? 3 : a.kind;
    const bool mixed = a.precision == TTG_PREC_MIXED;
    auto block = [P](int i, int j) { return P->tiles + P->off[i + (size_t)j * P->nb]; };
    auto lda = [P](int i) { return std::max(1, P->bs[i]); };
    auto block_2_thread = [=](int i, int j) { return (i + j * nb) % n_threads; };

    auto potf_block_2_prio = [=](int j) -> double {
        if (pk == 5) return 3.0;
        if (pk == 3) return (double)(9 * (nb - j) - 1) + 18 * nb * nb;
        if (pk == 2) return (double)(9 * (nb - j) - 1);
        if (pk == 6) return (double)(9 * nb + 9 * (nb - j));
        if (pk == 1) return 3.0 * (double)(nb - j);
        return 3.0;
    };
    auto trsm_block_2_prio = [=](Key2 ij) -> double {
        if (pk == 5) return 2.0;
        if (pk == 3) return (double)((nb - ij[0]) + nb * (9.0 * nb - 9.0 * ij[1] - 2.0) + 9 * nb * nb);
        if (pk == 2) return (double)(9 * (nb - ij[1]) - 2);
        if (pk == 6) return ij[0] <= ij[1] + 2 ? (double)(9 * nb + 9 * (nb - ij[1])) : (double)(9 * (nb - ij[1]) - 2);
        if (pk == 1) return 2.0 * (double)(nb - ij[0]);
        return 2.0;
    };
    auto gemm_block_2_prio = [=](Key3 kij) -> double {
        if (pk == 5) return kij[2] == kij[0] + 1 ? 2.0 : 1.0;
        if (pk == 3) {
            if (accumulate) return (double)(nb - kij[1]) + nb * (9.0 * nb - 9.0 * kij[2] - 2.0);
            return (double)(nb - kij[1]) + nb * (9.0 * nb - 3.0 * kij[2] - 6.0 * kij[0] - 2.0);
        }
        if (pk == 2) return (double)(9 * nb - 9 * kij[2] - 2);
        if (pk == 6) return kij[1] <= kij[2] + 2 ? (double)(9 * nb + 9 * (nb - kij[2])) : (double)(9 * (nb - kij[2]) - 2);
        if (pk == 1) return (double)(nb - kij[1]);
        return 1.0;
    };

    // Accumulation temporaries: one per (k, i, j) gemm of the accumulate flow.
    std::map<std::array<int, 3>, double*> tmp_of;
    if (accumulate) {
        for (int j = 0; j < nb; ++j)
            for (int i = j; i < nb; ++i)
                for (int k = 0; k < j; ++k) {
                    double* t = nullptr;
                    if (!dry) {
                        if (cudaMalloc((void**)&t, sizeof(double) * std::max(1, P->bs[i] * P->bs[j])) != cudaSuccess)
                            return TTG_ENOMEM;
                        P->tmp.push_back(t);
                    }
                    tmp_of[{k, i, j}] = t;
                }
    }

    tp_out.reset(new Threadpool_shared(n_threads, a.verb, "Wk_Chol_0_"));
    tp_out->set_critical_path_priority(a.kind == 4);
    Threadpool_shared& tp = *tp_out;
    if (!dry) tp.set_context(P->ctx);
    Taskflow<int> potrf(&tp, a.verb);
    Taskflow<Key2> trsm(&tp, a.verb);
    Taskflow<Key3> gemm(&tp, a.verb);
    Taskflow<Key3> accu(&tp, a.verb);

    potrf.set_task([&](int j) {
             if (mixed) gpu::record_op(ttg_mixed_potrf_op(P->mixed, j, upd));
             else gpu::LAPACKE_dpotrf(gpu::LAPACK_COL_MAJOR, 'L', P->bs[j], block(j, j), lda(j));
         })
        .set_fulfill([&](int j) {
            for (int i = j + 1; i < nb; i++) trsm.fulfill_promise({i, j});
        })
        .set_indegree([&](int j) { return accumulate ? (j == 0 ? 1 : j) : 1; })
        .set_priority(potf_block_2_prio)
        .set_mapping([&](int j) { return block_2_thread(j, j); })
        .set_name([](int j) { return "POTRF_" + std::to_string(j); });

    trsm.set_task([&](Key2 ij) {
            const int i = ij[0], j = ij[1];
            if (mixed) gpu::record_op(ttg_mixed_trsm_op(P->mixed, i, j, upd));
            else
                gpu::cblas_dtrsm(gpu::CblasColMajor, gpu::CblasRight, gpu::CblasLower, gpu::CblasTrans, gpu::CblasNonUnit,
                                 P->bs[i], P->bs[j], 1.0, block(j, j), lda(j), block(i, j), lda(i));
        })
        .set_fulfill([&](Key2 ij) {
            const int i = ij[0], j = ij[1];
            for (int k = j + 1; k < i; k++) gemm.fulfill_promise({j, i, k});
            for (int k = i; k < nb; k++) gemm.fulfill_promise({j, k, i});
        })
        .set_indegree([&](Key2 ij) { return accumulate ? 1 + ij[1] : 1 + (ij[1] == 0 ? 0 : 1); })
        .set_priority(trsm_block_2_prio)
        .set_mapping([&](Key2 ij) { return block_2_thread(ij[0], ij[1]); })
        .set_name([](Key2 ij) { return "TRSM_" + std::to_string(ij[0]) + "_" + std::to_string(ij[1]); });

    gemm.set_task([&](Key3 kij) {
            const int k = kij[0], i = kij[1], j = kij[2];
            double* C = accumulate ? tmp_of[{k, i, j}] : block(i, j);
            const double beta = accumulate ? 0.0 : 1.0;
            if (mixed) {
                gpu::record_op(ttg_mixed_update_op(P->mixed, k, i, j, upd));
            } else if (i == j) {
                gpu::cblas_dsyrk(gpu::CblasColMajor, gpu::CblasLower, gpu::CblasNoTrans, P->bs[i], P->bs[k], -1.0, block(i, k),
                                 lda(i), beta, C, lda(i));
            } else {
                gpu::cblas_dgemm(gpu::CblasColMajor, gpu::CblasNoTrans, gpu::CblasTrans, P->bs[i], P->bs[j], P->bs[k], -1.0,
                                 block(i, k), lda(i), block(j, k), lda(j), beta, C, lda(i));
            }
        })
        .set_fulfill([&](Key3 kij) {
            const int k = kij[0], i = kij[1], j = kij[2];
            if (accumulate) {
                accu.fulfill_promise(kij);
            } else if (k < j - 1) {
                gemm.fulfill_promise({k + 1, i, j});
            } else if (i == j) {
                potrf.fulfill_promise(i);
            } else {
                trsm.fulfill_promise({i, j});
            }
        })
        .set_indegree([&](Key3 kij) {
            if (accumulate) return kij[1] == kij[2] ? 1 : 2;
            return (kij[1] == kij[2] ? 1 : 2) + (kij[0] == 0 ? 0 : 1);
        })
        .set_priority(gemm_block_2_prio)
        .set_mapping([&](Key3 kij) { return block_2_thread(kij[1], kij[2]); })
        .set_binding([](Key3) { return false; })
        .set_name([](Key3 kij) {
            return "GEMM_" + std::to_string(kij[0]) + "_" + std::to_string(kij[1]) + "_" + std::to_string(kij[2]);
        });

    accu.set_task([&](Key3 kij) {
            const int k = kij[0], i = kij[1], j = kij[2];
            gpu::geadd(P->bs[i], P->bs[j], 1.0, tmp_of[{k, i, j}], lda(i), 1.0, block(i, j), lda(i));
        })
        .set_fulfill([&](Key3 kij) {
            if (kij[1] == kij[2]) potrf.fulfill_promise(kij[1]);
            else trsm.fulfill_promise({kij[1], kij[2]});
        })
        .set_indegree([](Key3) { return 1; })
        .set_mapping([&](Key3 kij) { return block_2_thread(kij[1], kij[2]); })
        .set_priority(gemm_block_2_prio)
        .set_binding([](Key3) { return true; })
        .set_name([](Key3 kij) {
            return "ACCU_" + std::to_string(kij[0]) + "_" + std::to_string(kij[1]) + "_" + std::to_string(kij[2]);
        });

    // Capture: seed potrf(0) and run the closures on the host; join() would
    // also execute on the device — here the graph is only built, the plan
    // runs it later (ttg_chol_plan_factor).
    potrf.fulfill_promise(0);
    try {
        if (dry) tp.capture_dry();
        else tp.capture_only();
    } catch (const std::exception& e) {
        fprintf(stderr, "ttg_chol_plan: %s\n", e.what());
        return TTG_EINVAL;
    }
    if (dry) return TTG_OK;
    // Kind of each device task, from the captured names' prefixes.
    const auto& nodes = tp.device_task_nodes();
    P->kind_of_dev.resize(nodes.size());
    for (size_t d = 0; d < nodes.size(); ++d) {
        const std::string nm = tp.node_name(nodes[d]);
        P->kind_of_dev[d] = nm[0] == 'P' ? 0 : nm[0] == 'T' ? 1 : nm[0] == 'G' ? 2 : nm[0] == 'A' ? 3 : -1;
    }
    return TTG_OK;
}

// The first attempt's graph of a mixed plan converts its own input: one
// input task per tile column j (FP64 plan input -> FP32 working tiles) that
// the column's first tasks wait for — POTRF_0 and TRSM_i_0 for column 0,
// GEMM_0_i_j for column j >= 1 (every later task of a tile depends on its
// first).  The input task has the highest priority among its successors'.
static ttg_status add_input_tasks(ttg_chol_plan* P) {
    Threadpool_shared& tp = *P->tp;
    const auto& nodes = tp.device_task_nodes();
    const int nb = P->nb;
    std::vector<std::vector<int>> succ(nb);
    std::vector<double> prio(nb, -1e300);
    std::vector<int> seen(tp.n_nodes(), 0);
    for (size_t d = 0; d < nodes.size(); ++d) {
        if (seen[nodes[d]]++) continue;  // the node's first device task only
        const std::string nm = tp.node_name(nodes[d]);
        int col = -1, a = 0, b = 0, c = 0;
        if (sscanf(nm.c_str(), "POTRF_%d", &a) == 1 && nm[0] == 'P') col = a == 0 ? 0 : -1;
        else if (sscanf(nm.c_str(), "TRSM_%d_%d", &a, &b) == 2) col = b == 0 ? 0 : -1;
        else if (sscanf(nm.c_str(), "GEMM_%d_%d_%d", &a, &b, &c) == 3) col = a == 0 ? c : -1;
        if (col < 0) continue;
        succ[col].push_back((int)d);
        prio[col] = std::max(prio[col], tp.device_priority((int)d));
    }
    std::vector<ttg_op> ops(nb);
    for (int j = 0; j < nb; ++j) {
        if (succ[j].empty()) return TTG_OK;  // not the expected graph: keep the separate conversion
        ops[j] = ttg_mixed_input_op(P->mixed, j, P->pristine);
    }
    try {
        tp.add_device_tasks(ops, prio, succ);
    } catch (const std::exception& e) {
        fprintf(stderr, "ttg_chol_plan: %s\n", e.what());
        return TTG_ECUDA;
    }
    P->input_tasks = true;
    return TTG_OK;
}

extern "C" ttg_status ttg_chol_plan_create(ttg_ctx* ctx, const ttg_chol_args* args, ttg_chol_plan** out) {
    if (!ctx || !args || !out) return TTG_EINVAL;
    *out = nullptr;
    if (args->block_size <= 0 || args->num_blocks <= 0 || args->n_threads <= 0) return TTG_EINVAL;
    if (args->precision != TTG_PREC_F64 && args->precision != TTG_PREC_MIXED) return TTG_EINVAL;
    if (args->precision == TTG_PREC_MIXED && args->accumulate) return TTG_EINVAL;
    if (args->precision == TTG_PREC_MIXED && (args->mixed_kind < 0 || args->mixed_kind > 3)) return TTG_EINVAL;
    std::unique_ptr<ttg_chol_plan> P(new ttg_chol_plan());
    P->ctx = ctx;
    P->args = *args;
    if (!cholesky_block_sizes(args->block_size, args->num_blocks, args->upper_block_size, P->bs)) return TTG_EINVAL;
    if (args->precision == TTG_PREC_MIXED && args->mixed_kind != 1) {
        // Tensor-core updates (mixed_kind 0, 2 and 3) need uniform tiles whose
        // size is a multiple of 128 (the MMA's M); checked before any
        // allocation.  FP32 updates (mixed_kind 1) take any tiles.
        for (int b : P->bs)
            if (b != P->bs[0]) return TTG_EINVAL;
        if (P->bs[0] % 128 != 0) return TTG_EINVAL;
    }
    P->nb = args->num_blocks;
    P->displ.assign(P->nb + 1, 0);
    for (int i = 0; i < P->nb; ++i) P->displ[i + 1] = P->displ[i] + P->bs[i];
    P->N = P->displ[P->nb];
    P->off.assign((size_t)P->nb * P->nb, 0);
    P->elems = ttg_tile_layout(P->bs.data(), P->nb, P->off.data());
    TTG_CUDA_CHECK(cudaSetDevice(ctx->device));
    TTG_CUDA_CHECK(cudaMalloc((void**)&P->tiles, sizeof(double) * std::max<int64_t>(1, P->elems)));
    TTG_CUDA_CHECK(cudaMalloc((void**)&P->pristine, sizeof(double) * std::max<int64_t>(1, P->elems)));
    if (args->precision == TTG_PREC_MIXED) {
        ttg_status s = ttg_mixed_state_create(ctx, P->N, P->nb, P->bs.data(), P->off.data(), P->tiles,
                                              args->mixed_kind == 1 ? 1 : 0, &P->mixed);
        if (s != TTG_OK) return s;
    }
    // Graphs: the first attempt's update arithmetic, then the remedies'.
    const bool tc = P->mixed && ttg_mixed_has_tc(P->mixed);
    const int first = !tc ? TTG_UPD_FP32
                          : (args->mixed_kind == 2 ? TTG_UPD_BF16X3 : (args->mixed_kind == 3 ? TTG_UPD_F16X2 : TTG_UPD_BF16));
    ttg_status s = chol_build_graph(P.get(), false, first, P->tp);
    if (s == TTG_OK && tc) s = chol_build_graph(P.get(), false, TTG_UPD_FP32, P->tp32);
    if (s == TTG_OK && tc && first != TTG_UPD_BF16X3) s = chol_build_graph(P.get(), false, TTG_UPD_BF16X3, P->tpx3);
    if (s == TTG_OK && P->mixed) s = add_input_tasks(P.get());
    if (s == TTG_OK) s = ttg_chol_plan_generate(P.get(), nullptr);
    if (s != TTG_OK) return s;  // P's destructor frees what was allocated
    *out = P.release();
    return TTG_OK;
}

// Capture the Cholesky graph without a device and write its DAG record.
extern "C" ttg_status ttg_chol_dag_dump(const ttg_chol_args* args, const char* prefix) {
    if (!args || !prefix || args->block_size <= 0 || args->num_blocks <= 0 || args->n_threads <= 0) return TTG_EINVAL;
    if (args->precision != TTG_PREC_F64) return TTG_EINVAL;
    ttg_chol_plan P;
    P.args = *args;
    if (!cholesky_block_sizes(args->block_size, args->num_blocks, args->upper_block_size, P.bs)) return TTG_EINVAL;
    P.nb = args->num_blocks;
    P.off.assign((size_t)P.nb * P.nb, 0);
    P.elems = ttg_tile_layout(P.bs.data(), P.nb, P.off.data());
    ttg_status s = chol_build_graph(&P, true, TTG_UPD_FP32, P.tp);
    if (s != TTG_OK) return s;
    P.tp->dump_dag(prefix);
    return TTG_OK;
}

extern "C" ttg_status ttg_chol_plan_destroy(ttg_chol_plan* P) {
    delete P;  // the destructor frees the device buffers
    return TTG_OK;
}

extern "C" int32_t ttg_chol_plan_n(const ttg_chol_plan* P, int32_t* h_bs) {
    if (!P) return 0;
    if (h_bs)
        for (int i = 0; i < P->nb; ++i) h_bs[i] = P->bs[i];
    return P->N;
}

extern "C" int32_t ttg_chol_plan_tasks(const ttg_chol_plan* P, double* capture_s) {
    if (!P) return 0;
    if (capture_s) *capture_s = P->tp->capture_seconds();
    return P->tp->n_device_tasks();
}

extern "C" double* ttg_chol_plan_tiles(ttg_chol_plan* P, const int64_t** h_off) {
    if (!P) return nullptr;
    if (h_off) *h_off = P->off.data();
    return P->tiles;
}

extern "C" ttg_status ttg_chol_plan_generate(ttg_chol_plan* P, void* stream) {
    if (!P) return TTG_EINVAL;
    ttg_status s;
    if (P->args.matrix == 1)
        s = ttg_gen_gram_tiles(P->ctx, P->N, P->bs.data(), P->nb, P->args.alpha, P->args.seed, P->pristine, stream);
    else
        s = ttg_gen_miniapp_tiles(P->ctx, P->bs.data(), P->nb, P->pristine, stream);
    if (s != TTG_OK) return s;
    if (P->solver) ttg_solver_input_changed(P->solver);
    return ttg_chol_plan_restore(P, stream);
}

// Copy the lower tiles of a dense host matrix into device tiles.
static ttg_status dense_to_tiles(const ttg_chol_plan* P, const double* h_A, double* d_tiles, cudaStream_t s) {
    for (int j = 0; j < P->nb; ++j)
        for (int i = j; i < P->nb; ++i) {
            if (P->bs[i] == 0 || P->bs[j] == 0) continue;
            TTG_CUDA_CHECK(cudaMemcpy2DAsync(d_tiles + P->off[i + (size_t)j * P->nb], sizeof(double) * P->bs[i],
                                             h_A + P->displ[i] + (size_t)P->displ[j] * P->N, sizeof(double) * P->N,
                                             sizeof(double) * P->bs[i], P->bs[j], cudaMemcpyHostToDevice, s));
        }
    return TTG_OK;
}

static ttg_status tiles_to_dense(const ttg_chol_plan* P, const double* d_tiles, double* h_A, cudaStream_t s) {
    for (int j = 0; j < P->nb; ++j)
        for (int i = j; i < P->nb; ++i) {
            if (P->bs[i] == 0 || P->bs[j] == 0) continue;
            TTG_CUDA_CHECK(cudaMemcpy2DAsync(h_A + P->displ[i] + (size_t)P->displ[j] * P->N, sizeof(double) * P->N,
                                             d_tiles + P->off[i + (size_t)j * P->nb], sizeof(double) * P->bs[i],
                                             sizeof(double) * P->bs[i], P->bs[j], cudaMemcpyDeviceToHost, s));
        }
    return TTG_OK;
}

extern "C" ttg_status ttg_chol_plan_set_matrix(ttg_chol_plan* P, const double* h_A, void* stream) {
    if (!P || !h_A) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(P->ctx->device));
    cudaStream_t s = (cudaStream_t)stream;
    ttg_status st = dense_to_tiles(P, h_A, P->pristine, s);
    if (st != TTG_OK) return st;
    TTG_CUDA_CHECK(cudaStreamSynchronize(s));
    if (P->solver) ttg_solver_input_changed(P->solver);
    return ttg_chol_plan_restore(P, stream);
}

extern "C" ttg_status ttg_chol_plan_restore(ttg_chol_plan* P, void* stream) {
    if (!P) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(P->ctx->device));
    TTG_CUDA_CHECK(cudaMemcpyAsync(P->tiles, P->pristine, sizeof(double) * P->elems, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
    return TTG_OK;
}

static ttg_status chol_factor_from(ttg_chol_plan* P, void* stream, ttg_report* rep, size_t first_attempt);

extern "C" ttg_status ttg_chol_plan_factor(ttg_chol_plan* P, void* stream, ttg_report* rep) {
    return chol_factor_from(P, stream, rep, 0);
}

// Factorisation starting at attempt `first_attempt` of the mixed chain.
static ttg_status chol_factor_from(ttg_chol_plan* P, void* stream, ttg_report* rep, size_t first_attempt) {
    if (!P) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(P->ctx->device));
    if (!P->mixed) {
        ttg_status s = P->tp->replay(stream);
        if (rep) *rep = P->tp->report();
        if (s == TTG_OK) ++P->factor_gen;
        return s;
    }
    // Mixed: BF16 tensor-core updates when available.  A trailing diagonal
    // block that loses positive definiteness (TTG_ENOTPD) means the update
    // precision is too low for the matrix's conditioning (BF16 rounding of
    // the panels perturbs A by about 2^-9·‖A‖): retry with split-BF16
    // tensor-core updates (FP32-level accuracy), then FP32 updates, then FP32
    // updates on A + 16·2^-24·diag(A), and last BF16 updates on A +
    // 8·2^-8·diag(A).  A shifted factor only preconditions: refinement always
    // solves the unshifted system.  Every attempt converts the plan's input
    // (pristine) afresh; the FP64 working tiles are only the diagonal POTRF's
    // scratch, so they need no restore.
    const bool tc = ttg_mixed_has_tc(P->mixed);
    const bool first_x3 = P->args.mixed_kind == 2;
    const bool first_f16 = P->args.mixed_kind == 3;
    struct Attempt {
        Threadpool_shared* tp;
        double shift;
        int upd;
        int remedy;
    };
    std::vector<Attempt> plan;
    Threadpool_shared* tp32 = tc ? P->tp32.get() : P->tp.get();
    if (tc && first_f16) plan.push_back({P->tp.get(), 0.0, TTG_UPD_F16X2, 5});
    else if (tc && !first_x3) plan.push_back({P->tp.get(), 0.0, TTG_UPD_BF16, 0});
    if (tc) plan.push_back({first_x3 ? P->tp.get() : P->tpx3.get(), 0.0, TTG_UPD_BF16X3, 4});
    plan.push_back({tp32, 0.0, TTG_UPD_FP32, 2});
    plan.push_back({tp32, 16.0 * 5.9604644775390625e-08, TTG_UPD_FP32, 3});
    if (tc && !first_x3 && !first_f16) plan.push_back({P->tp.get(), 8.0 * 0.00390625, TTG_UPD_BF16, 1});
    ttg_status s = TTG_OK;
    float total_ms = 0.f;
    const bool streamed = P->streaming;
    for (size_t a = std::min(first_attempt, plan.size() - 1); a < plan.size(); ++a) {
        // The plan's first graph converts its input in its input tasks; a
        // streamed input (ttg_chol_posv_host) opened the gate already.
        // The plan's first graph has input tasks: they convert a streamed
        // input (ttg_chol_posv_host opened the gate); for a resident input the
        // conversion kernel runs and they only pass.
        const bool graph_inputs = P->input_tasks && plan[a].tp == P->tp.get();
        const bool in_graph = graph_inputs && P->streaming;
        if (P->streaming && (!graph_inputs || plan[a].shift != 0.0)) return TTG_ESTATE;
        if (!in_graph && streamed) TTG_CUDA_CHECK(cudaStreamWaitEvent((cudaStream_t)stream, P->copy_ev[2], 0));  // all copies in
        s = ttg_mixed_prepare(P->mixed, stream, plan[a].shift, plan[a].upd, P->pristine, in_graph);
        if (s != TTG_OK) return s;
        if (graph_inputs && !in_graph) ttg_mixed_gate_begin(P->mixed, stream, true);
        P->streaming = false;  // a retry waits for the whole input
        s = plan[a].tp->replay(stream);
        const ttg_report r = plan[a].tp->report();
        total_ms += r.elapsed_ms;
        if (rep) {
            *rep = r;
            rep->elapsed_ms = total_ms;
        }
        P->remedy = plan[a].remedy;
        if (s != TTG_ENOTPD) break;
    }
    if (s == TTG_OK) ++P->factor_gen;
    return s;
}

extern "C" int32_t ttg_chol_plan_remedy(const ttg_chol_plan* P) { return P ? P->remedy : -1; }

extern "C" ttg_status ttg_chol_factor_host(ttg_chol_plan* P, const double* h_A, double* h_L, void* stream, ttg_report* rep) {
    if (!P || !h_A) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(P->ctx->device));
    cudaStream_t s = (cudaStream_t)stream;
    // The FP64 path factors the working tiles in place; the mixed path
    // factors the plan's input.
    ttg_status st = dense_to_tiles(P, h_A, P->mixed ? P->pristine : P->tiles, s);
    if (st != TTG_OK) return st;
    if (P->mixed && P->solver) ttg_solver_input_changed(P->solver);
    st = ttg_chol_plan_factor(P, stream, rep);
    if (st != TTG_OK) return st;
    if (h_L) {
        st = tiles_to_dense(P, P->mixed ? ttg_mixed_factor_tiles(P->mixed) : P->tiles, h_L, s);
        if (st != TTG_OK) return st;
        TTG_CUDA_CHECK(cudaStreamSynchronize(s));
        for (int j = 0; j < P->N; ++j) std::fill(h_L + (size_t)j * P->N, h_L + (size_t)j * P->N + j, 0.0);
    }
    return TTG_OK;
}

extern "C" int64_t ttg_chol_plan_tile_elems(const ttg_chol_plan* P) { return P ? P->elems : 0; }

extern "C" ttg_status ttg_chol_plan_copy_tiles(ttg_chol_plan* P, int32_t which, double* h_dst) {
    if (!P || !h_dst || (which != 0 && which != 1)) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(P->ctx->device));
    const double* src = which == 1 ? P->pristine : (P->mixed ? ttg_mixed_factor_tiles(P->mixed) : P->tiles);
    TTG_CUDA_CHECK(cudaMemcpy(h_dst, src, sizeof(double) * P->elems, cudaMemcpyDeviceToHost));
    return TTG_OK;
}

extern "C" ttg_status ttg_chol_factor_host_tiles(ttg_chol_plan* P, const double* h_in, double* h_out, void* stream,
                                                 ttg_report* rep) {
    if (!P || !h_in) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(P->ctx->device));
    cudaStream_t s = (cudaStream_t)stream;
    // The input becomes the plan's input (the mixed factorisation converts it
    // directly), then the FP64 working tiles are restored from it and factored.
    TTG_CUDA_CHECK(cudaMemcpyAsync(P->pristine, h_in, sizeof(double) * P->elems, cudaMemcpyHostToDevice, s));
    if (P->solver) ttg_solver_input_changed(P->solver);
    ttg_status st = P->mixed ? TTG_OK : ttg_chol_plan_restore(P, stream);
    if (st != TTG_OK) return st;
    st = ttg_chol_plan_factor(P, stream, rep);
    if (st != TTG_OK) return st;
    if (h_out) {
        const double* src = P->mixed ? ttg_mixed_factor_tiles(P->mixed) : P->tiles;
        TTG_CUDA_CHECK(cudaMemcpyAsync(h_out, src, sizeof(double) * P->elems, cudaMemcpyDeviceToHost, s));
    }
    TTG_CUDA_CHECK(cudaStreamSynchronize(s));
    return TTG_OK;
}

extern "C" ttg_status ttg_chol_plan_get_factor(ttg_chol_plan* P, double* h_L) {
    if (!P || !h_L) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(P->ctx->device));
    const double* src = P->tiles;
    if (P->mixed) src = ttg_mixed_factor_tiles(P->mixed);
    ttg_status st = tiles_to_dense(P, src, h_L, nullptr);
    if (st != TTG_OK) return st;
    TTG_CUDA_CHECK(cudaStreamSynchronize(nullptr));
    for (int j = 0; j < P->N; ++j) std::fill(h_L + (size_t)j * P->N, h_L + (size_t)j * P->N + j, 0.0);
    return TTG_OK;
}

extern "C" ttg_status ttg_chol_plan_get_input(ttg_chol_plan* P, double* h_A) {
    if (!P || !h_A) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(P->ctx->device));
    ttg_status st = tiles_to_dense(P, P->pristine, h_A, nullptr);
    if (st != TTG_OK) return st;
    TTG_CUDA_CHECK(cudaStreamSynchronize(nullptr));
    for (int j = 0; j < P->N; ++j)
        for (int i = 0; i < j; ++i) h_A[i + (size_t)j * P->N] = h_A[j + (size_t)i * P->N];
    return TTG_OK;
}

static ttg_status plan_solve(ttg_chol_plan* P, const double* d_B, double* d_X, const ttg_solve_opts* o, ttg_solve_report* rep,
                             void* stream, bool* weak_first_step) {
    if (!P || !o || !d_B || !d_X) return TTG_EINVAL;
    if (P->factor_gen == 0) return TTG_ESTATE;
    TTG_CUDA_CHECK(cudaSetDevice(P->ctx->device));
    cudaStream_t s = (cudaStream_t)stream;
    const bool mixed = P->mixed != nullptr;
    if (!P->solver) {
        ttg_status st = ttg_solver_create(P->ctx, P->N, P->nb, P->bs.data(), P->off.data(), mixed, &P->solver);
        if (st != TTG_OK) return st;
    }
    auto t0 = std::chrono::steady_clock::now();
    const float* L32 = mixed ? ttg_mixed_factor32(P->mixed) : nullptr;
    if (P->solver_gen != P->factor_gen) {
        ttg_status st = ttg_solver_factor_done(P->solver, P->tiles, L32, s);
        if (st != TTG_OK) return st;
        P->solver_gen = P->factor_gen;
        if (getenv("TTG_SOLVE_VERBOSE")) {
            cudaStreamSynchronize(s);
            fprintf(stderr, "[ttg solve] %-28s %9.3f ms\n", "invert diagonal tiles",
                    std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
        }
    }
    ttg_solve_report r{};
    ttg_status st = ttg_solver_solve(P->solver, P->pristine, P->tiles, L32, d_B, d_X, o, &r, s, weak_first_step);
    r.remedy = mixed ? P->remedy : 0;
    r.solve_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (rep) *rep = r;
    return st;
}

extern "C" ttg_status ttg_chol_plan_solve(ttg_chol_plan* P, const double* d_B, double* d_X, const ttg_solve_opts* o,
                                          ttg_solve_report* rep, void* stream) {
    return plan_solve(P, d_B, d_X, o, rep, stream, nullptr);
}

// The solve that follows a factorisation.  FP16 keeps 11 significant bits
// over a narrow exponent range, so on an ill-conditioned matrix (small
// pivots, factor entries far below their block row's scale) the split-FP16
// factor (remedy 5) preconditions poorly: when its first classic refinement
// step gains less than 10×, the plan factors again with split-BF16 updates
// (remedy 4) and solves from the start — cheaper than a long GMRES on the
// weaker preconditioner.
static ttg_status solve_after_factor(ttg_chol_plan* P, const double* d_B, double* d_X, const ttg_solve_opts* o, ttg_solve_report* r,
                                     void* stream, float factor_ms) {
    bool weak = false;
    const bool check = P->mixed && P->remedy == 5 && o->refine == 0;
    ttg_status st = plan_solve(P, d_B, d_X, o, r, stream, check ? &weak : nullptr);
    if (st == TTG_OK && weak) {
        const double first_ms = r->solve_ms;
        ttg_report fr{};
        st = chol_factor_from(P, stream, &fr, 1);  // the split-BF16 attempt
        if (st != TTG_OK) return st;
        factor_ms += fr.elapsed_ms;
        st = plan_solve(P, d_B, d_X, o, r, stream, nullptr);
        r->solve_ms += first_ms;
    }
    r->factor_ms = factor_ms;
    return st;
}

extern "C" ttg_status ttg_chol_posv(ttg_chol_plan* P, const double* d_B, double* d_X, const ttg_solve_opts* o,
                                   ttg_solve_report* rep, void* stream) {
    if (!P || !o) return TTG_EINVAL;
    // The FP64 path factors the working tiles in place: restore them from the
    // input.  The mixed path converts the input itself.
    ttg_status st = P->mixed ? TTG_OK : ttg_chol_plan_restore(P, stream);
    if (st != TTG_OK) return st;
    ttg_report fr{};
    st = ttg_chol_plan_factor(P, stream, &fr);
    if (st != TTG_OK) return st;
    ttg_solve_report r{};
    st = solve_after_factor(P, d_B, d_X, o, &r, stream, fr.elapsed_ms);
    if (rep) *rep = r;
    return st;
}

static ttg_status ensure_host_b(ttg_chol_plan* P, size_t blk) {
    if (P->host_b_elems >= blk) return TTG_OK;
    if (P->d_b) cudaFree(P->d_b);
    P->d_b = nullptr;
    P->host_b_elems = 0;
    TTG_CUDA_CHECK(cudaMalloc((void**)&P->d_b, sizeof(double) * 2 * blk));
    P->host_b_elems = blk;
    return TTG_OK;
}

static ttg_status ensure_host_events(ttg_chol_plan* P) {
    for (cudaEvent_t& e : P->host_ev)
        if (!e) TTG_CUDA_CHECK(cudaEventCreate(&e));
    return TTG_OK;
}

// Phase times of a host-buffer call (events 0..3 recorded around the copies).
static void host_phases(ttg_chol_plan* P, ttg_solve_report* rep, std::chrono::steady_clock::time_point t0) {
    if (!rep) return;
    float a = 0.f, b = 0.f, c = 0.f;
    cudaEventElapsedTime(&a, P->host_ev[0], P->host_ev[1]);
    cudaEventElapsedTime(&c, P->host_ev[1], P->host_ev[2]);
    cudaEventElapsedTime(&b, P->host_ev[2], P->host_ev[3]);
    rep->h2d_ms = a;
    rep->d2h_ms = b;
    rep->compute_ms = c;
    rep->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

extern "C" ttg_status ttg_chol_solve_host(ttg_chol_plan* P, const double* h_B, double* h_X, const ttg_solve_opts* o,
                                         ttg_solve_report* rep, void* stream) {
    if (!P || !o || !h_B || !h_X || o->nrhs < 1 || o->nrhs > 16) return TTG_EINVAL;
    const auto t0 = std::chrono::steady_clock::now();
    TTG_CUDA_CHECK(cudaSetDevice(P->ctx->device));
    cudaStream_t s = (cudaStream_t)stream;
    const size_t blk = (size_t)P->N * o->nrhs;
    ttg_status st = ensure_host_b(P, blk);
    if (st == TTG_OK) st = ensure_host_events(P);
    if (st != TTG_OK) return st;
    TTG_CUDA_CHECK(cudaEventRecord(P->host_ev[0], s));
    TTG_CUDA_CHECK(cudaMemcpyAsync(P->d_b, h_B, sizeof(double) * blk, cudaMemcpyHostToDevice, s));
    TTG_CUDA_CHECK(cudaEventRecord(P->host_ev[1], s));
    st = ttg_chol_plan_solve(P, P->d_b, P->d_b + blk, o, rep, stream);
    if (st != TTG_OK && st != TTG_ENOCONV) return st;
    TTG_CUDA_CHECK(cudaEventRecord(P->host_ev[2], s));
    TTG_CUDA_CHECK(cudaMemcpyAsync(h_X, P->d_b + blk, sizeof(double) * blk, cudaMemcpyDeviceToHost, s));
    TTG_CUDA_CHECK(cudaEventRecord(P->host_ev[3], s));
    TTG_CUDA_CHECK(cudaStreamSynchronize(s));
    host_phases(P, rep, t0);
    return st;
}


// Stream the host input tiles of a mixed plan into the plan input while the
// factorisation runs: on a copy stream, the diagonal tiles first (the block-
// row scales are computed from them before the launch), then each tile
// column's remaining tiles, each followed by its arrival word; the input
// tasks of the graph wait for the words.  Returns with the caller's stream
// ordered after the diagonal tiles.
static ttg_status stream_input(ttg_chol_plan* P, const double* h_tiles, cudaStream_t s) {
    if (!P->copy_s) TTG_CUDA_CHECK(cudaStreamCreateWithFlags(&P->copy_s, cudaStreamNonBlocking));
    for (cudaEvent_t& e : P->copy_ev)
        if (!e) TTG_CUDA_CHECK(cudaEventCreate(&e));
    const uint32_t gen = ttg_mixed_gate_begin(P->mixed, s, false);
    uint32_t* gate = ttg_mixed_gate(P->mixed);
    TTG_CUDA_CHECK(cudaEventRecord(P->copy_ev[0], s));  // after the caller's earlier work and the new generation
    TTG_CUDA_CHECK(cudaStreamWaitEvent(P->copy_s, P->copy_ev[0], 0));
    TTG_CUDA_CHECK(cudaEventRecord(P->host_ev[0], P->copy_s));
    const int nb = P->nb;
    for (int j = 0; j < nb; ++j) {
        const int64_t o = P->off[j + (size_t)j * nb];
        TTG_CUDA_CHECK(cudaMemcpyAsync(P->pristine + o, h_tiles + o, sizeof(double) * P->bs[j] * P->bs[j], cudaMemcpyHostToDevice,
                                       P->copy_s));
    }
    TTG_CUDA_CHECK(cudaEventRecord(P->copy_ev[1], P->copy_s));
    for (int j = 0; j < nb; ++j) {
        const int64_t o = P->off[j + (size_t)j * nb] + (int64_t)P->bs[j] * P->bs[j];
        int64_t rest = 0;
        for (int i = j + 1; i < nb; ++i) rest += (int64_t)P->bs[i] * P->bs[j];
        if (rest > 0)
            TTG_CUDA_CHECK(cudaMemcpyAsync(P->pristine + o, h_tiles + o, sizeof(double) * rest, cudaMemcpyHostToDevice, P->copy_s));
        ttg_status st = ttg_stream_write_u32(P->copy_s, gate + 1 + j, gen);
        if (st != TTG_OK) return st;
    }
    TTG_CUDA_CHECK(cudaEventRecord(P->copy_ev[2], P->copy_s));
    TTG_CUDA_CHECK(cudaStreamWaitEvent(s, P->copy_ev[1], 0));
    if (P->solver) ttg_solver_input_changed(P->solver);
    P->streaming = true;
    return TTG_OK;
}

extern "C" ttg_status ttg_chol_posv_host(ttg_chol_plan* P, const double* h_tiles, const double* h_B, double* h_X,
                                        const ttg_solve_opts* o, ttg_solve_report* rep, void* stream) {
    if (!P || !o || !h_B || !h_X || o->nrhs < 1 || o->nrhs > 16) return TTG_EINVAL;
    const auto t0 = std::chrono::steady_clock::now();
    TTG_CUDA_CHECK(cudaSetDevice(P->ctx->device));
    cudaStream_t s = (cudaStream_t)stream;
    const size_t blk = (size_t)P->N * o->nrhs;
    ttg_status sb = ensure_host_b(P, blk);
    if (sb == TTG_OK) sb = ensure_host_events(P);
    if (sb != TTG_OK) return sb;
    if (h_tiles && P->mixed && P->input_tasks) {
        // The input streams in while the factorisation runs.
        ttg_status st = stream_input(P, h_tiles, s);
        if (st != TTG_OK) {
            P->streaming = false;
            cudaStreamSynchronize(P->copy_s);
            return st;
        }
        TTG_CUDA_CHECK(cudaMemcpyAsync(P->d_b, h_B, sizeof(double) * blk, cudaMemcpyHostToDevice, s));
        TTG_CUDA_CHECK(cudaEventRecord(P->host_ev[1], s));
        ttg_report fr{};
        st = ttg_chol_plan_factor(P, stream, &fr);
        P->streaming = false;
        // Whatever the outcome, the copies end before the input is used again.
        cudaError_t ce = cudaStreamWaitEvent(s, P->copy_ev[2], 0);
        if (st != TTG_OK) {
            cudaStreamSynchronize(P->copy_s);
            return st;
        }
        TTG_CUDA_CHECK(ce);
        ttg_solve_report r{};
        st = solve_after_factor(P, P->d_b, P->d_b + blk, o, &r, stream, fr.elapsed_ms);
        if (rep) *rep = r;
        if (st != TTG_OK && st != TTG_ENOCONV) return st;
        TTG_CUDA_CHECK(cudaEventRecord(P->host_ev[2], s));
        TTG_CUDA_CHECK(cudaMemcpyAsync(h_X, P->d_b + blk, sizeof(double) * blk, cudaMemcpyDeviceToHost, s));
        TTG_CUDA_CHECK(cudaEventRecord(P->host_ev[3], s));
        TTG_CUDA_CHECK(cudaStreamSynchronize(s));
        if (rep) {
            float a = 0.f, b = 0.f, c = 0.f;
            cudaEventElapsedTime(&a, P->host_ev[0], P->copy_ev[2]);  // the whole input copy (overlapped)
            cudaEventElapsedTime(&c, P->host_ev[1], P->host_ev[2]);
            cudaEventElapsedTime(&b, P->host_ev[2], P->host_ev[3]);
            rep->h2d_ms = a;
            rep->compute_ms = c;
            rep->d2h_ms = b;
            rep->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        }
        return st;
    }
    TTG_CUDA_CHECK(cudaEventRecord(P->host_ev[0], s));
    if (h_tiles) {
        TTG_CUDA_CHECK(cudaMemcpyAsync(P->pristine, h_tiles, sizeof(double) * P->elems, cudaMemcpyHostToDevice, s));
        if (P->solver) ttg_solver_input_changed(P->solver);
    }
    TTG_CUDA_CHECK(cudaMemcpyAsync(P->d_b, h_B, sizeof(double) * blk, cudaMemcpyHostToDevice, s));
    TTG_CUDA_CHECK(cudaEventRecord(P->host_ev[1], s));
    ttg_status st = ttg_chol_posv(P, P->d_b, P->d_b + blk, o, rep, stream);
    if (st != TTG_OK && st != TTG_ENOCONV) return st;
    TTG_CUDA_CHECK(cudaEventRecord(P->host_ev[2], s));
    TTG_CUDA_CHECK(cudaMemcpyAsync(h_X, P->d_b + blk, sizeof(double) * blk, cudaMemcpyDeviceToHost, s));
    TTG_CUDA_CHECK(cudaEventRecord(P->host_ev[3], s));
    TTG_CUDA_CHECK(cudaStreamSynchronize(s));
    host_phases(P, rep, t0);
    return st;
}

extern "C" ttg_status ttg_chol_plan_dump_dag(ttg_chol_plan* P, const char* prefix) {
    if (!P || !prefix) return TTG_EINVAL;
    P->tp->dump_dag(prefix);
    return TTG_OK;
}

extern "C" ttg_status ttg_chol_plan_write_log(ttg_chol_plan* P, const char* log_path, const char* deps_path) {
    if (!P) return TTG_EINVAL;
    if (log_path) {
        std::ofstream f(log_path);
        if (!f || !P->tp->write_log(f)) return TTG_EINVAL;
    }
    if (deps_path) {
        std::ofstream f(deps_path);
        if (!f) return TTG_EINVAL;
        P->tp->write_deps(f);
    }
    return TTG_OK;
}

extern "C" ttg_status ttg_chol_plan_kind_times(ttg_chol_plan* P, double* potrf_ms, double* trsm_ms, double* gemm_ms, double* accu_ms) {
    if (!P) return TTG_EINVAL;
    const int nd = (int)P->kind_of_dev.size();
    std::vector<int64_t> s(P->tp->n_uploaded_tasks()), e(P->tp->n_uploaded_tasks());
    ttg_status st = ttg_trace(P->ctx, s.data(), e.data(), nullptr);
    if (st != TTG_OK) return st;
    double t[4] = {0, 0, 0, 0};
    for (int d = 0; d < nd; ++d)
        if (s[d] >= 0 && P->kind_of_dev[d] >= 0) t[P->kind_of_dev[d]] += (e[d] - s[d]) * 1e-6;
    if (potrf_ms) *potrf_ms = t[0];
    if (trsm_ms) *trsm_ms = t[1];
    if (gemm_ms) *gemm_ms = t[2];
    if (accu_ms) *accu_ms = t[3];
    return TTG_OK;
}

extern "C" ttg_status ttg_chol_plan_trace_dump(ttg_chol_plan* P, const char* path) {
    if (!P || !path) return TTG_EINVAL;
    const auto& nodes = P->tp->device_task_nodes();
    const int nd = (int)nodes.size(), nu = P->tp->n_uploaded_tasks();
    std::vector<int64_t> s(nu), e(nu), busy(nu);
    std::vector<int32_t> w(nu);
    ttg_status st = ttg_trace(P->ctx, s.data(), e.data(), w.data());
    if (st == TTG_OK) st = ttg_trace_busy(P->ctx, busy.data());
    if (st != TTG_OK) return st;
    FILE* f = fopen(path, "w");
    if (!f) return TTG_EINVAL;
    fprintf(f, "name,start_ns,end_ns,worker,busy_ns\n");
    for (int d = 0; d < nu; ++d)
        fprintf(f, "%s,%lld,%lld,%d,%lld\n", d < nd ? P->tp->node_name(nodes[d]).c_str() : ("INPUT_" + std::to_string(d - nd)).c_str(),
                (long long)s[d], (long long)e[d], w[d], (long long)busy[d]);
    fclose(f);
    return TTG_OK;
}

// ------------------------------------------------------------------ GEMM

struct ttg_gemm_plan {
    ttg_ctx* ctx = nullptr;
    ttg_gemm_args args{};
    int N = 0, b = 0, nb = 0;
    double *A = nullptr, *B = nullptr, *C = nullptr;  // tiles, b×b each, tile (i,j) at (i + j·nb)·b²
    std::unique_ptr<Threadpool_shared> tp;
    // Frees whatever was allocated (early returns of ttg_gemm_plan_create too).
    ~ttg_gemm_plan() {
        if (ctx) cudaSetDevice(ctx->device);
        tp.reset();
        if (A) cudaFree(A);
        if (B) cudaFree(B);
        if (C) cudaFree(C);
    }
};

static ttg_status gemm_build_graph(ttg_gemm_plan* Pp, bool dry) {
    const ttg_gemm_args* a = &Pp->args;
    const int nb = Pp->nb, b = Pp->b, n_threads = a->n_threads;
    auto tile = [Pp](double* M, int i, int j) { return M + ((size_t)i + (size_t)j * Pp->nb) * Pp->b * Pp->b; };
    Pp->tp.reset(new Threadpool_shared(n_threads, a->verb, "Wk_Gemm_0_"));
    Threadpool_shared& tp = *Pp->tp;
    if (!dry) tp.set_context(Pp->ctx);
    Taskflow<Key2> send_Aij(&tp, a->verb);
    Taskflow<Key2> send_Bij(&tp, a->verb);
    Taskflow<Key3> gemm_Cikj(&tp, a->verb);

    send_Aij.set_task([&](Key2 ij) {
                for (int k = 0; k < nb; k++) gemm_Cikj.fulfill_promise({ij[0], ij[1], k});
            })
        .set_indegree([](Key2) { return 1; })
        .set_priority([&](Key2 ij) { return (double)(nb - ij[1]); })
        .set_mapping([&](Key2 ij) { return (ij[0] + ij[1] * nb) % n_threads; })
        .set_name([](Key2 ij) { return "send_A_" + std::to_string(ij[0]) + "_" + std::to_string(ij[1]); });

    send_Bij.set_task([&](Key2 ij) {
                for (int k = 0; k < nb; k++) gemm_Cikj.fulfill_promise({k, ij[0], ij[1]});
            })
        .set_indegree([](Key2) { return 1; })
        .set_priority([&](Key2 ij) { return (double)(nb - ij[0]); })
        .set_mapping([&](Key2 ij) { return (ij[0] + ij[1] * nb) % n_threads; })
        .set_name([](Key2 ij) { return "send_B_" + std::to_string(ij[0]) + "_" + std::to_string(ij[1]); });

    gemm_Cikj.set_task([&](Key3 ikj) {
                 const int i = ikj[0], k = ikj[1], j = ikj[2];
                 gpu::cblas_dgemm(gpu::CblasColMajor, gpu::CblasNoTrans, gpu::CblasNoTrans, b, b, b, 1.0, tile(Pp->A, i, k), b,
                                  tile(Pp->B, k, j), b, 1.0, tile(Pp->C, i, j), b);
                 if (k < nb - 1) gemm_Cikj.fulfill_promise({i, k + 1, j});
             })
        .set_indegree([](Key3 ikj) { return ikj[1] == 0 ? 2 : 3; })
        .set_mapping([&](Key3 ikj) { return (ikj[0] + ikj[2] * nb) % n_threads; })
        .set_name([](Key3 ikj) {
            return "prod_C_" + std::to_string(ikj[0]) + "_" + std::to_string(ikj[1]) + "_" + std::to_string(ikj[2]);
        });

    for (int i = 0; i < nb; i++)
        for (int j = 0; j < nb; j++) {
            send_Aij.fulfill_promise({i, j});
            send_Bij.fulfill_promise({i, j});
        }
    try {
        if (dry) tp.capture_dry();
        else tp.capture_only();
    } catch (const std::exception& e) {
        fprintf(stderr, "ttg_gemm_plan: %s\n", e.what());
        return TTG_EINVAL;
    }
    return TTG_OK;
}

// Capture the block GEMM graph without a device and write its DAG record.
extern "C" ttg_status ttg_gemm_dag_dump(const ttg_gemm_args* a, const char* prefix) {
    if (!a || !prefix || a->block_size <= 0 || a->matrix_size <= 0 || a->matrix_size % a->block_size != 0 || a->n_threads <= 0)
        return TTG_EINVAL;
    ttg_gemm_plan P;
    P.args = *a;
    P.N = a->matrix_size;
    P.b = a->block_size;
    P.nb = P.N / P.b;
    ttg_status s = gemm_build_graph(&P, true);
    if (s != TTG_OK) return s;
    P.tp->dump_dag(prefix);
    return TTG_OK;
}

extern "C" ttg_status ttg_gemm_plan_create(ttg_ctx* ctx, const ttg_gemm_args* a, ttg_gemm_plan** out) {
    if (!ctx || !a || !out) return TTG_EINVAL;
    *out = nullptr;
    if (a->block_size <= 0 || a->matrix_size <= 0 || a->matrix_size % a->block_size != 0 || a->n_threads <= 0)
        return TTG_EINVAL;
    std::unique_ptr<ttg_gemm_plan> P(new ttg_gemm_plan());
    P->ctx = ctx;
    P->args = *a;
    P->N = a->matrix_size;
    P->b = a->block_size;
    P->nb = P->N / P->b;
    const size_t elems = (size_t)P->N * P->N;
    TTG_CUDA_CHECK(cudaSetDevice(ctx->device));
    TTG_CUDA_CHECK(cudaMalloc((void**)&P->A, sizeof(double) * elems));
    TTG_CUDA_CHECK(cudaMalloc((void**)&P->B, sizeof(double) * elems));
    TTG_CUDA_CHECK(cudaMalloc((void**)&P->C, sizeof(double) * elems));
    // Inputs in tile layout: val_global (gemm_shared.hpp:74-76, A = B) or
    // iid U[-1,1] (A from stream 2, B from stream 3 of the seed).
    {
        ttg_status s = ttg_gen_gemm_tiles(ctx, P->N, P->b, a->inputs, a->seed, P->A, P->B, nullptr);
        if (s != TTG_OK) return s;
    }
    ttg_status st = gemm_build_graph(P.get(), false);
    if (st != TTG_OK) return st;  // P's destructor frees the tiles
    *out = P.release();
    return TTG_OK;
}

extern "C" ttg_status ttg_gemm_plan_destroy(ttg_gemm_plan* P) {
    delete P;  // the destructor frees the device tiles
    return TTG_OK;
}

extern "C" int32_t ttg_gemm_plan_tasks(const ttg_gemm_plan* P, double* capture_s) {
    if (!P) return 0;
    if (capture_s) *capture_s = P->tp->capture_seconds();
    return P->tp->n_device_tasks();
}

extern "C" ttg_status ttg_gemm_plan_run(ttg_gemm_plan* P, void* stream, ttg_report* rep) {
    if (!P) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(P->ctx->device));
    TTG_CUDA_CHECK(cudaMemsetAsync(P->C, 0, sizeof(double) * (size_t)P->N * P->N, (cudaStream_t)stream));
    ttg_status s = P->tp->replay(stream);
    if (rep) *rep = P->tp->report();
    return s;
}

// Dense column-major N×N host matrix <-> tiles (b×b, tile (i,j) at (i + j·nb)·b²).
static ttg_status gemm_dense_to_tiles(const ttg_gemm_plan* P, const double* h, double* d, cudaStream_t s) {
    for (int j = 0; j < P->nb; ++j)
        for (int i = 0; i < P->nb; ++i)
            TTG_CUDA_CHECK(cudaMemcpy2DAsync(d + ((size_t)i + (size_t)j * P->nb) * P->b * P->b, sizeof(double) * P->b,
                                             h + (size_t)i * P->b + (size_t)j * P->b * P->N, sizeof(double) * P->N,
                                             sizeof(double) * P->b, P->b, cudaMemcpyHostToDevice, s));
    return TTG_OK;
}

static ttg_status gemm_tiles_to_dense(const ttg_gemm_plan* P, const double* d, double* h, cudaStream_t s) {
    for (int j = 0; j < P->nb; ++j)
        for (int i = 0; i < P->nb; ++i)
            TTG_CUDA_CHECK(cudaMemcpy2DAsync(h + (size_t)i * P->b + (size_t)j * P->b * P->N, sizeof(double) * P->N,
                                             d + ((size_t)i + (size_t)j * P->nb) * P->b * P->b, sizeof(double) * P->b,
                                             sizeof(double) * P->b, P->b, cudaMemcpyDeviceToHost, s));
    return TTG_OK;
}

extern "C" ttg_status ttg_gemm_host(ttg_gemm_plan* P, const double* h_A, const double* h_B, double* h_C, void* stream,
                                    ttg_report* rep) {
    if (!P || !h_A || !h_B) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(P->ctx->device));
    cudaStream_t s = (cudaStream_t)stream;
    ttg_status st = gemm_dense_to_tiles(P, h_A, P->A, s);
    if (st == TTG_OK) st = gemm_dense_to_tiles(P, h_B, P->B, s);
    if (st == TTG_OK) st = ttg_gemm_plan_run(P, stream, rep);
    if (st == TTG_OK && h_C) {
        st = gemm_tiles_to_dense(P, P->C, h_C, s);
        if (st == TTG_OK) TTG_CUDA_CHECK(cudaStreamSynchronize(s));
    }
    return st;
}

extern "C" ttg_status ttg_gemm_plan_get_C(ttg_gemm_plan* P, double* h_C) {
    if (!P || !h_C) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(P->ctx->device));
    ttg_status st = gemm_tiles_to_dense(P, P->C, h_C, nullptr);
    if (st != TTG_OK) return st;
    TTG_CUDA_CHECK(cudaStreamSynchronize(nullptr));
    return TTG_OK;
}

extern "C" ttg_status ttg_gemm_plan_dump_dag(ttg_gemm_plan* P, const char* prefix) {
    if (!P || !prefix) return TTG_EINVAL;
    P->tp->dump_dag(prefix);
    return TTG_OK;
}
