// ttg_serve.cu — the request loop of include/ttg_serve.h.
//
// Host side: request generation (Philox, so a stream is reproducible), the
// real-time loop (arrivals, admission under the HBM budget, LRU eviction of
// resident factors, one launch per free lane built from the waiting
// requests with the DAG builder of batch_graph.h), and latency statistics.
// Device side: the executor, the stream-ordered input generators of
// ttg_gen.cu, and a backward-error kernel.  Device memory of requests comes
// from the stream-ordered pool (cudaMallocAsync), so admitting a request
// never waits for the other lane.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <list>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/ttg.h"
#include "../../include/ttg_philox.h"
#include "../../include/ttg_serve.h"
#include "batch_graph.h"
#include "exec.cuh"
#include "tile_f64.cuh"
#include "ttg_mixed_api.h"
#include "ttg_internal.h"

using namespace ttg::batch;

namespace {

constexpr int kRowsPerBlock = 256;  // backward-error rows per block

// One request's operands for the backward-error kernels.
struct BwdItem {
    int N, tile, nrhs;
    const double* A;  // packed lower tiles, full diagonal tiles
    const double* B;  // nrhs × N row blocks
    const double* X;
    unsigned long long* acc;  // [2·nrhs + 1]: max |r_q|, max |x_q|, max row sum (as ordered bit patterns)
};

__device__ __forceinline__ void atomic_max_pos(unsigned long long* p, double v) {
    // Non-negative doubles order like their bit patterns; NaN maps to +inf.
    if (!(v == v)) v = INFINITY;
    atomicMax(p, (unsigned long long)__double_as_longlong(v));
}

// Grid (items, row slices): block (i, s) handles rows [256 s, 256 s + 256) of item i.
__global__ void serve_bwd_partial(const BwdItem* __restrict__ items) {
    const BwdItem it = items[blockIdx.x];
    const int r = blockIdx.y * kRowsPerBlock + threadIdx.x;
    const int N = it.N, t = it.tile, nr = it.nrhs;
    const int nb = (N + t - 1) / t;
    auto bs = [&](int i) { return i < nb - 1 ? t : N - (nb - 1) * t; };
    auto off = [&](int i, int j) { return (int64_t)t * ((int64_t)j * N - (int64_t)t * j * (j - 1) / 2) + (int64_t)(i - j) * t * bs(j); };
    if (r >= N) return;
    double acc[16];
    for (int q = 0; q < 16; ++q) acc[q] = q < nr ? it.B[q + (int64_t)r * nr] : 0.0;
    double asum = 0.0;
    const int bi = r / t, li = r - bi * t;
    for (int c = 0; c < N; ++c) {
        const int bj = c / t, lj = c - bj * t;
        const double a = r >= c ? it.A[off(bi, bj) + li + (int64_t)lj * bs(bi)] : it.A[off(bj, bi) + lj + (int64_t)li * bs(bj)];
        asum += fabs(a);
        for (int q = 0; q < 16; ++q)
            if (q < nr) acc[q] = fma(-a, it.X[q + (int64_t)c * nr], acc[q]);
    }
    for (int q = 0; q < nr; ++q) {
        atomic_max_pos(it.acc + q, fabs(acc[q]));
        atomic_max_pos(it.acc + nr + q, fabs(it.X[q + (int64_t)r * nr]));
    }
    atomic_max_pos(it.acc + 2 * nr, asum);
}

__global__ void serve_bwd_final(const BwdItem* __restrict__ items, int n, double* err) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const BwdItem it = items[i];
        const double a = __longlong_as_double((long long)it.acc[2 * it.nrhs]);
        double worst = 0.0;
        for (int q = 0; q < it.nrhs; ++q) {
            const double rq = __longlong_as_double((long long)it.acc[q]);
            const double xq = __longlong_as_double((long long)it.acc[it.nrhs + q]);
            const double be = xq > 0 ? rq / (a * xq) : (rq > 0 ? INFINITY : 0.0);
            worst = (be != be) ? INFINITY : fmax(worst, be);
        }
        err[i] = worst;
    }
}

double u01_at(uint32_t seed, uint32_t i, uint32_t k) {
    ttg_u32x4 ctr = {{i, 0x5e47u, k, 0u}};
    const ttg_u32x4 x = ttg_philox4x32_10(ctr, seed, 0x9e3779b9u);
    return ttg_u01(x.v[0], x.v[1]);
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

extern "C" int32_t ttg_serve_tile(int32_t n) { return n <= 256 ? 64 : (n <= 2048 ? 128 : 256); }

struct ServeRequest {
    int N = 0, tile = 0;
    uint32_t seed_a = 0, seed_b = 0;
    double arrival = 0.0;
    int followup_of = -1;  // request whose factor this one reuses
    int ir_steps = 0;
    // Run state.
    bool queued = false, done = false;
    int retries = 0;
    double finish = 0.0, bwd = 0.0;
    double* B = nullptr;  // device vectors of the attempt in flight
    double* X = nullptr;
    double* R = nullptr;
    float* D32 = nullptr;
    double* D64 = nullptr;  // mixed factorisation scratch
    uint8_t* tc = nullptr;  // mixed, tensor-core updates: header, scales, panel slots
    size_t work_bytes = 0;
    // Open lanes: the lane and in-flight slot of the attempt, its phase (1
    // published, 2 backward error under way) and its attempt number.
    int lane = -1, slot = -1, phase = 0, attempt = 0;
    int key = -1;  // resident factor it factors or uses
    std::vector<double> result;
};

struct Resident {
    int N = 0, tile = 0;
    uint32_t seed_a = 0;
    double* A64 = nullptr;
    double* W64 = nullptr;
    float* W32 = nullptr;
    size_t bytes = 0;
    bool complete = false;  // the factorisation finished
    int users = 0;          // launches in flight that read it
    cudaStream_t last = nullptr;
    std::list<int>::iterator lru;
};

struct Lane {
    ttg_ctx* ctx = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t done = nullptr;
    bool busy = false;
    Graph g;
    std::vector<int> reqs;
    BwdItem* h_items = nullptr;  // pinned
    BwdItem* d_items = nullptr;
    unsigned long long* d_acc = nullptr;
    double* h_err = nullptr;     // pinned
    double* d_err = nullptr;
    // Tensor-core systems of the launch: their headers (pinned staging) and
    // the diagonal tiles whose block-row scales run before the executor.
    uint8_t* h_hdr = nullptr;  // pinned, max_batch headers
    std::vector<TcRowScaleItem> rs;
    TcRowScaleItem* h_rs = nullptr;  // pinned
    TcRowScaleItem* d_rs = nullptr;
    int rs_cap = 0, n_hdr = 0;
};

// An open lane: one executor launch that keeps taking work (an epoch).  Its
// arena holds the tasks of the epoch's requests back to back — ops, counters,
// successor lists, team counters, one first-in-first-out queue — and the
// host appends a request's tasks on the lane's copy stream, then publishes
// them (task and root counts) with stream-ordered 32-bit writes that the idle
// workers poll (exec.cuh, admit_roots).  An epoch whose arena is full is
// closed: its launch ends once every published task has run, and the next
// epoch starts from an empty arena.
// Left to the side stream (on the SMs the lanes leave free): the input
// generators (an O(N³) int8 product per synthetic request), block-row scales
// and backward errors.
// Where the open loop's host thread is (TTG_SERVE_VERBOSE reports it from a
// watchdog thread, so that a blocking call shows by name).
std::atomic<const char*> g_open_at{"start"};
constexpr int kOpenTasks = 1 << 20;         // tasks per epoch
constexpr int64_t kOpenEdges = 8ll << 20;   // successor entries per epoch
constexpr int kOpenParts = 4 << 20;         // queue slots per epoch
constexpr int kOpenTeams = 16384;           // team POTRFs per epoch
constexpr int kOpenInflight = 64;           // requests in flight per lane
struct OpenLane {
    ttg_ctx* ctx = nullptr;
    cudaStream_t ks = nullptr, cs = nullptr;  // the executor; copies and publication
    cudaEvent_t kdone = nullptr;
    bool running = false, closing = false;
    int cap_tasks = kOpenTasks;  // tasks per epoch (TTG_SERVE_EPOCH_TASKS lowers it)
    ttg_op* ops = nullptr;
    int *count = nullptr, *runs = nullptr, *parts = nullptr, *part_next = nullptr, *part_done = nullptr;
    uint8_t* level = nullptr;
    int32_t* bind = nullptr;
    int64_t* succ_ptr = nullptr;
    int32_t* succ_idx = nullptr;
    int *team_slot = nullptr, *team_ctr = nullptr, *roots = nullptr;
    int *qbuf = nullptr, *q_off = nullptr, *q_head = nullptr, *q_tail = nullptr;
    int *bq = nullptr;  // unused bound queues (offsets, heads, tails: zeros)
    int *status = nullptr, *pub = nullptr, *admit = nullptr;
    int n_tasks = 0, n_roots = 0, n_teams = 0, n_parts = 0;
    int64_t n_edges = 0;
    int n_inflight = 0;
    std::vector<int> slot_req;  // request in each in-flight slot, or -1
    BwdItem* h_items = nullptr;  // pinned, per slot
    BwdItem* d_items = nullptr;
    unsigned long long* d_acc = nullptr;
    double* h_err = nullptr;  // pinned, per slot
    double* d_err = nullptr;
    std::vector<cudaEvent_t> ev;  // per slot: backward error read
    std::vector<TcRowScaleItem> rs;
    TcRowScaleItem* d_rs = nullptr;
    int rs_cap = 0;
};

struct ttg_serve {
    int device = 0, sms = 0;
    // Open lanes (admission 1).
    std::vector<OpenLane> open;
    cudaStream_t side = nullptr;  // input generation, block-row scales, backward errors
    int* h_flag = nullptr;        // host-mapped, per request: the attempt whose tasks all ran
    int* d_flag = nullptr;
    ttg_serve_args a{};
    std::vector<ServeRequest> req;
    std::unordered_map<int, Resident> res;  // keyed by the request that first factored the matrix
    std::list<int> lru;                     // complete, idle factors: front = least recent
    std::vector<Lane> lanes;
    size_t used = 0, peak = 0, budget = 0;
    int evictions = 0, misses = 0, launches = 0, retries = 0;
};

namespace {

size_t factor_bytes(const ttg_serve* s, int N, int tile) {
    System S;
    S.set_size(N, tile);
    const size_t e = (size_t)S.elems();
    return e * 8 + (s->a.precision == TTG_PREC_MIXED ? e * 4 : e * 8);
}

// Tensor-core data of a mixed factorisation: header, slot and block-row
// scales (256-byte aligned), then the panel slots.
size_t tc_scale_bytes(const System& S) { return ((size_t)(S.nb * (S.nb + 1) / 2 + S.nb) * 4 + 255) / 256 * 256; }
size_t tc_bytes(const System& S) { return kTcHeaderBytes + tc_scale_bytes(S) + ttg_mixed_tc_slot_elems(S.tile, S.nb) * 2; }

size_t work_bytes(const ttg_serve* s, int N, int tile, bool factor) {
    const size_t v = (size_t)N * s->a.nrhs;
    size_t b = v * 16;  // B, X
    if (s->a.precision == TTG_PREC_MIXED) {
        b += v * 12;  // R, D32
        if (factor) {
            System S;
            S.set_size(N, tile);
            b += (size_t)S.nb * S.tile * S.tile * 8;  // diagonal POTRF scratch
            if (System::tc_fits(S.N, S.tile)) b += tc_bytes(S);
        }
    }
    return b;
}

template <class T>
ttg_status pool_alloc(T** p, size_t count, cudaStream_t s) {
    *p = nullptr;
    TTG_CUDA_CHECK(cudaMallocAsync((void**)p, sizeof(T) * std::max<size_t>(1, count), s));
    return TTG_OK;
}

template <class T>
void pool_free(T*& p, cudaStream_t s) {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
}

// Free least-recently-used idle factors until `need` more bytes fit.
bool make_room(ttg_serve* s, size_t need) {
    while (s->used + need > s->budget) {
        if (s->lru.empty()) return false;
        const int k = s->lru.front();
        s->lru.pop_front();
        Resident& r = s->res[k];
        cudaStream_t st = r.last ? r.last : s->lanes[0].s;
        pool_free(r.A64, st);
        pool_free(r.W64, st);
        pool_free(r.W32, st);
        s->used -= r.bytes;
        s->res.erase(k);
        ++s->evictions;
    }
    return true;
}

void release_factor(ttg_serve* s, int k, cudaStream_t st) {
    Resident& r = s->res[k];
    r.last = st;
    if (--r.users == 0 && r.complete) r.lru = s->lru.insert(s->lru.end(), k);
}

void use_factor(ttg_serve* s, int k) {
    Resident& r = s->res[k];
    if (r.users == 0 && r.complete) s->lru.erase(r.lru);
    ++r.users;
}

// Try to add request i to lane L's launch; false when it must wait.
// Where an admitted request goes: the stream that allocates and generates
// its operands (stream-ordered), the graph its tasks are added to, the
// diagonal tiles whose block-row scales must be computed before it runs, and
// the pinned staging of its tensor-core header (null: a pageable copy).
struct AdmitTarget {
    ttg_ctx* ctx;  // the generators' device context
    cudaStream_t st;
    Graph* g;
    std::vector<TcRowScaleItem>* rs;
    uint8_t* h_hdr;
    int* n_hdr;
    int max_hdr;
};

bool admit_to(ttg_serve* s, AdmitTarget& T, int i, ttg_status* err) {
    ServeRequest& q = s->req[i];
    const bool mixed = s->a.precision == TTG_PREC_MIXED;
    int key = q.followup_of >= 0 ? q.followup_of : i;
    // A follow-up whose first factorisation has not been launched or is still
    // running waits for it; one whose factor was evicted factors again.
    bool need_factor = true;
    auto it = s->res.find(key);
    if (it != s->res.end()) {
        if (!it->second.complete) return false;
        need_factor = false;
    } else if (q.followup_of >= 0) {
        const ServeRequest& t = s->req[q.followup_of];
        if (!t.done) return false;
    }
    const size_t fb = need_factor ? factor_bytes(s, q.N, q.tile) : 0;
    const size_t wb = work_bytes(s, q.N, q.tile, need_factor);
    if (!need_factor) use_factor(s, key);  // pin it before making room
    if (!make_room(s, fb + wb)) {
        if (!need_factor) release_factor(s, key, T.st);
        return false;
    }
    cudaStream_t st = T.st;
    System S;
    S.set_size(q.N, q.tile);
    S.mixed = mixed;
    S.nrhs = s->a.nrhs;
    S.ir_steps = q.ir_steps;
    S.factored = !need_factor;
    ttg_status e = TTG_OK;
    if (need_factor) {
        if (q.followup_of >= 0) ++s->misses;
        Resident r;
        r.N = q.N;
        r.tile = q.tile;
        r.seed_a = q.seed_a;
        r.bytes = fb;
        const size_t el = (size_t)S.elems();
        if ((e = pool_alloc(&r.A64, el, st)) == TTG_OK)
            e = mixed ? pool_alloc(&r.W32, el, st) : pool_alloc(&r.W64, el, st);
        if (e == TTG_OK) e = ttg_gen_gram_async(T.ctx, q.N, q.tile, s->a.alpha, q.seed_a, r.A64, st);
        if (e == TTG_OK && !mixed)
            e = cudaMemcpyAsync(r.W64, r.A64, sizeof(double) * el, cudaMemcpyDeviceToDevice, st) == cudaSuccess ? TTG_OK : TTG_ECUDA;
        r.users = 1;
        r.last = st;
        s->res[key] = r;
        s->used += fb;
    }
    const Resident& r = s->res[key];
    const size_t v = (size_t)q.N * s->a.nrhs;
    if (e == TTG_OK) e = pool_alloc(&q.B, v, st);
    if (e == TTG_OK) e = pool_alloc(&q.X, v, st);
    if (e == TTG_OK && mixed) {
        if ((e = pool_alloc(&q.R, v, st)) == TTG_OK) e = pool_alloc(&q.D32, v, st);
        if (e == TTG_OK && need_factor) e = pool_alloc(&q.D64, (size_t)S.nb * S.tile * S.tile, st);
        // Split-BF16 updates on the tensor cores when the tiles allow it.
        if (e == TTG_OK && need_factor && System::tc_fits(S.N, S.tile) && (!T.h_hdr || *T.n_hdr < T.max_hdr)) {
            e = pool_alloc(&q.tc, tc_bytes(S), st);
            if (e == TTG_OK) {
                float* slot_scale = (float*)(q.tc + kTcHeaderBytes);
                float* rowscale = slot_scale + S.nb * (S.nb + 1) / 2;
                __nv_bfloat16* slots = (__nv_bfloat16*)(q.tc + kTcHeaderBytes + tc_scale_bytes(S));
                std::vector<uint8_t> local(T.h_hdr ? 0 : kTcHeaderBytes);
                uint8_t* h = T.h_hdr ? T.h_hdr + kTcHeaderBytes * (size_t)*T.n_hdr : local.data();
                e = ttg_mixed_tc_header(h, q.tc, slots, slot_scale, rowscale, S.tile, S.nb, &S.tc_tables);
                // (A pageable source is staged before the call returns.)
                if (e == TTG_OK)
                    e = cudaMemcpyAsync(q.tc, h, kTcHeaderBytes, cudaMemcpyHostToDevice, st) == cudaSuccess ? TTG_OK : TTG_ECUDA;
                if (e == TTG_OK) {
                    ++*T.n_hdr;
                    for (int i = 0; i < S.nb; ++i) T.rs->push_back(TcRowScaleItem{r.A64 + S.off(i, i), S.bs(i), S.bs(i), rowscale + i});
                }
            }
        }
    }
    if (e == TTG_OK) e = ttg_gen_rhs_rows_async(q.N, s->a.nrhs, q.seed_b, q.B, st);
    if (e == TTG_OK && !mixed)
        e = cudaMemcpyAsync(q.X, q.B, sizeof(double) * v, cudaMemcpyDeviceToDevice, st) == cudaSuccess ? TTG_OK : TTG_ECUDA;
    q.work_bytes = wb;
    s->used += wb;
    s->peak = std::max(s->peak, s->used);
    q.key = key;
    if (e != TTG_OK) {
        *err = e;
        return true;
    }
    S.A64 = r.A64;
    S.W64 = r.W64;
    S.W32 = r.W32;
    S.D64 = q.D64;
    S.B = q.B;
    S.X = q.X;
    S.R = q.R;
    S.D32 = q.D32;
    add_system(*T.g, S);
    return true;
}

bool admit(ttg_serve* s, Lane& L, int i, ttg_status* err) {
    AdmitTarget T{L.ctx, L.s, &L.g, &L.rs, L.h_hdr, &L.n_hdr, s->a.max_batch};
    if (!admit_to(s, T, i, err)) return false;
    L.reqs.push_back(i);
    return true;
}

// Build, upload and launch lane L's next launch from the waiting requests.
ttg_status dispatch(ttg_serve* s, Lane& L, std::deque<int>& queue) {
    L.g.clear();
    L.reqs.clear();
    L.rs.clear();
    L.n_hdr = 0;
    ttg_status err = TTG_OK;
    double flops = 0.0;
    for (auto it = queue.begin(); it != queue.end() && (int)L.reqs.size() < s->a.max_batch;) {
        const int i = *it;
        const ServeRequest& q = s->req[i];
        const bool factors = s->res.find(q.followup_of >= 0 ? q.followup_of : i) == s->res.end();
        const double f = factors ? (double)q.N * q.N * q.N / 3.0 : 0.0;
        // Keep launches short enough that the other lane gets work too.
        if (!L.reqs.empty() && flops + f > 4e11) break;
        if (admit(s, L, i, &err)) {
            if (err != TTG_OK) return err;
            flops += f;
            it = queue.erase(it);
        } else {
            ++it;
        }
    }
    if (L.reqs.empty()) return TTG_OK;
    ttg_status st = L.g.finish(true);
    if (st != TTG_OK) return st;
    ttg_graph_desc d = L.g.desc();
    if ((st = ttg_graph_upload(L.ctx, &d)) != TTG_OK) return st;
    // Block-row scales of the launch's tensor-core factorisations.
    if ((int)L.rs.size() > L.rs_cap) return TTG_EINVAL;
    if (!L.rs.empty()) {
        std::copy(L.rs.begin(), L.rs.end(), L.h_rs);
        TTG_CUDA_CHECK(cudaMemcpyAsync(L.d_rs, L.h_rs, sizeof(TcRowScaleItem) * L.rs.size(), cudaMemcpyHostToDevice, L.s));
        if ((st = ttg_mixed_row_scales(L.d_rs, (int)L.rs.size(), L.s)) != TTG_OK) return st;
    }
    ttg_mixed_set_tc(L.ctx, L.n_hdr > 0);
    if ((st = ttg_launch(L.ctx, L.s)) != TTG_OK) return st;
    // Backward errors of the launch, then the completion event.
    const int n = (int)L.reqs.size();
    for (int k = 0; k < n; ++k) {
        const ServeRequest& q = s->req[L.reqs[k]];
        L.h_items[k] = BwdItem{q.N, q.tile, s->a.nrhs, s->res[q.key].A64, q.B, q.X, L.d_acc + (size_t)k * 33};
    }
    int slices = 1;
    for (int k = 0; k < n; ++k) slices = std::max(slices, (s->req[L.reqs[k]].N + kRowsPerBlock - 1) / kRowsPerBlock);
    TTG_CUDA_CHECK(cudaMemcpyAsync(L.d_items, L.h_items, sizeof(BwdItem) * n, cudaMemcpyHostToDevice, L.s));
    TTG_CUDA_CHECK(cudaMemsetAsync(L.d_acc, 0, sizeof(unsigned long long) * 33 * n, L.s));
    ttg_note_launch();
    serve_bwd_partial<<<dim3(n, slices), kRowsPerBlock, 0, L.s>>>(L.d_items);
    ttg_note_launch();
    serve_bwd_final<<<1, 128, 0, L.s>>>(L.d_items, n, L.d_err);
    TTG_CUDA_CHECK(cudaGetLastError());
    TTG_CUDA_CHECK(cudaMemcpyAsync(L.h_err, L.d_err, sizeof(double) * n, cudaMemcpyDeviceToHost, L.s));
    if (s->a.keep_results) {
        for (int k = 0; k < n; ++k) {
            ServeRequest& q = s->req[L.reqs[k]];
            q.result.assign((size_t)q.N * s->a.nrhs, 0.0);
        }
    }
    TTG_CUDA_CHECK(cudaEventRecord(L.done, L.s));
    L.busy = true;
    ++s->launches;
    return TTG_OK;
}

// Lane L finished: collect results, release memory, requeue retries.
ttg_status complete(ttg_serve* s, Lane& L, std::deque<int>& queue, double t) {
    ttg_report rep{};
    ttg_status st = ttg_wait(L.ctx, &rep);
    if (st != TTG_OK) return st;
    const bool mixed = s->a.precision == TTG_PREC_MIXED;
    for (size_t k = 0; k < L.reqs.size(); ++k) {
        const int i = L.reqs[k];
        ServeRequest& q = s->req[i];
        q.bwd = L.h_err[k];
        if (s->a.keep_results) {
            // Row blocks (ld nrhs) to N × nrhs column-major.
            std::vector<double> v((size_t)q.N * s->a.nrhs);
            TTG_CUDA_CHECK(cudaMemcpy(v.data(), q.X, sizeof(double) * v.size(), cudaMemcpyDeviceToHost));
            for (int c = 0; c < s->a.nrhs; ++c)
                for (int r = 0; r < q.N; ++r) q.result[r + (size_t)c * q.N] = v[c + (size_t)r * s->a.nrhs];
        }
        pool_free(q.B, L.s);
        pool_free(q.X, L.s);
        pool_free(q.R, L.s);
        pool_free(q.D32, L.s);
        pool_free(q.D64, L.s);
        pool_free(q.tc, L.s);
        s->used -= q.work_bytes;
        q.work_bytes = 0;
        Resident& r = s->res[q.key];
        r.complete = true;
        release_factor(s, q.key, L.s);
        if (mixed && !(q.bwd <= s->a.tol) && q.retries < 2) {
            // Not yet at the target: solve again with twice the refinement.
            ++q.retries;
            ++s->retries;
            q.ir_steps *= 2;
            queue.push_front(i);
            continue;
        }
        q.done = true;
        q.finish = t;
    }
    L.busy = false;
    return TTG_OK;
}

}  // namespace

namespace {

// ------------------------------------------------------------ open lanes

using ttg::kMaxLevels;
using ttg::kTeamStride;
using ttg::team_fits;

template <class T>
cudaError_t dev_zero(T** p, size_t count) {
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(1, count));
    if (e == cudaSuccess) e = cudaMemset(*p, 0, sizeof(T) * std::max<size_t>(1, count));
    return e;
}

ttg_status open_lane_setup(ttg_serve* s, OpenLane& L, int workers) {
    ttg_opts o{};
    o.device = s->device;
    o.workers = workers;
    o.timeout_s = 60.0;
    ttg_status st = ttg_create(&L.ctx, &o);
    if (st != TTG_OK) return st;
    L.ctx->coop = false;  // lanes share the GPU
    if (const char* v = getenv("TTG_SERVE_EPOCH_TASKS")) L.cap_tasks = std::max(256, std::min(kOpenTasks, atoi(v)));
    cudaError_t e = cudaStreamCreateWithFlags(&L.ks, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&L.cs, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&L.kdone, cudaEventDisableTiming);
    if (e == cudaSuccess) e = dev_zero(&L.ops, kOpenTasks);
    if (e == cudaSuccess) e = dev_zero(&L.count, kOpenTasks);
    if (e == cudaSuccess) e = dev_zero(&L.runs, kOpenTasks);
    if (e == cudaSuccess) e = dev_zero(&L.parts, kOpenTasks);
    if (e == cudaSuccess) e = dev_zero(&L.part_next, kOpenTasks);
    if (e == cudaSuccess) e = dev_zero(&L.part_done, kOpenTasks);
    if (e == cudaSuccess) e = dev_zero(&L.level, kOpenTasks);
    if (e == cudaSuccess) e = dev_zero(&L.bind, kOpenTasks);
    if (e == cudaSuccess) e = dev_zero(&L.succ_ptr, (size_t)kOpenTasks + 1);
    if (e == cudaSuccess) e = dev_zero(&L.succ_idx, (size_t)kOpenEdges);
    if (e == cudaSuccess) e = dev_zero(&L.team_slot, kOpenTasks);
    if (e == cudaSuccess) e = dev_zero(&L.team_ctr, (size_t)kOpenTeams * kTeamStride);
    if (e == cudaSuccess) e = dev_zero(&L.roots, kOpenTasks);
    if (e == cudaSuccess) e = dev_zero(&L.qbuf, kOpenParts);
    if (e == cudaSuccess) e = dev_zero(&L.q_off, 2);
    if (e == cudaSuccess) e = dev_zero(&L.q_head, (size_t)kMaxLevels * 32);
    if (e == cudaSuccess) e = dev_zero(&L.q_tail, (size_t)kMaxLevels * 32);
    if (e == cudaSuccess) e = dev_zero(&L.bq, (size_t)3 * (workers + 1));
    if (e == cudaSuccess) e = dev_zero(&L.status, 8);
    if (e == cudaSuccess) e = dev_zero(&L.pub, 4);
    if (e == cudaSuccess) e = dev_zero(&L.admit, 2);
    if (e == cudaSuccess) {
        const int off[2] = {0, kOpenParts};
        e = cudaMemcpy(L.q_off, off, sizeof(off), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMallocHost((void**)&L.h_items, sizeof(BwdItem) * kOpenInflight);
    if (e == cudaSuccess) e = cudaMalloc((void**)&L.d_items, sizeof(BwdItem) * kOpenInflight);
    if (e == cudaSuccess) e = cudaMalloc((void**)&L.d_acc, sizeof(unsigned long long) * 33 * kOpenInflight);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&L.h_err, sizeof(double) * kOpenInflight);
    if (e == cudaSuccess) e = cudaMalloc((void**)&L.d_err, sizeof(double) * kOpenInflight);
    L.rs_cap = s->a.n_max / 128 + 2;  // the diagonal tiles of one request
    if (e == cudaSuccess) e = cudaMalloc((void**)&L.d_rs, sizeof(TcRowScaleItem) * (size_t)L.rs_cap);
    L.slot_req.assign(kOpenInflight, -1);
    L.ev.assign(kOpenInflight, nullptr);
    for (int k = 0; k < kOpenInflight && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&L.ev[k], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        ttg_set_last_cuda_error(e, "open lane set-up", __FILE__, __LINE__);
        return e == cudaErrorMemoryAllocation ? TTG_ENOMEM : TTG_ECUDA;
    }
    return TTG_OK;
}

void open_lane_free(OpenLane& L) {
    if (L.ks) cudaStreamSynchronize(L.ks);
    if (L.cs) cudaStreamSynchronize(L.cs);
    for (void* p : {(void*)L.ops, (void*)L.count, (void*)L.runs, (void*)L.parts, (void*)L.part_next, (void*)L.part_done,
                    (void*)L.level, (void*)L.bind, (void*)L.succ_ptr, (void*)L.succ_idx, (void*)L.team_slot, (void*)L.team_ctr,
                    (void*)L.roots, (void*)L.qbuf, (void*)L.q_off, (void*)L.q_head, (void*)L.q_tail, (void*)L.bq, (void*)L.status,
                    (void*)L.pub, (void*)L.admit, (void*)L.d_items, (void*)L.d_acc, (void*)L.d_err, (void*)L.d_rs})
        if (p) cudaFree(p);
    if (L.h_items) cudaFreeHost(L.h_items);
    if (L.h_err) cudaFreeHost(L.h_err);
    for (cudaEvent_t e : L.ev)
        if (e) cudaEventDestroy(e);
    if (L.kdone) cudaEventDestroy(L.kdone);
    if (L.ks) cudaStreamDestroy(L.ks);
    if (L.cs) cudaStreamDestroy(L.cs);
    if (L.ctx) ttg_destroy(L.ctx);
}

// Start an epoch: an empty arena and the executor launch that serves it.
ttg_status open_epoch_start(ttg_serve* s, OpenLane& L) {
    g_open_at = "epoch start";
    TTG_CUDA_CHECK(cudaMemsetAsync(L.qbuf, 0xff, sizeof(int) * (size_t)kOpenParts, L.ks));  // every slot unwritten (-1)
    TTG_CUDA_CHECK(cudaMemsetAsync(L.q_head, 0, sizeof(int) * kMaxLevels * 32, L.ks));
    TTG_CUDA_CHECK(cudaMemsetAsync(L.q_tail, 0, sizeof(int) * kMaxLevels * 32, L.ks));
    TTG_CUDA_CHECK(cudaMemsetAsync(L.status, 0, sizeof(int) * 8, L.ks));
    TTG_CUDA_CHECK(cudaMemsetAsync(L.pub, 0, sizeof(int) * 4, L.ks));
    TTG_CUDA_CHECK(cudaMemsetAsync(L.admit, 0, sizeof(int) * 2, L.ks));
    // The copy stream publishes only after the reset.
    TTG_CUDA_CHECK(cudaEventRecord(L.kdone, L.ks));
    TTG_CUDA_CHECK(cudaStreamWaitEvent(L.cs, L.kdone, 0));
    L.n_tasks = L.n_roots = L.n_teams = L.n_parts = 0;
    L.n_edges = 0;
    ttg::ExecParams p{};
    p.ops = L.ops;
    p.n_tasks = kOpenTasks;
    p.n_runnable = 0;
    p.count = L.count;
    p.runs = L.runs;
    p.parts = L.parts;
    p.part_next = L.part_next;
    p.part_done = L.part_done;
    p.succ_ptr = L.succ_ptr;
    p.succ_idx = L.succ_idx;
    p.level = L.level;
    p.bind = L.bind;
    p.n_levels = 1;
    p.n_workers = L.ctx->workers;
    p.qbuf = L.qbuf;
    p.q_off = L.q_off;
    p.q_head = L.q_head;
    p.q_tail = L.q_tail;
    p.bq_buf = L.bq;
    p.bq_off = L.bq;
    p.bq_head = L.bq + (L.ctx->workers + 1);
    p.bq_tail = L.bq + 2 * (L.ctx->workers + 1);
    p.has_bound = 0;
    p.done = L.status + 0;
    p.err = L.status + 1;
    p.err_task = L.status + 2;
    p.err_info = L.status + 3;
    p.trace = nullptr;
    p.timeout_ns = (long long)(L.ctx->timeout_s * 1e9);
    p.team_ctr = L.team_ctr;
    p.team_slot = L.team_slot;
    p.pub = L.pub;
    p.roots = L.roots;
    p.admit = L.admit;
    ttg_mixed_set_tc(L.ctx, true);
    ttg_status st = ttg_launch_mixed(L.ctx, p, L.ks);
    if (st != TTG_OK) return st;
    TTG_CUDA_CHECK(cudaEventRecord(L.kdone, L.ks));
    ++s->launches;
    L.running = true;
    L.closing = false;
    return TTG_OK;
}

// Close the epoch: the launch ends once every published task has run.
ttg_status open_close(OpenLane& L) {
    if (!L.running || L.closing) return TTG_OK;
    L.closing = true;
    return ttg_stream_write_u32(L.cs, (uint32_t*)(L.pub + 2), 1u);
}

// Upper bound of the tasks of one request's graph (batch_graph.h, plus its
// last task): factor nb + nb(nb-1)/2 + (nb³-nb)/6 + nb(nb+1)/2 tasks, each
// solve nb² + nb, each refinement round 2 + nb(nb+2) + nb more, and the
// conversions around them.  Its edges stay within 8 and its parts within 32
// per task of the bound (tests/test_abi.py checks all three).
long open_task_bound(int N, int tile, int ir_steps) {
    System S;
    S.set_size(N, tile);
    const long nb = S.nb;
    const long fac = nb + nb * (nb - 1) / 2 + (nb * nb * nb - nb) / 6 + nb * (nb + 1) / 2;
    const long per_solve = nb * nb + nb;
    return fac + 2 * nb + per_solve + (long)(ir_steps + 1) * (2 + nb * (nb + 2) + per_solve + nb) + 1;
}

// The request's last task: after every sink of its graph.
void add_signal_task(Graph& g, int attempt, int* flag) {
    std::vector<char> has_succ(g.ops.size(), 0);
    for (auto& e : g.edges) has_succ[e.first] = 1;
    ttg_op sig{};
    sig.kind = ttg::kOpSignal;
    sig.prec = TTG_PREC_MIXED;
    sig.m = attempt;
    sig.c = flag;
    const int t = g.add(sig);
    for (int u = 0; u < t; ++u)
        if (!has_succ[u]) g.edge(u, t);
}

// Admit request i into lane L: operands on the side stream, its tasks (and a
// last task that raises its host flag) appended to the arena and published.
// false: it must wait — no room in this epoch (*full), no request slot free
// in this lane (*busy), or memory / its factor not ready (neither).
bool open_admit(ttg_serve* s, OpenLane& L, int i, bool* full, bool* busy, ttg_status* err) {
    *full = *busy = false;
    if (L.n_inflight >= kOpenInflight) {
        *busy = true;  // no request slot free: another lane, or later
        return false;
    }
    ServeRequest& q = s->req[i];
    Graph g;
    L.rs.clear();
    int n_hdr = 0;
    AdmitTarget T{L.ctx, s->side, &g, &L.rs, nullptr, &n_hdr, 0};
    // Room first, from upper bounds of the request's graph.
    {
        System S;
        S.set_size(q.N, q.tile);
        const long nb = S.nb;
        const long est = open_task_bound(q.N, q.tile, q.ir_steps);
        const bool fits_empty = est <= L.cap_tasks && 8 * est <= kOpenEdges && 32 * est <= kOpenParts && nb <= kOpenTeams &&
                                nb <= L.rs_cap;
        if (!fits_empty) {
            ttg_set_last_cuda_error(cudaErrorInvalidValue, "open lane: a request exceeds an empty epoch", __FILE__, __LINE__);
            *err = TTG_EINVAL;
            return true;
        }
        if (L.n_tasks + est > L.cap_tasks || L.n_edges + 8 * est > kOpenEdges || L.n_parts + 32 * est > kOpenParts ||
            L.n_teams + nb > kOpenTeams) {
            *full = true;
            return false;
        }
    }
    g_open_at = "admit: operands";
    if (!admit_to(s, T, i, err)) return false;
    if (*err != TTG_OK) return true;
    g_open_at = "admit: row scales";
    // Block-row scales of its tensor-core factorisation (after its input).
    if (!L.rs.empty()) {
        cudaError_t e = cudaMemcpyAsync(L.d_rs, L.rs.data(), sizeof(TcRowScaleItem) * L.rs.size(), cudaMemcpyHostToDevice, s->side);
        if (e != cudaSuccess) {
            *err = TTG_ECUDA;
            return true;
        }
        if ((*err = ttg_mixed_row_scales(L.d_rs, (int)L.rs.size(), s->side)) != TTG_OK) return true;
    }
    add_signal_task(g, ++q.attempt, s->d_flag + i);
    if ((*err = g.finish(false)) != TTG_OK) return true;
    const int n = (int)g.ops.size();
    const int base = L.n_tasks;
    const int64_t ebase = L.n_edges;
    std::vector<int> parts(n), team(n, -1), roots;
    std::vector<int64_t> ptr(n + 1);
    std::vector<int32_t> idx(g.idx.size()), bind(n, -1);
    std::vector<uint8_t> level(n, 0);
    int nparts = 0, nteam = 0;
    for (int t = 0; t < n; ++t) {
        parts[t] = ttg_task_parts(g.ops[t], true);
        nparts += parts[t];
        if (g.ops[t].kind == TTG_OP_POTRF_L && team_fits(g.ops[t].n)) team[t] = L.n_teams + nteam++;
        if (g.init[t] == 0) roots.push_back(base + t);
        ptr[t] = ebase + g.ptr[t];
    }
    ptr[n] = ebase + g.ptr[n];
    for (size_t e = 0; e < g.idx.size(); ++e) idx[e] = base + g.idx[e];
    if (base + n > L.cap_tasks || ebase + (int64_t)idx.size() > kOpenEdges || L.n_parts + nparts > kOpenParts ||
        L.n_teams + nteam > kOpenTeams) {
        ttg_set_last_cuda_error(cudaErrorInvalidValue, "open lane: a request's graph exceeds its bounds", __FILE__, __LINE__);
        *err = TTG_EINVAL;  // the bounds above are wrong
        return true;
    }
    // Into the arena after its operands, then published.
    int slot = -1;
    for (int k = 0; k < kOpenInflight && slot < 0; ++k)
        if (L.slot_req[k] < 0) slot = k;
    if (slot < 0) {
        *err = TTG_EINVAL;  // n_inflight said there was one
        return true;
    }
    g_open_at = "admit: publish copies";
    cudaEvent_t ready = L.ev[slot];
    auto ok = [&](cudaError_t e) { return e == cudaSuccess; };
    bool good = ok(cudaEventRecord(ready, s->side)) && ok(cudaStreamWaitEvent(L.cs, ready, 0)) &&
                ok(cudaMemcpyAsync(L.ops + base, g.ops.data(), sizeof(ttg_op) * n, cudaMemcpyHostToDevice, L.cs)) &&
                ok(cudaMemcpyAsync(L.count + base, g.init.data(), sizeof(int) * n, cudaMemcpyHostToDevice, L.cs)) &&
                ok(cudaMemcpyAsync(L.parts + base, parts.data(), sizeof(int) * n, cudaMemcpyHostToDevice, L.cs)) &&
                ok(cudaMemcpyAsync(L.level + base, level.data(), n, cudaMemcpyHostToDevice, L.cs)) &&
                ok(cudaMemcpyAsync(L.bind + base, bind.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, L.cs)) &&
                ok(cudaMemcpyAsync(L.succ_ptr + base, ptr.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, L.cs)) &&
                (idx.empty() || ok(cudaMemcpyAsync(L.succ_idx + ebase, idx.data(), sizeof(int32_t) * idx.size(), cudaMemcpyHostToDevice, L.cs))) &&
                ok(cudaMemcpyAsync(L.team_slot + base, team.data(), sizeof(int) * n, cudaMemcpyHostToDevice, L.cs)) &&
                ok(cudaMemcpyAsync(L.roots + L.n_roots, roots.data(), sizeof(int) * roots.size(), cudaMemcpyHostToDevice, L.cs)) &&
                ok(cudaMemsetAsync(L.runs + base, 0, sizeof(int) * n, L.cs)) &&
                ok(cudaMemsetAsync(L.part_next + base, 0, sizeof(int) * n, L.cs)) &&
                ok(cudaMemsetAsync(L.part_done + base, 0, sizeof(int) * n, L.cs)) &&
                (nteam == 0 || ok(cudaMemsetAsync(L.team_ctr + (size_t)L.n_teams * kTeamStride, 0,
                                                  sizeof(int) * (size_t)nteam * kTeamStride, L.cs)));
    if (!good) {
        ttg_set_last_cuda_error(cudaGetLastError(), "open lane publish", __FILE__, __LINE__);
        *err = TTG_ECUDA;
        return true;
    }
    L.n_tasks += n;
    L.n_edges += (int64_t)idx.size();
    L.n_parts += nparts;
    L.n_teams += nteam;
    L.n_roots += (int)roots.size();
    g_open_at = "admit: publish words";
    if ((*err = ttg_stream_write_u32(L.cs, (uint32_t*)L.pub, (uint32_t)L.n_tasks)) != TTG_OK) return true;
    if ((*err = ttg_stream_write_u32(L.cs, (uint32_t*)(L.pub + 1), (uint32_t)L.n_roots)) != TTG_OK) return true;
    L.slot_req[slot] = i;
    ++L.n_inflight;
    q.lane = (int)(&L - s->open.data());
    q.slot = slot;
    q.phase = 1;
    return true;
}

// The lane's executor failed (timeout, overcount, not positive definite):
// its status words, read after the launch ended.
ttg_status open_lane_error(OpenLane& L) {
    int h[4] = {0, 0, 0, 0};
    TTG_CUDA_CHECK(cudaMemcpy(h, L.status, sizeof(h), cudaMemcpyDeviceToHost));
    return (ttg_status)h[1];
}

// Completions of lane L: a raised flag starts the request's backward error on
// the side stream; a finished backward error ends the request (or retries it
// with twice the refinement rounds).  Returns the requests completed.
int open_poll(ttg_serve* s, OpenLane& L, std::deque<int>& queue, double t, ttg_status* err) {
    int done = 0;
    const bool mixed = s->a.precision == TTG_PREC_MIXED;
    const volatile int* flag = s->h_flag;
    for (int k = 0; k < kOpenInflight; ++k) {
        const int i = L.slot_req[k];
        if (i < 0) continue;
        ServeRequest& q = s->req[i];
        if (q.phase == 1 && flag[i] == q.attempt) {
            g_open_at = "poll: backward error";
            int slices = (q.N + kRowsPerBlock - 1) / kRowsPerBlock;
            L.h_items[k] = BwdItem{q.N, q.tile, s->a.nrhs, s->res[q.key].A64, q.B, q.X, L.d_acc + (size_t)k * 33};
            cudaError_t e = cudaMemcpyAsync(L.d_items + k, L.h_items + k, sizeof(BwdItem), cudaMemcpyHostToDevice, s->side);
            if (e == cudaSuccess) e = cudaMemsetAsync(L.d_acc + (size_t)k * 33, 0, sizeof(unsigned long long) * 33, s->side);
            if (e == cudaSuccess) {
                ttg_note_launch();
                serve_bwd_partial<<<dim3(1, slices), kRowsPerBlock, 0, s->side>>>(L.d_items + k);
                ttg_note_launch();
                serve_bwd_final<<<1, 128, 0, s->side>>>(L.d_items + k, 1, L.d_err + k);
                e = cudaGetLastError();
            }
            if (e == cudaSuccess) e = cudaMemcpyAsync(L.h_err + k, L.d_err + k, sizeof(double), cudaMemcpyDeviceToHost, s->side);
            if (e == cudaSuccess) e = cudaEventRecord(L.ev[k], s->side);
            if (e != cudaSuccess) {
                ttg_set_last_cuda_error(e, "open lane backward error", __FILE__, __LINE__);
                *err = TTG_ECUDA;
                return done;
            }
            q.phase = 2;
        } else if (q.phase == 2 && cudaEventQuery(L.ev[k]) == cudaSuccess) {
            g_open_at = "poll: completion";
            q.bwd = L.h_err[k];
            if (s->a.keep_results) {
                std::vector<double> v((size_t)q.N * s->a.nrhs);
                if (cudaMemcpy(v.data(), q.X, sizeof(double) * v.size(), cudaMemcpyDeviceToHost) != cudaSuccess) {
                    *err = TTG_ECUDA;
                    return done;
                }
                q.result.assign((size_t)q.N * s->a.nrhs, 0.0);
                for (int c = 0; c < s->a.nrhs; ++c)
                    for (int r = 0; r < q.N; ++r) q.result[r + (size_t)c * q.N] = v[c + (size_t)r * s->a.nrhs];
            }
            pool_free(q.B, s->side);
            pool_free(q.X, s->side);
            pool_free(q.R, s->side);
            pool_free(q.D32, s->side);
            pool_free(q.D64, s->side);
            pool_free(q.tc, s->side);
            s->used -= q.work_bytes;
            q.work_bytes = 0;
            Resident& r = s->res[q.key];
            r.complete = true;
            release_factor(s, q.key, s->side);
            L.slot_req[k] = -1;
            --L.n_inflight;
            q.phase = 0;
            q.lane = q.slot = -1;
            if (mixed && !(q.bwd <= s->a.tol) && q.retries < 2) {
                ++q.retries;
                ++s->retries;
                q.ir_steps *= 2;
                queue.push_front(i);
                continue;
            }
            q.done = true;
            q.finish = t;
            ++done;
        }
    }
    return done;
}

// The request loop with open lanes.
ttg_status serve_loop_open(ttg_serve* s, double t0, int* completed_out) {
    const int n = (int)s->req.size();
    const bool verbose = getenv("TTG_SERVE_VERBOSE") != nullptr;
    double next_report = 2.0;
    std::deque<int> queue;
    int next = 0, completed = 0;
    ttg_status st = TTG_OK;
    std::atomic<bool> stop{false};
    std::atomic<int> done_count{0};
    std::thread watch;
    if (verbose)
        watch = std::thread([&] {
            while (!stop) {
                std::this_thread::sleep_for(std::chrono::seconds(2));
                if (!stop)
                    fprintf(stderr, "[ttg serve] watchdog t %.1f s: completed %d, host thread at: %s\n", now_s() - t0,
                            done_count.load(), g_open_at.load());
            }
        });
    struct Join {
        std::atomic<bool>& stop;
        std::thread& w;
        ~Join() {
            stop = true;
            if (w.joinable()) w.join();
        }
    } join{stop, watch};
    while (completed < n) {
        done_count = completed;
        g_open_at = "loop";
        const double t = now_s() - t0;
        bool progress = false;
        while (next < n && s->req[next].arrival <= t) {
            queue.push_back(next++);
            progress = true;
        }
        for (OpenLane& L : s->open) {
            const int d = open_poll(s, L, queue, now_s() - t0, &st);
            if (st != TTG_OK) return st;
            completed += d;
            progress = progress || d > 0;
            if (L.running && cudaEventQuery(L.kdone) == cudaSuccess) {
                // The launch ended: after its close once its requests are
                // through, or early by an error (a request still in flight
                // would never be done).
                if ((st = open_lane_error(L)) != TTG_OK) return st;
                if (L.n_inflight > 0) {
                    // Every request of a closed epoch raises its flag before
                    // the launch ends; poll once more before calling it lost.
                    const int d2 = open_poll(s, L, queue, now_s() - t0, &st);
                    if (st != TTG_OK) return st;
                    completed += d2;
                    bool lost = false;
                    for (int k = 0; k < kOpenInflight; ++k)
                        if (L.slot_req[k] >= 0 && s->req[L.slot_req[k]].phase == 1) lost = true;
                    if (lost) {
                        ttg_set_last_cuda_error(cudaErrorLaunchFailure, "open lane: the launch ended before a request was done",
                                                __FILE__, __LINE__);
                        return TTG_ETIMEOUT;
                    }
                    continue;  // backward errors still running
                }
                L.running = false;
                L.closing = false;  // free for the next epoch
                progress = true;
            }
        }
        // Admission: each waiting request, in arrival order, into the open
        // lane with the fewest requests in flight; a lane whose epoch is full
        // closes (a new epoch starts once its launch has ended).
        for (auto it = queue.begin(); it != queue.end();) {
            const int i = *it;
            bool admitted = false;
            std::vector<OpenLane*> order;
            for (OpenLane& L : s->open)
                if (!L.closing) order.push_back(&L);
            std::sort(order.begin(), order.end(), [](const OpenLane* a, const OpenLane* b) { return a->n_inflight < b->n_inflight; });
            for (OpenLane* L : order) {
                if (!L->running && (st = open_epoch_start(s, *L)) != TTG_OK) return st;
                bool full = false, busy = false;
                admitted = open_admit(s, *L, i, &full, &busy, &st);
                if (st != TTG_OK) return st;
                if (admitted) break;
                if (busy) continue;
                if (full) {
                    if ((st = open_close(*L)) != TTG_OK) return st;
                    continue;
                }
                break;  // memory, or its factor is not ready: it waits
            }
            if (admitted) {
                it = queue.erase(it);
                progress = true;
            } else {
                ++it;
            }
        }
        bool any = false;
        for (OpenLane& L : s->open) any = any || L.n_inflight > 0 || L.closing;
        if (!any && !queue.empty() && !progress) return TTG_ENOMEM;  // nothing in flight and nothing admitted
        if (verbose && now_s() - t0 > next_report) {
            next_report += 2.0;
            fprintf(stderr, "[ttg serve] t %.1f s: completed %d of %d, waiting %zu, arrived %d\n", now_s() - t0, completed, n,
                    queue.size(), next);
            for (const OpenLane& L : s->open)
                fprintf(stderr,
                        "[ttg serve]   lane: running %d closing %d in flight %d, tasks %d roots %d parts %d edges %lld; "
                        "copies idle %d, launch ended %d, side idle %d\n",
                        (int)L.running, (int)L.closing, L.n_inflight, L.n_tasks, L.n_roots, L.n_parts, (long long)L.n_edges,
                        (int)(cudaStreamQuery(L.cs) == cudaSuccess), (int)(cudaEventQuery(L.kdone) == cudaSuccess),
                        (int)(cudaStreamQuery(s->side) == cudaSuccess));
        }
        if (!progress) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    g_open_at = "drain";
    for (OpenLane& L : s->open)
        if ((st = open_close(L)) != TTG_OK) return st;
    for (OpenLane& L : s->open) {
        cudaStreamSynchronize(L.cs);
        cudaStreamSynchronize(L.ks);
        if (L.running && (st = open_lane_error(L)) != TTG_OK) return st;
        L.running = false;
    }
    cudaStreamSynchronize(s->side);
    *completed_out = completed;
    return TTG_OK;
}

}  // namespace

extern "C" ttg_status ttg_serve_create(int device, const ttg_serve_args* a, ttg_serve** out) {
    if (!a || !out || a->n_requests < 1 || !(a->rate > 0) || a->n_min < 1 || a->n_max < a->n_min || a->n_max > 131072 ||
        a->nrhs < 1 || a->nrhs > 16 || a->lanes < 1 || a->max_batch < 1 || !(a->hbm_budget_gb > 0) || a->ir_steps < 0 ||
        (a->precision != TTG_PREC_F64 && a->precision != TTG_PREC_MIXED) || a->admission < 0 || a->admission > 1 ||
        (a->admission == 1 && a->precision != TTG_PREC_MIXED))
        return TTG_EINVAL;
    *out = nullptr;
    TTG_CUDA_CHECK(cudaSetDevice(device));
    ttg_serve* s = new ttg_serve();
    s->device = device;
    s->a = *a;
    s->budget = (size_t)(a->hbm_budget_gb * 1e9);
    cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, device);
    // Requests.
    s->req.resize(a->n_requests);
    std::vector<int> factors;
    double t = 0.0;
    const double lo = std::log((double)a->n_min), hi = std::log((double)a->n_max);
    for (int i = 0; i < a->n_requests; ++i) {
        ServeRequest& q = s->req[i];
        if (i > 0) t += -std::log(1.0 - u01_at(a->seed, i, 0)) / a->rate;
        q.arrival = t;
        q.seed_b = a->seed + (uint32_t)i;
        q.ir_steps = a->ir_steps;
        if (!factors.empty() && u01_at(a->seed, i, 1) < a->followup_frac) {
            const int window = std::min<int>(32, (int)factors.size());
            const int pick = std::min(window - 1, (int)(u01_at(a->seed, i, 2) * window));
            const int tgt = factors[factors.size() - 1 - pick];
            q.followup_of = tgt;
            q.N = s->req[tgt].N;
            q.seed_a = s->req[tgt].seed_a;
        } else {
            q.N = std::min(a->n_max, std::max(a->n_min, (int)std::lround(std::exp(lo + u01_at(a->seed, i, 3) * (hi - lo)))));
            q.seed_a = a->seed + (uint32_t)i;
            factors.push_back(i);
        }
        q.tile = ttg_serve_tile(q.N);
    }
    if (a->admission == 1 && a->precision == TTG_PREC_MIXED) {
        // Open lanes, with half the SMs (TTG_SERVE_SPARE_SMS sets the count)
        // left to the side stream's kernels: at 1000 requests/s on two lanes
        // 16, 48 and 76 spare SMs gave 36, 91 and 127 solves/s — the input
        // generators are the side stream's largest share.
        int spare = s->sms / 2;
        if (const char* v = getenv("TTG_SERVE_SPARE_SMS")) spare = std::max(1, std::min(s->sms - a->lanes, atoi(v)));
        const int workers = std::max(1, (s->sms - spare) / a->lanes);
        cudaError_t e = cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaHostAlloc((void**)&s->h_flag, sizeof(int) * (size_t)a->n_requests, cudaHostAllocMapped);
        if (e == cudaSuccess) {
            memset(s->h_flag, 0, sizeof(int) * (size_t)a->n_requests);
            e = cudaHostGetDevicePointer((void**)&s->d_flag, s->h_flag, 0);
        }
        if (e != cudaSuccess) {
            ttg_set_last_cuda_error(e, "serve open set-up", __FILE__, __LINE__);
            ttg_serve_destroy(s);
            return TTG_ECUDA;
        }
        // Every kernel the side stream launches is loaded before the first
        // lane starts: with lazy module loading a first launch waits for the
        // device to be idle, and a lane's executor is never idle until closed.
        cudaFuncAttributes fa;
        ttg_status pst = ttg_gen_preload();
        if (pst == TTG_OK) pst = ttg_mixed_row_scales_preload();
        if (pst == TTG_OK && (cudaFuncGetAttributes(&fa, serve_bwd_partial) != cudaSuccess ||
                              cudaFuncGetAttributes(&fa, serve_bwd_final) != cudaSuccess))
            pst = TTG_ECUDA;
        if (pst != TTG_OK) {
            ttg_serve_destroy(s);
            return pst;
        }
        s->open.resize(a->lanes);
        for (OpenLane& L : s->open) {
            ttg_status st = open_lane_setup(s, L, workers);
            if (st != TTG_OK) {
                ttg_serve_destroy(s);
                return st;
            }
        }
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t thr = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
        *out = s;
        return TTG_OK;
    }
    // Lanes: one executor context and stream each.
    const int workers = std::max(1, s->sms / a->lanes);
    s->lanes.resize(a->lanes);
    const int maxb = a->max_batch;
    for (Lane& L : s->lanes) {
        ttg_opts o{};
        o.device = device;
        o.workers = workers;
        o.timeout_s = 60.0;
        ttg_status st = ttg_create(&L.ctx, &o);
        cudaError_t e = cudaSuccess;
        if (st == TTG_OK) {
            L.ctx->coop = false;  // lanes share the GPU
            e = cudaStreamCreateWithFlags(&L.s, cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&L.done, cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaMallocHost((void**)&L.h_items, sizeof(BwdItem) * maxb);
            if (e == cudaSuccess) e = cudaMalloc((void**)&L.d_items, sizeof(BwdItem) * maxb);
            if (e == cudaSuccess) e = cudaMalloc((void**)&L.d_acc, sizeof(unsigned long long) * 33 * maxb);
            if (e == cudaSuccess) e = cudaMallocHost((void**)&L.h_err, sizeof(double) * maxb);
            if (e == cudaSuccess) e = cudaMalloc((void**)&L.d_err, sizeof(double) * maxb);
            // Diagonal tiles of the launch's factorisations: nb <= n_max / 128 + 1.
            L.rs_cap = maxb * (a->n_max / 128 + 2);
            if (e == cudaSuccess) e = cudaMallocHost((void**)&L.h_hdr, kTcHeaderBytes * (size_t)maxb);
            if (e == cudaSuccess) e = cudaMallocHost((void**)&L.h_rs, sizeof(TcRowScaleItem) * (size_t)L.rs_cap);
            if (e == cudaSuccess) e = cudaMalloc((void**)&L.d_rs, sizeof(TcRowScaleItem) * (size_t)L.rs_cap);
        }
        if (st != TTG_OK || e != cudaSuccess) {
            if (e != cudaSuccess) ttg_set_last_cuda_error(e, "serve lane set-up", __FILE__, __LINE__);
            ttg_serve_destroy(s);
            return st != TTG_OK ? st : TTG_ECUDA;
        }
    }
    // Keep freed request memory in the pool (no release to the driver between requests).
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    *out = s;
    return TTG_OK;
}

extern "C" void ttg_serve_destroy(ttg_serve* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    for (OpenLane& L : s->open) {
        open_close(L);  // a running epoch ends once its published tasks have run
        open_lane_free(L);
    }
    if (s->side) {
        cudaStreamSynchronize(s->side);
        cudaStreamDestroy(s->side);
    }
    if (s->h_flag) cudaFreeHost(s->h_flag);
    for (Lane& L : s->lanes)
        if (L.s) cudaStreamSynchronize(L.s);
    for (auto& kv : s->res) {
        Resident& r = kv.second;
        for (void* p : {(void*)r.A64, (void*)r.W64, (void*)r.W32})
            if (p) cudaFree(p);
    }
    for (ServeRequest& q : s->req)
        for (void* p : {(void*)q.B, (void*)q.X, (void*)q.R, (void*)q.D32, (void*)q.D64, (void*)q.tc})
            if (p) cudaFree(p);
    for (Lane& L : s->lanes) {
        if (L.ctx) ttg_destroy(L.ctx);
        if (L.done) cudaEventDestroy(L.done);
        if (L.s) cudaStreamDestroy(L.s);
        if (L.h_items) cudaFreeHost(L.h_items);
        if (L.d_items) cudaFree(L.d_items);
        if (L.h_hdr) cudaFreeHost(L.h_hdr);
        if (L.h_rs) cudaFreeHost(L.h_rs);
        if (L.d_rs) cudaFree(L.d_rs);
        if (L.d_acc) cudaFree(L.d_acc);
        if (L.h_err) cudaFreeHost(L.h_err);
        if (L.d_err) cudaFree(L.d_err);
    }
    delete s;
}

extern "C" ttg_status ttg_serve_run(ttg_serve* s, ttg_serve_report* rep, double* h_latency_ms) {
    if (!s) return TTG_EINVAL;
    TTG_CUDA_CHECK(cudaSetDevice(s->device));
    const int n = (int)s->req.size();
    std::deque<int> queue;
    int next = 0, completed = 0;
    const double t0 = now_s();
    ttg_status st = TTG_OK;
    if (!s->open.empty()) {
        st = serve_loop_open(s, t0, &completed);
        if (st != TTG_OK) {
            for (OpenLane& L : s->open) {
                open_close(L);
                cudaStreamSynchronize(L.cs);
                cudaStreamSynchronize(L.ks);
            }
            return st;
        }
    }
    while (completed < n && st == TTG_OK) {
        const double t = now_s() - t0;
        bool progress = false;
        while (next < n && s->req[next].arrival <= t) {
            queue.push_back(next++);
            progress = true;
        }
        for (Lane& L : s->lanes) {
            if (L.busy && cudaEventQuery(L.done) == cudaSuccess) {
                if ((st = complete(s, L, queue, now_s() - t0)) != TTG_OK) break;
                for (int i : L.reqs) completed += s->req[i].done;
                progress = true;
            }
        }
        if (st != TTG_OK) break;
        bool any_busy = false;
        for (Lane& L : s->lanes) {
            if (!L.busy && !queue.empty()) {
                if ((st = dispatch(s, L, queue)) != TTG_OK) break;
                progress = progress || L.busy;
            }
            any_busy = any_busy || L.busy;
        }
        if (st != TTG_OK) break;
        // Nothing running and nothing admitted: the waiting requests cannot
        // fit the budget even with every idle factor evicted.
        if (!any_busy && !queue.empty()) {
            st = TTG_ENOMEM;
            break;
        }
        if (!progress) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    for (Lane& L : s->lanes) cudaStreamSynchronize(L.s);
    if (st != TTG_OK) return st;
    // Statistics.
    std::vector<double> lat(n);
    double fl = 0.0, worst = 0.0, last = 0.0;
    int factorisations = 0, followups = 0, unconv = 0;
    for (int i = 0; i < n; ++i) {
        const ServeRequest& q = s->req[i];
        lat[i] = (q.finish - q.arrival) * 1e3;
        last = std::max(last, q.finish);
        if (q.followup_of < 0) {
            ++factorisations;
            fl += (double)q.N * q.N * q.N / 3.0;
        } else {
            ++followups;
        }
        worst = std::max(worst, q.bwd);
        if (!(q.bwd <= s->a.tol)) ++unconv;
    }
    if (h_latency_ms) std::copy(lat.begin(), lat.end(), h_latency_ms);
    if (rep) {
        std::vector<double> sorted = lat;
        std::sort(sorted.begin(), sorted.end());
        auto pct = [&](double p) { return sorted[std::min<size_t>(n - 1, (size_t)std::floor(p * (n - 1) + 0.5))]; };
        ttg_serve_report r{};
        r.completed = completed;
        r.factorisations = factorisations;
        r.followups = followups;
        r.followup_misses = s->misses;
        r.evictions = s->evictions;
        r.launches = s->launches;
        r.retries = s->retries;
        r.unconverged = unconv;
        r.wall_s = last;
        r.p50_ms = pct(0.50);
        r.p99_ms = pct(0.99);
        double sum = 0.0;
        for (double v : lat) sum += v;
        r.mean_ms = sum / n;
        r.max_ms = sorted.back();
        r.solves_per_s = last > 0 ? n / last : 0.0;
        r.tflops = last > 0 ? fl / last / 1e12 : 0.0;
        r.worst_bwd_err = worst;
        r.peak_gb = s->peak / 1e9;
        *rep = r;
    }
    return TTG_OK;
}

extern "C" ttg_status ttg_serve_request(const ttg_serve* s, int32_t i, int32_t* n, int32_t* tile, uint32_t* seed_a, uint32_t* seed_b,
                                        double* arrival_s, int32_t* followup_of, double* bwd_err, int32_t* ir_steps) {
    if (!s || i < 0 || i >= (int)s->req.size()) return TTG_EINVAL;
    const ServeRequest& q = s->req[i];
    if (n) *n = q.N;
    if (tile) *tile = q.tile;
    if (seed_a) *seed_a = q.seed_a;
    if (seed_b) *seed_b = q.seed_b;
    if (arrival_s) *arrival_s = q.arrival;
    if (followup_of) *followup_of = q.followup_of;
    if (bwd_err) *bwd_err = q.bwd;
    if (ir_steps) *ir_steps = q.ir_steps;
    return TTG_OK;
}

extern "C" ttg_status ttg_serve_get_x(const ttg_serve* s, int32_t i, double* h_X) {
    if (!s || !h_X || i < 0 || i >= (int)s->req.size()) return TTG_EINVAL;
    const ServeRequest& q = s->req[i];
    if (!q.done || q.result.empty()) return TTG_ESTATE;
    std::copy(q.result.begin(), q.result.end(), h_X);
    return TTG_OK;
}

// Test hook (no device work): the open-lane bound of one request and the
// graph it admits — a system of N (tile, nrhs, ir_steps; mixed or FP64;
// factored = a follow-up's solve only; tc = tensor-core updates where the
// tiles allow) plus its last task.  out[5]: the bound, tasks, edges, parts
// (as the executor counts them), tile rows.  Never dereferences the fake
// device addresses it builds the ops with.
extern "C" ttg_status ttg_internal_open_request_graph(int32_t N, int32_t tile, int32_t nrhs, int32_t ir_steps, int32_t mixed,
                                                      int32_t factored, int32_t tc, int64_t* out) {
    if (N < 1 || tile < 1 || nrhs < 1 || ir_steps < 0 || !out) return TTG_EINVAL;
    using namespace ttg::batch;
    System S;
    S.set_size(N, tile);
    S.mixed = mixed != 0;
    S.nrhs = nrhs;
    S.ir_steps = ir_steps;
    S.factored = factored != 0;
    static char fake[64];  // stands in for every device array (never read)
    S.A64 = S.W64 = S.D64 = S.B = S.X = S.R = (double*)fake;
    S.W32 = S.D32 = (float*)fake;
    if (S.mixed && tc && System::tc_fits(S.N, S.tile)) S.tc_tables = fake;
    Graph g;
    add_system(g, S);
    add_signal_task(g, 1, (int*)fake);
    const ttg_status st = g.finish(false);
    if (st != TTG_OK) return st;
    int64_t parts = 0;
    for (const ttg_op& op : g.ops) parts += ttg_task_parts(op, true);
    out[0] = open_task_bound(N, S.tile, ir_steps);
    out[1] = (int64_t)g.ops.size();
    out[2] = (int64_t)g.idx.size();
    out[3] = parts;
    out[4] = S.nb;
    return TTG_OK;
}
