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
#include <chrono>
#include <cmath>
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

struct ttg_serve {
    int device = 0, sms = 0;
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
bool admit(ttg_serve* s, Lane& L, int i, ttg_status* err) {
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
        if (!need_factor) release_factor(s, key, L.s);
        return false;
    }
    cudaStream_t st = L.s;
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
        if (e == TTG_OK) e = ttg_gen_gram_async(L.ctx, q.N, q.tile, s->a.alpha, q.seed_a, r.A64, st);
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
        if (e == TTG_OK && need_factor && System::tc_fits(S.N, S.tile) && L.n_hdr < s->a.max_batch) {
            e = pool_alloc(&q.tc, tc_bytes(S), st);
            if (e == TTG_OK) {
                float* slot_scale = (float*)(q.tc + kTcHeaderBytes);
                float* rowscale = slot_scale + S.nb * (S.nb + 1) / 2;
                __nv_bfloat16* slots = (__nv_bfloat16*)(q.tc + kTcHeaderBytes + tc_scale_bytes(S));
                uint8_t* h = L.h_hdr + kTcHeaderBytes * (size_t)L.n_hdr;
                e = ttg_mixed_tc_header(h, q.tc, slots, slot_scale, rowscale, S.tile, S.nb, &S.tc_tables);
                if (e == TTG_OK)
                    e = cudaMemcpyAsync(q.tc, h, kTcHeaderBytes, cudaMemcpyHostToDevice, st) == cudaSuccess ? TTG_OK : TTG_ECUDA;
                if (e == TTG_OK) {
                    ++L.n_hdr;
                    for (int i = 0; i < S.nb; ++i) L.rs.push_back(TcRowScaleItem{r.A64 + S.off(i, i), S.bs(i), S.bs(i), rowscale + i});
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
    add_system(L.g, S);
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

extern "C" ttg_status ttg_serve_create(int device, const ttg_serve_args* a, ttg_serve** out) {
    if (!a || !out || a->n_requests < 1 || !(a->rate > 0) || a->n_min < 1 || a->n_max < a->n_min || a->n_max > 131072 ||
        a->nrhs < 1 || a->nrhs > 16 || a->lanes < 1 || a->max_batch < 1 || !(a->hbm_budget_gb > 0) || a->ir_steps < 0 ||
        (a->precision != TTG_PREC_F64 && a->precision != TTG_PREC_MIXED))
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
