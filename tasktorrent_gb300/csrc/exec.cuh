// exec.cuh — the persistent task-graph executor (replaces ttor::Threadpool_shared).
//
// Reference behaviour kept (tasktorrent/src/threadpool_shared.cpp):
//   - a task runs once its dependency counter reaches zero, then its
//     fulfill() decrements its successors (Taskflow::fulfill_promise,
//     taskflow.hpp:241-296) — here the successor lists are the edges recorded
//     on the host and the decrement is an atomicSub on a device counter;
//   - higher priority runs first (less_pTask, tasks.cpp:13-16) — here 32
//     priority levels, each a FIFO, scanned by the 32 lanes of warp 0;
//   - bound tasks run only on their mapped worker (insert(.., binding=true),
//     threadpool_shared.cpp:214-223) — here a per-worker queue;
//   - completion when no task is left (test_completion, :73-79) — here when the
//     completed count reaches the number of runnable tasks;
//   - a negative count is an error (taskflow.hpp:278-282) — here an atomicSub
//     that finds a counter already at zero sets TTG_EOVERCOUNT.
// Every wait is bounded: a worker that sees no progress for timeout_ns sets
// TTG_ETIMEOUT and returns; nothing traps.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ttg.h"

namespace ttg {

// Priority levels: kMaxLevels FIFO queues, scanned 32 at a time by the lanes
// of warp 0 (kLevelGroups loads per lane, issued together).
constexpr int kMaxLevels = 128;
constexpr int kLevelGroups = kMaxLevels / 32;
// Trace words per task: first-part start, release time, releasing worker,
// summed part durations (ns of the global timer).
constexpr int kTraceWords = 4;
// Counter words per team task (the POTRF tasks shared by several blocks).
constexpr int kTeamStride = 256;
// 128×256 tensor-core output blocks per part of a mixed-path GEMM update,
// run back to back in the part's block so that each block's epilogue
// overlaps the next block's MMAs (split-BF16 factorisation, N = 32768, tile
// 512: 99.0 ms with 2, 94.5 ms with 4, 95.1 ms with 8).
constexpr int kTcBlocksPerPart = 4;

struct ExecParams {
    const ttg_op* ops;
    int n_tasks;      // tasks in the graph
    int n_runnable;   // tasks that will reach zero
    int* count;       // dependency counters
    int* runs;        // per-task run count
    const int* parts; // blocks sharing each task (>= 1)
    int* part_next;   // next part index to hand out
    int* part_done;   // parts finished
    const int64_t* succ_ptr;
    const int32_t* succ_idx;
    const uint8_t* level;   // priority level, 0 = highest
    const int32_t* bind;    // -1 or worker
    int n_levels;
    int n_workers;
    int* qbuf;              // all level queues back to back
    const int* q_off;       // [n_levels + 1]
    int* q_head;            // [kMaxLevels * 32] (one 128-byte line per level)
    int* q_tail;
    int* bq_buf;            // per-worker bound queues back to back
    const int* bq_off;      // [n_workers + 1]
    int* bq_head;           // [n_workers]
    int* bq_tail;
    int has_bound;
    int* done;              // completed tasks
    int* err;               // first error status
    int* err_task;
    int* err_info;
    long long* trace;       // [kTraceWords * n_tasks] start, end, worker, busy; or null
    long long timeout_ns;
    int* team_ctr;          // kTeamStride words per team task, zero at launch; or null
    const int* team_slot;   // per task: its team counter block, -1 if none; or null
    // Open graph (a serving lane that takes new work while it runs), or null:
    // pub[0] tasks published, pub[1] roots published, pub[2] closed flag —
    // written by the host's copy stream after the tasks' data; roots[] the
    // published root tasks in order; admit[0] roots pushed so far, admit[1]
    // a lock held by the worker that pushes them.  The launch ends when the
    // graph is closed and every published task has run.
    const int* pub;
    const int* roots;
    int* admit;
};

// Internal op kind of open graphs: a request's last task, which writes op.m
// to the host-visible word op.c once every task it depends on has run.
constexpr int kOpSignal = 99;

__device__ __forceinline__ long long globaltimer() {
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ int ld_volatile(const int* p) { return *(const volatile int*)p; }
__device__ __forceinline__ void st_volatile(int* p, int v) { *(volatile int*)p = v; }

__device__ __forceinline__ void set_error(const ExecParams& p, int status, int task, int info) {
    if (atomicCAS(p.err, 0, status) == 0) {
        *p.err_task = task;
        *p.err_info = info;
    }
}

// Wait for a reserved queue slot to be written by its producer.  Returns the
// task id, or -1 after timeout (error already set).
__device__ inline int wait_slot(const ExecParams& p, int* slot) {
    long long t0 = 0;
    for (int it = 0;; ++it) {
        int v = ld_volatile(slot);
        if (v >= 0) return v;
        if ((it & 63) == 0) {
            long long now = globaltimer();
            if (it == 0) t0 = now;
            else if (now - t0 > p.timeout_ns) {
                set_error(p, TTG_ETIMEOUT, -1, 0);
                return -1;
            }
        }
    }
}

// The task tables are read through L2 only: an open graph appends entries
// while the launch runs, after a block may have cached their line in L1.
__device__ __forceinline__ int ld_tab(const int* a) { return __ldcg(a); }
__device__ __forceinline__ int64_t ld_tab(const int64_t* a) { return (int64_t)__ldcg((const long long*)a); }
__device__ __forceinline__ int ld_tab(const uint8_t* a) { return __ldcg((const unsigned char*)a); }
__device__ __forceinline__ ttg_op ld_op(const ttg_op* a) {
    static_assert(sizeof(ttg_op) % 8 == 0, "ttg_op words");
    ttg_op o;
    const unsigned long long* s = (const unsigned long long*)a;
    unsigned long long* d = (unsigned long long*)&o;
#pragma unroll
    for (int i = 0; i < (int)(sizeof(ttg_op) / 8); ++i) d[i] = __ldcg(s + i);
    return o;
}

__device__ inline void push_ready(const ExecParams& p, int s);

// Open graphs (lane 0 of an idle worker): push the roots published since the
// last admission onto their queues, under the admission lock.
__device__ inline void admit_roots(const ExecParams& p) {
    const int want = ld_volatile(p.pub + 1);
    if (ld_volatile(p.admit) >= want) return;
    if (atomicCAS(p.admit + 1, 0, 1) != 0) return;  // another worker is admitting
    __threadfence();
    const int have = ld_volatile(p.admit);
    const int upto = ld_volatile(p.pub + 1);
    __threadfence();  // the roots (and their tasks) were written before pub[1]
    for (int r = have; r < upto; ++r) push_ready(p, ld_volatile(p.roots + r));
    __threadfence();
    st_volatile(p.admit, upto);
    __threadfence();
    atomicExch(p.admit + 1, 0);
}

// Called by all lanes of warp 0.  Returns a claimed task id and its part
// (*part, the same on all lanes), or -1 to exit.
//
// Queues hold one slot per part of a ready task.  A level queue is a
// counting semaphore over its slots: q_tail[lvl·32] reserves slots for the
// producers, q_tail[lvl·32 + 1] counts the slots written and not yet claimed
// ("available", raised after the writes), q_head[lvl·32] hands out slots.  A
// claimer reserves with an atomic decrement of the available count (undone
// when it was empty) and then takes the next slot with an atomic increment
// of the head: two fetch-and-adds, no retried compare-and-swap, so claims do
// not serialise on the head.  The part index comes from the task's part
// counter.  A bound queue (one worker) is read in order.
__device__ inline int claim_task(const ExecParams& p, int* part) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x;
    int last_done = -1, last_target = -1;
    long long idle_since = 0;
    {
        int e = 0;
        if (lane == 0) e = ld_volatile(p.err);
        if (__shfl_sync(0xffffffffu, e, 0) != 0) return -1;
    }
    for (unsigned spin = 0;; ++spin) {
        if (p.has_bound) {
            int task = -1;
            if (lane == 0) {
                const int h = p.bq_head[w];
                if (h < ld_volatile(p.bq_tail + w)) {
                    task = wait_slot(p, p.bq_buf + p.bq_off[w] + h);
                    if (task >= 0) p.bq_head[w] = h + 1;
                    else task = -2;
                }
            }
            task = __shfl_sync(0xffffffffu, task, 0);
            if (task == -2) return -1;
            if (task >= 0) {
                int pt = 0;
                if (lane == 0) pt = atomicAdd(p.part_next + task, 1);
                *part = __shfl_sync(0xffffffffu, pt, 0);
                __threadfence();
                return task;
            }
        }
        int av[kLevelGroups];
#pragma unroll
        for (int g = 0; g < kLevelGroups; ++g) {
            const int l = g * 32 + lane;
            av[g] = l < p.n_levels ? ld_volatile(p.q_tail + l * 32 + 1) : 0;
        }
        unsigned mask = 0;
        int grp = 0;
#pragma unroll
        for (int g = kLevelGroups - 1; g >= 0; --g) {
            const unsigned m = __ballot_sync(0xffffffffu, g * 32 + lane < p.n_levels && av[g] > 0);
            if (m) {
                mask = m;
                grp = g;
            }
        }
        if (mask) {
            const int lvl = grp * 32 + __ffs(mask) - 1;
            int got = -1, pt = 0;
            if (lane == (lvl & 31)) {
                if (atomicSub(p.q_tail + lvl * 32 + 1, 1) > 0) {
                    // Reserved: slot k exists; its producer may still be writing it.
                    const int k = atomicAdd(p.q_head + lvl * 32, 1);
                    const int t = wait_slot(p, p.qbuf + p.q_off[lvl] + k);
                    if (t < 0) {
                        got = -2;
                    } else {
                        pt = atomicAdd(p.part_next + t, 1);
                        got = t;
                    }
                } else {
                    atomicAdd(p.q_tail + lvl * 32 + 1, 1);  // it was empty: undo
                }
            }
            got = __shfl_sync(0xffffffffu, got, lvl & 31);
            if (got == -2) return -1;
            if (got >= 0) {
                *part = __shfl_sync(0xffffffffu, pt, lvl & 31);
                __threadfence();
                return got;
            }
            continue;  // lost the race for the last slots; rescan at once
        }
        int d = 0, e = 0, target = p.n_runnable, closed = 1;
        if (lane == 0) {
            if (p.pub) {
                // The closed flag first: once it is seen, pub[0] is final.
                admit_roots(p);
                closed = ld_volatile(p.pub + 2);
                __threadfence();
                target = ld_volatile(p.pub);
                __threadfence();
            }
            d = ld_volatile(p.done);
            e = ld_volatile(p.err);
        }
        d = __shfl_sync(0xffffffffu, d, 0);
        e = __shfl_sync(0xffffffffu, e, 0);
        target = __shfl_sync(0xffffffffu, target, 0);
        closed = __shfl_sync(0xffffffffu, closed, 0);
        if ((closed && d >= target) || e != 0) return -1;
        long long now = 0;
        if (lane == 0) now = globaltimer();
        now = __shfl_sync(0xffffffffu, now, 0);
        // An open graph with every published task done waits for more work
        // (or its closing) up to ten times the no-progress limit.
        const bool waiting = d >= target;
        if (d != last_done || target != last_target) {
            last_done = d;
            last_target = target;
            idle_since = now;
        } else if (now - idle_since > (waiting ? 10 * p.timeout_ns : p.timeout_ns)) {
            if (lane == 0) set_error(p, TTG_ETIMEOUT, -1, 0);
            return -1;
        }
        __nanosleep(spin < 64 ? 32 : 256);
    }
}

__device__ __forceinline__ void push_ready(const ExecParams& p, int s) {
    const int b = ld_tab(p.bind + s);
    const int P = ld_tab(p.parts + s);
    // Every task is pushed at most once (only the decrement that finds the
    // counter at one pushes), so a queue never outgrows the number of tasks
    // assigned to it; the bound checks below only guard against a corrupted
    // graph.
    // A task of P parts takes P consecutive slots, one per part.
    if (b >= 0) {
        const int w = b % p.n_workers;
        const int slot = atomicAdd(p.bq_tail + w, P);
        if (p.bq_off[w] + slot + P <= p.bq_off[w + 1]) {
            for (int q = 0; q < P; ++q) st_volatile(p.bq_buf + p.bq_off[w] + slot + q, s);
        } else {
            set_error(p, TTG_EOVERCOUNT, s, 0);
        }
    } else {
        const int lvl = ld_tab(p.level + s);
        const int slot = atomicAdd(p.q_tail + lvl * 32, P);
        if (p.q_off[lvl] + slot + P <= p.q_off[lvl + 1]) {
            for (int q = 0; q < P; ++q) st_volatile(p.qbuf + p.q_off[lvl] + slot + q, s);
            __threadfence();
            atomicAdd(p.q_tail + lvl * 32 + 1, P);  // available once written
        } else {
            set_error(p, TTG_EOVERCOUNT, s, 0);
        }
    }
}

// Called by all lanes of warp 0 after the block finished task t.
__device__ inline void fulfil_successors(const ExecParams& p, int t) {
    const int lane = threadIdx.x & 31;
    __threadfence();  // release the tile writes of the whole block (after bar.sync)
    const int64_t e0 = ld_tab(p.succ_ptr + t), e1 = ld_tab(p.succ_ptr + t + 1);
    for (int64_t e = e0 + lane; e < e1; e += 32) {
        const int s = ld_tab(p.succ_idx + e);
        const int old = atomicSub(p.count + s, 1);
        if (old == 1) {
            __threadfence();
            push_ready(p, s);
        } else if (old < 1) {
            set_error(p, TTG_EOVERCOUNT, s, 0);
        }
    }
    __syncwarp();
    if (lane == 0) {
        atomicAdd(p.runs + t, 1);
        __threadfence();
        atomicAdd(p.done, 1);
    }
}

// The persistent kernel body: `RunOp(op, part, parts, smem, team, fin)` runs
// one part of a tile task on the whole block and returns 0 or an error info
// (POTRF failing column); team is the task's team counter block or null.  The
// block that finishes the last part of a task fulfils its successors — except
// for team tasks, whose parts set *fin (shared, -1 on entry) to 1 in the block
// that completed the work and to 0 elsewhere: that block fulfils at once, and
// parts that start later find nothing left to do.
template <class RunOp>
__device__ void executor_loop(const ExecParams& p, double* smem, RunOp run_op) {
    __shared__ int s_task, s_part, s_info, s_last, s_fin;
    long long t_part = 0;  // thread 0: start of the current part (trace)
    for (;;) {
        if (threadIdx.x < 32) {
            int part = 0;
            const int t = claim_task(p, &part);
            if (threadIdx.x == 0) {
                s_task = t;
                s_fin = -1;
                if (t >= 0) {
                    s_part = part;
                    if (p.trace) {
                        t_part = globaltimer();
                        if (part == 0) p.trace[kTraceWords * (size_t)t] = t_part;
                    }
                }
            }
        }
        __syncthreads();
        const int t = s_task;
        if (t < 0) break;
        const ttg_op op = ld_op(p.ops + t);
        const int nparts = ld_tab(p.parts + t);
        int* team = nullptr;
        if (p.team_slot) {
            const int slot = ld_tab(p.team_slot + t);
            if (slot >= 0) team = p.team_ctr + (size_t)slot * kTeamStride;
        }
        const int info = run_op(op, s_part, nparts, smem, team, &s_fin);
        __syncthreads();
        if (threadIdx.x == 0) {
            s_info = info;
            __threadfence();  // release this part's writes (after bar.sync)
            const int finished = atomicAdd(p.part_done + t, 1);
            s_last = s_fin >= 0 ? s_fin == 1 : finished == nparts - 1;
            if (s_last) __threadfence();  // acquire the other parts' writes
            if (p.trace) atomicAdd((unsigned long long*)(p.trace + kTraceWords * (size_t)t + 3),
                                   (unsigned long long)(globaltimer() - t_part));
        }
        __syncwarp();
        if (threadIdx.x < 32) {
            if (threadIdx.x == 0 && s_info != 0) set_error(p, TTG_ENOTPD, t, s_info);
            if (s_last) {
                if (threadIdx.x == 0 && p.trace) {
                    p.trace[kTraceWords * (size_t)t + 1] = globaltimer();
                    p.trace[kTraceWords * (size_t)t + 2] = blockIdx.x;
                }
                fulfil_successors(p, t);
            }
        }
        __syncthreads();  // s_task/s_part are rewritten by the next claim
    }
}

}  // namespace ttg
