// ttor::Threadpool_shared for GB300 — same interface as the reference
// (tasktorrent/src/threadpool_shared.hpp:79-126), different engine.
//
// The reference runs Task closures on n CPU threads with work stealing
// (threadpool_shared.cpp:81-198).  Here the closures run once on the host in
// *capture* order when join() is called: each task body records the tile
// operations it would have computed (ttor::gpu::cblas_dgemm, LAPACKE_dpotrf,
// ... in gpu_blas.hpp) and the promises it makes (Taskflow::fulfill_promise).
// join() then uploads that task graph through the C ABI (include/ttg.h) and
// one persistent kernel executes it on the GPU: blocks pop ready tasks from
// device queues by priority and decrement successor counters with atomics.
//
// Kept from the reference:
//   - constructor arguments, start()/insert()/join()/is_done()/set_logger()/size();
//   - insert() takes ownership of the Task (deleted after it ran);
//   - `where` must be in [0, size()) (threadpool_shared.cpp:205-209);
//   - bound tasks (binding = true) run mutually exclusively on one worker;
//   - priorities order ready tasks (higher first);
//   - seeding may happen before or after start(); join() returns when every
//     task that became ready has run.
// Differences (documented, by construction of a device executor):
//   - host side effects of task bodies happen during the capture, before the
//     device runs the recorded tile operations; a task graph must not depend
//     on values computed by the tile operations;
//   - size() is the mapping modulus (the reference's thread count); the
//     device uses one persistent block per SM unless set_workers() says
//     otherwise.
#ifndef TTOR_GB300_THREADPOOL_SHARED_HPP
#define TTOR_GB300_THREADPOOL_SHARED_HPP

#include <algorithm>
#include <array>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <functional>
#include <memory>
#include <mutex>
#include <queue>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../../include/ttg.h"
#include "tasks.hpp"
#include "util.hpp"

namespace ttor {

namespace detail {

// One captured task (a node of the device graph).
struct Node {
    std::unique_ptr<Task> task;          // closures; run once during capture
    std::function<std::string()> name;   // evaluated lazily (logs and dumps)
    double priority = 0.0;
    int bind = -1;                       // worker for bound tasks
    int indegree = 1;                    // f_indegree(k)
    int promises = 0;                    // promises received (root and tasks)
    int in_edges = 0;                    // promises received from tasks
    bool ready = false;
    bool ran = false;
    std::vector<ttg_op> ops;             // recorded tile operations
    std::vector<int> succ;               // nodes promised by this task (one per call)
};

struct Capture;
inline Capture*& current_capture() {
    static thread_local Capture* c = nullptr;
    return c;
}

struct Capture {
    std::vector<Node> nodes;
    int current = -1;                    // node whose closures are running
    void record_op(const ttg_op& op) {
        if (current < 0) throw std::logic_error("ttor::gpu: tile operation called outside a task body");
        nodes[current].ops.push_back(op);
    }
};

// Process-wide default device context.
inline ttg_ctx*& default_ctx_slot() {
    static ttg_ctx* c = nullptr;
    return c;
}

}  // namespace detail

namespace gpu {

// The device context used by thread pools that were not given one.  Created
// on first use on device $TTG_DEVICE (default 0).
inline ttg_ctx* default_context() {
    ttg_ctx*& c = detail::default_ctx_slot();
    if (!c) {
        ttg_opts o{};
        const char* dev = getenv("TTG_DEVICE");
        o.device = dev ? atoi(dev) : 0;
        o.timeout_s = 30.0;
        ttg_status s = ttg_create(&c, &o);
        if (s != TTG_OK) {
            c = nullptr;
            throw std::runtime_error(std::string("ttor::gpu: cannot create device context: ") + ttg_strerror(s));
        }
    }
    return c;
}

}  // namespace gpu

class Threadpool_shared {
   public:
    Threadpool_shared(int n_threads, int verb = 0, std::string basename = "Wk_", bool start_immediately = true)
        : n_threads_(n_threads), verb_(verb), basename_(std::move(basename)) {
        if (n_threads <= 0) throw std::invalid_argument("Threadpool_shared: n_threads must be positive");
        if (start_immediately) start();
    }
    virtual ~Threadpool_shared() {
        if (own_ctx_ && ctx_) ttg_destroy(ctx_);
    }
    Threadpool_shared(const Threadpool_shared&) = delete;
    Threadpool_shared& operator=(const Threadpool_shared&) = delete;

    void start() { started_ = true; }

    // Raw insertion of a task (ownership is taken).  From the main thread the
    // task is ready at once; from inside a running task it becomes a
    // successor of that task.
    void insert(Task* t, int where, bool binding = false) {
        check_where(where, t ? t->c_name() : "?");
        std::lock_guard<std::mutex> g(mtx_);
        const int id = new_node_locked();
        detail::Node& n = cap_.nodes[id];
        n.task.reset(t);
        std::string nm = t->name;
        n.name = [nm]() { return nm; };
        n.priority = t->priority;
        n.bind = binding ? where : -1;
        n.indegree = 1;
        promise_locked(id);
        make_ready_locked(id);
    }

    // Capture every ready task, then run the recorded graph on the GPU.
    void join() {
        if (!started_) throw std::logic_error("Threadpool_shared::join() before start()");
        capture();
        build_and_upload();
        run_device();
        done_ = true;
    }

    // Capture and upload without running (extension: plans that run the
    // graph later with replay()).
    void capture_only() {
        if (!started_) throw std::logic_error("Threadpool_shared::capture_only() before start()");
        capture();
        build_and_upload();
    }

    // Capture only, no device (extension): the graph can be inspected with
    // dump_dag(); runs are the capture's.
    void capture_dry() {
        if (!started_) throw std::logic_error("Threadpool_shared::capture_dry() before start()");
        capture();
    }

    // Run the last uploaded graph again (same tiles, same DAG) — the replay of
    // a captured plan.  Extension: not in the reference.
    ttg_status replay(void* stream = nullptr) {
        if (!uploaded_) return TTG_ESTATE;
        return run_device(stream);
    }

    bool is_done() { return done_; }
    void set_logger(Logger* logger) { logger_ = logger; }
    int size() { return n_threads_; }

    // Extensions (not in the reference): device context, worker count, trace.
    void set_context(ttg_ctx* c) { ctx_ = c; own_ctx_ = false; }
    void set_workers(int w) { workers_ = w; }
    ttg_ctx* context() {
        if (!ctx_) {
            if (workers_ > 0 || logger_ || trace_) {
                ttg_opts o{};
                const char* dev = getenv("TTG_DEVICE");
                o.device = dev ? atoi(dev) : 0;
                o.workers = workers_;
                o.timeout_s = 30.0;
                o.trace = logger_ ? 1 : trace_;
                if (ttg_create(&ctx_, &o) != TTG_OK) throw std::runtime_error("Threadpool_shared: cannot create device context");
                own_ctx_ = true;
            } else {
                ctx_ = gpu::default_context();
            }
        }
        return ctx_;
    }
    void set_trace(bool on) { trace_ = on ? 1 : 0; }
    // Extension: replace the captured priorities by the longest remaining
    // path of each device task (ttg_critical_path_priority).
    void set_critical_path_priority(bool on) { cp_prio_ = on; }
    const ttg_report& report() const { return report_; }
    ttg_status status() const { return report_.status; }
    double capture_seconds() const { return capture_s_; }
    int n_device_tasks() const { return (int)dev_node_.size(); }
    // Node (captured task) of each device task, and the task names.
    const std::vector<int>& device_task_nodes() const { return dev_node_; }
    // Extension: device-only tasks appended to the uploaded graph (tasks the
    // captured program does not have, e.g. the input conversion of a
    // mixed-precision plan).  ops[e] runs with priority prio[e] and promises
    // the device tasks succ[e] (whose counters each grow by one); the graph is
    // uploaded again.  Call after capture_only().
    void add_device_tasks(const std::vector<ttg_op>& ops, const std::vector<double>& prio, const std::vector<std::vector<int>>& succ) {
        if (!uploaded_) throw std::logic_error("Threadpool_shared::add_device_tasks() before the graph was captured");
        const int nd = (int)g_ops_.size();
        std::vector<int64_t> ptr(g_ptr_);
        std::vector<int32_t> idx(g_idx_);
        for (size_t e = 0; e < ops.size(); ++e) {
            g_ops_.push_back(ops[e]);
            g_init_.push_back(0);
            g_prio_.push_back(prio[e]);
            g_bind_.push_back(-1);
            for (int d : succ[e]) {
                if (d < 0 || d >= nd) throw std::out_of_range("Threadpool_shared::add_device_tasks(): successor");
                idx.push_back(d);
                ++g_init_[d];
            }
            ptr.push_back((int64_t)idx.size());
        }
        g_ptr_ = std::move(ptr);
        g_idx_ = std::move(idx);
        extra_tasks_ += (int)ops.size();
        upload();
    }
    // Priority of uploaded device task d.
    double device_priority(int d) const { return g_prio_.at(d); }
    // Device tasks appended by add_device_tasks (they follow the captured ones).
    int n_extra_device_tasks() const { return extra_tasks_; }
    // All tasks of the uploaded graph (the size of the context's per-task
    // records: ttg_task_record, ttg_trace).
    int n_uploaded_tasks() const { return (int)dev_node_.size() + extra_tasks_; }
    std::string node_name(int node) const { return cap_.nodes[node].name ? cap_.nodes[node].name() : "_"; }
    int n_nodes() const { return (int)cap_.nodes.size(); }

    // DAG record in the oracle's format: <prefix>.tasks.csv lists
    // name,indegree,promises,runs for every task that received a promise;
    // <prefix>.edges.csv lists "src,dst" per promise ("ROOT" = main thread).
    void dump_dag(const std::string& prefix) const {
        std::vector<std::vector<std::string>> rows;
        std::vector<int32_t> runs(n_uploaded_tasks(), 0);
        std::vector<int> node_runs(cap_.nodes.size(), 0);
        if (uploaded_) {
            ttg_task_record(ctx_, runs.data(), nullptr);
            // A node ran on the device when its last device task ran.
            for (size_t d = 0; d < dev_node_.size(); ++d)
                if (dev_last_[d]) node_runs[dev_node_[d]] += runs[d];
        }
        std::vector<std::pair<std::string, std::array<long, 3>>> tasks;
        for (size_t i = 0; i < cap_.nodes.size(); ++i) {
            const detail::Node& n = cap_.nodes[i];
            const long r = uploaded_ ? node_runs[i] : (n.ran ? 1 : 0);
            tasks.push_back({n.name ? n.name() : "_", {n.indegree, n.promises, r}});
        }
        std::sort(tasks.begin(), tasks.end());
        // Merge duplicate names (a key fulfilled past its indegree opens a new node).
        std::ofstream tf(prefix + ".tasks.csv");
        tf << "name,indegree,promises,runs\n";
        for (size_t i = 0; i < tasks.size();) {
            size_t j = i;
            std::array<long, 3> acc = tasks[i].second;
            while (++j < tasks.size() && tasks[j].first == tasks[i].first) {
                acc[1] += tasks[j].second[1];
                acc[2] += tasks[j].second[2];
            }
            tf << tasks[i].first << "," << acc[0] << "," << acc[1] << "," << acc[2] << "\n";
            i = j;
        }
        std::vector<std::pair<std::string, std::string>> edges;
        for (size_t i = 0; i < cap_.nodes.size(); ++i) {
            const detail::Node& n = cap_.nodes[i];
            for (int r = 0; r < n.promises - n.in_edges; ++r) edges.push_back({"ROOT", node_name((int)i)});
            for (int s : n.succ) edges.push_back({node_name((int)i), node_name(s)});
        }
        std::sort(edges.begin(), edges.end());
        std::ofstream ef(prefix + ".edges.csv");
        for (auto& e : edges) ef << e.first << "," << e.second << "\n";
        // <prefix>.prio.csv: name,priority of every task as captured (the
        // value its Taskflow's priority function gave).
        std::vector<std::pair<std::string, double>> prio;
        for (size_t i = 0; i < cap_.nodes.size(); ++i) prio.push_back({node_name((int)i), cap_.nodes[i].priority});
        std::sort(prio.begin(), prio.end());
        prio.erase(std::unique(prio.begin(), prio.end(), [](const auto& a, const auto& b) { return a.first == b.first; }), prio.end());
        std::ofstream pf(prefix + ".prio.csv");
        pf << "name,priority\n";
        for (auto& e : prio) pf << e.first << "," << e.second << "\n";
    }

    // ---- used by Taskflow<K> (not part of the reference interface) ----
    int capture_new_node(Task* t, std::function<std::string()> name, int where, bool binding, int indegree) {
        check_where(where, "task");
        std::lock_guard<std::mutex> g(mtx_);
        const int id = new_node_locked();
        detail::Node& n = cap_.nodes[id];
        n.task.reset(t);
        n.name = std::move(name);
        n.priority = t->priority;
        n.bind = binding ? where : -1;
        n.indegree = indegree;
        return id;
    }
    void capture_promise(int node) {
        std::lock_guard<std::mutex> g(mtx_);
        promise_locked(node);
    }
    void capture_ready(int node) {
        std::lock_guard<std::mutex> g(mtx_);
        make_ready_locked(node);
    }
    int verb() const { return verb_; }

   protected:
    void check_where(int where, const char* name) {
        if (where < 0 || where >= n_threads_) {
            printf("Error: where = %d (num threads = %d) for %s\n", where, n_threads_, name);
            throw std::out_of_range("Threadpool_shared: mapping out of range");
        }
    }

   private:
    int new_node_locked() {
        cap_.nodes.emplace_back();
        return (int)cap_.nodes.size() - 1;
    }
    void promise_locked(int node) {
        detail::Node& n = cap_.nodes[node];
        n.promises++;
        if (cap_.current >= 0) {
            n.in_edges++;
            cap_.nodes[cap_.current].succ.push_back(node);
        }
    }
    void make_ready_locked(int node) {
        detail::Node& n = cap_.nodes[node];
        n.ready = true;
        ready_.push({n.priority, -(long)node});
    }

    // Run the ready closures on the host in priority order (FIFO among equal
    // priorities), recording tile operations and promises.
    void capture() {
        timer t0 = wctime();
        detail::Capture*& slot = detail::current_capture();
        detail::Capture* saved = slot;
        slot = &cap_;
        while (true) {
            int id;
            {
                std::lock_guard<std::mutex> g(mtx_);
                if (ready_.empty()) break;
                id = (int)(-ready_.top().second);
                ready_.pop();
                cap_.current = id;
            }
            // The task body may create nodes (the vector can grow): hold the
            // closure, not a reference into the vector.
            std::unique_ptr<Task> t;
            {
                std::lock_guard<std::mutex> g(mtx_);
                t = std::move(cap_.nodes[id].task);
            }
            if (verb_ > 1) printf("[%s] capturing %s\n", basename_.c_str(), node_name(id).c_str());
            if (t) {
                t->run();
                t->fulfill();
            }
            t.reset();  // ownership: deleted after it ran
            std::lock_guard<std::mutex> g(mtx_);
            cap_.nodes[id].ran = true;
            cap_.current = -1;
        }
        slot = saved;
        capture_s_ += elapsed(t0, wctime());
    }

    // Device graph: one device task per recorded operation, chained inside a
    // node; a node without operations is one no-op task.  Nodes that never
    // became ready are left out (the reference never runs them either).
    void build_and_upload() {
        const int nn = (int)cap_.nodes.size();
        std::vector<int> first(nn, -1), last(nn, -1);
        dev_node_.clear();
        dev_last_.clear();
        std::vector<ttg_op> ops;
        for (int i = 0; i < nn; ++i) {
            const detail::Node& n = cap_.nodes[i];
            if (!n.ran) continue;
            first[i] = (int)ops.size();
            if (n.ops.empty()) {
                ttg_op nop{};
                nop.kind = TTG_OP_NOP;
                ops.push_back(nop);
                dev_node_.push_back(i);
            } else {
                for (const ttg_op& o : n.ops) {
                    ops.push_back(o);
                    dev_node_.push_back(i);
                }
            }
            last[i] = (int)ops.size() - 1;
        }
        dev_last_.assign(ops.size(), 0);
        for (int i = 0; i < nn; ++i)
            if (last[i] >= 0) dev_last_[last[i]] = 1;
        const int nd = (int)ops.size();
        std::vector<int32_t> init(nd, 0), bind(nd, -1);
        std::vector<double> prio(nd, 0.0);
        std::vector<int64_t> ptr(nd + 1, 0);
        std::vector<int32_t> idx;
        for (int d = 0; d < nd; ++d) {
            const int i = dev_node_[d];
            const detail::Node& n = cap_.nodes[i];
            prio[d] = n.priority;
            bind[d] = n.bind;
            if (d == first[i]) {
                init[d] = n.in_edges;
            } else {
                init[d] = 1;  // chained after the previous operation of the node
            }
            if (d != last[i]) {
                idx.push_back(d + 1);
            } else {
                for (int s : n.succ)
                    if (first[s] >= 0) idx.push_back(first[s]);
            }
            ptr[d + 1] = (int64_t)idx.size();
        }
        // Device counters only count promises from tasks that ran; a node
        // that ran has all its promises (it became ready), so in_edges is
        // exact for it.
        g_ops_ = std::move(ops);
        g_init_ = std::move(init);
        g_prio_ = std::move(prio);
        g_bind_ = std::move(bind);
        g_ptr_ = std::move(ptr);
        g_idx_ = std::move(idx);
        if (cp_prio_) {
            ttg_graph_desc g{};
            g.n_tasks = (int32_t)g_ops_.size();
            g.ops = g_ops_.data();
            g.succ_ptr = g_ptr_.data();
            g.succ_idx = g_idx_.data();
            if (ttg_critical_path_priority(&g, g_prio_.data()) != TTG_OK)
                throw std::runtime_error("Threadpool_shared: critical-path priorities failed");
        }
        upload();
        uploaded_ = true;
    }

    // Upload the recorded graph (again, if another graph replaced it in the
    // context since).
    void upload() {
        ttg_graph_desc g{};
        g.n_tasks = (int32_t)g_ops_.size();
        g.ops = g_ops_.data();
        g.init_count = g_init_.data();
        g.priority = g_prio_.data();
        g.bind = g_bind_.data();
        g.succ_ptr = g_ptr_.data();
        g.succ_idx = g_idx_.data();
        ttg_status s = ttg_graph_upload(context(), &g);
        if (s != TTG_OK) throw std::runtime_error(std::string("Threadpool_shared: graph upload failed: ") + ttg_strerror(s));
        graph_gen_ = ttg_graph_generation(context());
    }

    ttg_status run_device(void* stream = nullptr) {
        if (ttg_graph_generation(context()) != graph_gen_) {
            try {
                upload();
            } catch (const std::exception&) {
                return TTG_ECUDA;
            }
        }
        timer t0 = wctime();
        ttg_status s = ttg_run(context(), stream, &report_);
        timer t1 = wctime();
        last_run_t0_ = t0;
        if (verb_ > 0)
            printf("[%s] device run: %lld tasks, %.3f ms, status %s\n", basename_.c_str(), (long long)report_.tasks_run,
                   report_.elapsed_ms, ttg_strerror(s));
        // On stderr (stdout carries the application's own output).  A tile that
        // is not positive definite is reported by the status; callers that
        // retry with a remedy (the mixed Cholesky plan) see it only at verb > 0.
        if (s != TTG_OK && s != TTG_EUNDERRUN && (s != TTG_ENOTPD || verb_ > 0))
            fprintf(stderr, "Error: device executor: %s\n", ttg_strerror(s));
        if (logger_) fill_logger(t0, t1);
        return s;
    }

public:
    // Extension: the last device run's timeline in the Logger's CSV format
    // ("<basename><worker>>run><task>,<start>,<end>", times in seconds), as
    // 2d_cholesky writes with --log (needs a context created with trace).
    bool write_log(std::ostream& os) {
        Logger lg(std::max(1, (int)dev_node_.size()));
        Logger* keep = logger_;
        logger_ = &lg;
        fill_logger(last_run_t0_, last_run_t0_);
        logger_ = keep;
        if (lg.n_events() == 0) return false;
        os << lg;
        return true;
    }
    // Extension: the captured dependencies in the DepsLogger's CSV format
    // ("<task>,<successor>" per promise made by a task), as 2d_cholesky writes
    // with --depslog.
    void write_deps(std::ostream& os) const {
        for (size_t i = 0; i < cap_.nodes.size(); ++i)
            for (int s : cap_.nodes[i].succ) os << node_name((int)i) << "," << node_name(s) << "\n";
    }

private:
    // Device trace -> Logger events named "<basename><worker>>run><task>".
    void fill_logger(timer t0, timer t1) {
        const int nd = (int)dev_node_.size();
        std::vector<int64_t> s(n_uploaded_tasks()), e(n_uploaded_tasks());
        std::vector<int32_t> w(n_uploaded_tasks());
        if (ttg_trace(ctx_, s.data(), e.data(), w.data()) != TTG_OK) return;
        (void)t1;
        for (int d = 0; d < nd; ++d) {
            if (s[d] < 0) continue;
            auto ev = std::make_unique<Event>(basename_ + std::to_string(w[d]) + ">run>" + node_name(dev_node_[d]));
            ev->start = t0 + std::chrono::nanoseconds(s[d]);
            ev->end = t0 + std::chrono::nanoseconds(e[d]);
            logger_->add_event(std::move(ev));
        }
    }

    int n_threads_;
    int verb_;
    std::string basename_;
    bool started_ = false;
    bool done_ = false;
    bool uploaded_ = false;
    int workers_ = 0;
    int trace_ = 0;
    Logger* logger_ = nullptr;
    ttg_ctx* ctx_ = nullptr;
    bool own_ctx_ = false;
    ttg_report report_{};
    timer last_run_t0_ = wctime();
    double capture_s_ = 0.0;
    std::mutex mtx_;
    detail::Capture cap_;
    std::priority_queue<std::pair<double, long>> ready_;
    std::vector<int> dev_node_;
    std::vector<char> dev_last_;
    // The recorded graph, kept for re-uploads.
    std::vector<ttg_op> g_ops_;
    std::vector<int32_t> g_init_, g_bind_, g_idx_;
    std::vector<double> g_prio_;
    bool cp_prio_ = false;
    int extra_tasks_ = 0;
    std::vector<int64_t> g_ptr_;
    uint64_t graph_gen_ = 0;
};

#ifdef TTOR_SHARED
typedef Threadpool_shared Threadpool;
#endif

}  // namespace ttor

#endif
