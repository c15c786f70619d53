/*
 * runtime.hpp — TEST INFRASTRUCTURE ONLY.  A CPU restatement of the
 * reference's shared-memory runtime, with the same interface as
 * ttor::Taskflow<K> / ttor::Threadpool_shared so that the oracle's task
 * graphs (dag.hpp) run unchanged on it or on the reference's own runtime.
 *
 * Restated behaviour (paths inside the reference project):
 *  - tasktorrent/src/taskflow.hpp: fulfill_promise inserts at once when the
 *    indegree is 1 (:245-249); otherwise the counter of key k is created at
 *    the indegree on the first promise, decremented on each promise, and at
 *    zero the entry is erased and the task inserted (:256-295); a negative
 *    count is reported (:278-282).  The reference serialises counter updates
 *    by running them as bound max-priority tasks on the mapped thread; here a
 *    per-thread mutex guards the same map.
 *  - tasktorrent/src/threadpool_shared.cpp: a ready (stealable) and a bound
 *    priority queue per thread, the higher-priority top wins and bound wins
 *    ties (:104-142); stealing from the other threads' ready queues in
 *    round-robin order (:143-169); run() then fulfill() (:36-70); a +1
 *    sentinel released by join() (:81-85, :234-241); thread 0 declares
 *    completion when nothing is in flight (:73-79, :180-191).
 */
#ifndef TTG_ORACLE_RUNTIME_HPP
#define TTG_ORACLE_RUNTIME_HPP

#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <memory>
#include <mutex>
#include <queue>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace orc {

struct Task {
    std::function<void()> run, fulfill;
    double priority = 0.0;
    std::string name = "_";
};

struct ByPrio {
    bool operator()(const Task* a, const Task* b) const { return a->priority < b->priority; }
};
typedef std::priority_queue<Task*, std::vector<Task*>, ByPrio> PQ;

class Threadpool {
   public:
    Threadpool(int n, int verb = 0, std::string basename = "Wk_", bool start_immediately = true)
        : ready_(n), bound_(n), rmtx_(n), bmtx_(n), n_(n) {
        (void)verb;
        (void)basename;
        if (start_immediately) start();
    }
    ~Threadpool() {
        if (started_ && !joined_) join();
    }
    int size() const { return n_; }

    void start() {
        started_ = true;
        ++in_flight_; /* sentinel */
        for (int self = 0; self < n_; ++self) threads_.emplace_back([this, self] { loop(self); });
    }

    void insert(Task* t, int where, bool binding) {
        if (where < 0 || where >= n_) {
            fprintf(stderr, "oracle: bad mapping %d for %s\n", where, t->name.c_str());
            abort();
        }
        ++in_flight_;
        if (binding) {
            std::lock_guard<std::mutex> g(bmtx_[where]);
            bound_[where].push(t);
        } else {
            std::lock_guard<std::mutex> g(rmtx_[where]);
            ready_[where].push(t);
        }
    }

    void join() {
        --in_flight_; /* release the sentinel */
        for (auto& t : threads_) t.join();
        joined_ = true;
    }

   private:
    void loop(int self) {
        while (true) {
            Task* t = nullptr;
            {
                std::lock_guard<std::mutex> g1(rmtx_[self]);
                std::lock_guard<std::mutex> g2(bmtx_[self]);
                PQ& r = ready_[self];
                PQ& b = bound_[self];
                if (!r.empty() && !b.empty()) {
                    if (b.top()->priority >= r.top()->priority) { t = b.top(); b.pop(); }
                    else { t = r.top(); r.pop(); }
                } else if (!r.empty()) { t = r.top(); r.pop(); }
                else if (!b.empty()) { t = b.top(); b.pop(); }
            }
            for (int j = 1; !t && j < n_; ++j) {
                const int other = (self + j) % n_;
                std::lock_guard<std::mutex> g(rmtx_[other]);
                if (!ready_[other].empty()) { t = ready_[other].top(); ready_[other].pop(); }
            }
            if (t) {
                t->run();
                t->fulfill();
                delete t;
                --in_flight_;
            } else {
                if (self == 0 && in_flight_.load() == 0) done_.store(true);
                if (done_.load()) return;
                std::this_thread::sleep_for(std::chrono::microseconds(10));
            }
        }
    }

    std::vector<PQ> ready_, bound_;
    std::vector<std::mutex> rmtx_, bmtx_;
    std::vector<std::thread> threads_;
    std::atomic<int> in_flight_{0};
    std::atomic<bool> done_{false};
    int n_;
    bool started_ = false;
    bool joined_ = false;
};

template <class K>
struct KeyHash {
    size_t operator()(const K& k) const {
        uint64_t h = 1469598103934665603ULL;
        for (size_t i = 0; i < k.size(); ++i) h = (h ^ (uint32_t)k[i]) * 1099511628211ULL;
        return (size_t)h;
    }
};
template <>
struct KeyHash<int> {
    size_t operator()(int k) const { return std::hash<int>()(k); }
};

template <class K>
class Taskflow {
   public:
    Taskflow(Threadpool* p, int verb = 0) : tp_(p), maps_(p->size()), mtx_(p->size()) { (void)verb; }

    Taskflow& set_task(std::function<void(K)> f) { run_ = f; return *this; }
    Taskflow& set_fulfill(std::function<void(K)> f) { fulfill_ = f; return *this; }
    Taskflow& set_mapping(std::function<int(K)> f) { mapping_ = f; return *this; }
    Taskflow& set_binding(std::function<int(K)> f) { binding_ = f; return *this; }
    Taskflow& set_indegree(std::function<int(K)> f) { indegree_ = f; return *this; }
    Taskflow& set_name(std::function<std::string(K)> f) { name_ = f; return *this; }
    Taskflow& set_priority(std::function<double(K)> f) { prio_ = f; return *this; }
    std::string name(K k) { return name_(k); }

    void fulfill_promise(K k) {
        const int indeg = indegree_(k);
        if (indeg == 1) { insert(k); return; }
        const int where = mapping_(k);
        bool ready = false;
        {
            std::lock_guard<std::mutex> g(mtx_[where]);
            auto& m = maps_[where];
            auto it = m.find(k);
            if (it == m.end()) it = m.emplace(k, indeg).first;
            const int c = --it->second;
            if (c < 0) fprintf(stderr, "Error: count < 0 for %s\n", name_(k).c_str());
            if (c == 0) { m.erase(it); ready = true; }
        }
        if (ready) insert(k);
    }

   private:
    void insert(K k) {
        Task* t = new Task();
        t->run = [this, k]() { run_(k); };
        t->fulfill = [this, k]() { fulfill_(k); };
        t->priority = prio_(k);
        tp_->insert(t, mapping_(k), binding_(k) != 0);
    }

    Threadpool* tp_;
    std::vector<std::unordered_map<K, int, KeyHash<K>>> maps_;
    std::vector<std::mutex> mtx_;
    std::function<void(K)> run_ = [](K) {};
    std::function<void(K)> fulfill_ = [](K) {};
    std::function<int(K)> mapping_ = [](K) { return 0; };
    std::function<int(K)> binding_ = [](K) { return 0; };
    std::function<int(K)> indegree_ = [](K) { return 1; };
    std::function<std::string(K)> name_ = [](K) { return std::string("_"); };
    std::function<double(K)> prio_ = [](K) { return 0.0; };
};

}  // namespace orc

#endif
