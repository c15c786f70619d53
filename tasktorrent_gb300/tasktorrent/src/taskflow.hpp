// ttor::Taskflow<K> for GB300 — the parametrized task graph front end with the
// reference's interface (tasktorrent/src/taskflow.hpp:41-297): set_task,
// set_fulfill, set_mapping, set_binding, set_indegree, set_name,
// set_priority, name(k), fulfill_promise(k).
//
// fulfill_promise keeps the reference's counting rule (:241-296): a task with
// indegree 1 is inserted at once; otherwise a counter is created at the
// indegree on the first promise, decremented on each promise, and the task is
// inserted (and the entry erased) when it reaches zero — so a key promised
// past its indegree opens a new instance, exactly as in the reference.  The
// difference is where it happens: promises are recorded by the thread pool's
// capture (each promise made inside a task body becomes a graph edge) and the
// recorded graph runs on the GPU at join().
#ifndef TTOR_GB300_TASKFLOW_HPP
#define TTOR_GB300_TASKFLOW_HPP

#include <cassert>
#include <cstdio>
#include <functional>
#include <string>
#include <unordered_map>
#include <utility>

#include "hashes.hpp"
#include "threadpool_shared.hpp"
#include "util.hpp"

namespace ttor {

template <class K>
class Taskflow {
   private:
    Threadpool_shared* tp;
    int verb;

    // key -> (open node, remaining promises)
    typedef std::unordered_map<K, std::pair<int, int>, hash_int_N<K>> map_t;
    map_t dep_map;

    std::function<void(K)> f_run;
    std::function<void(K)> f_fulfill;
    std::function<int(K)> f_mapping;
    std::function<bool(K)> f_binding;
    std::function<int(K)> f_indegree;
    std::function<std::string(K)> f_name;
    std::function<double(K)> f_prio;

    int new_node(K k, int indegree) {
        Task* t = new Task();
        t->run = [this, k]() { f_run(k); };
        t->fulfill = [this, k]() { f_fulfill(k); };
        t->priority = f_prio(k);
        const int where = f_mapping(k);
        const bool binding = f_binding(k);
        // The name is evaluated lazily (dumps, logs) from a copy of the name
        // function, so it stays valid after this Taskflow is gone.
        std::function<std::string(K)> fn = f_name;
        return tp->capture_new_node(t, [fn, k]() { return fn(k); }, where, binding, indegree);
    }

   public:
    Taskflow(Threadpool_shared* tp_, int verb_ = 0) : tp(tp_), verb(verb_) {
        f_name = [](K k) { (void)k; return std::string("_"); };
        f_run = [](K k) { (void)k; printf("Taskflow: undefined task function\n"); };
        f_fulfill = [](K k) { (void)k; };
        f_mapping = [](K k) { (void)k; printf("Taskflow: undefined mapping function\n"); return 0; };
        f_binding = [](K k) { (void)k; return false; };
        f_indegree = [](K k) { (void)k; printf("Taskflow: undefined indegree function\n"); return 0; };
        f_prio = [](K k) { (void)k; return 0.0; };
    }

    Taskflow& set_task(std::function<void(K)> f) { f_run = f; return *this; }
    Taskflow& set_fulfill(std::function<void(K)> f) { f_fulfill = f; return *this; }
    Taskflow& set_mapping(std::function<int(K)> f) { f_mapping = f; return *this; }
    // Takes int(K) like the reference (taskflow.hpp:169).
    Taskflow& set_binding(std::function<int(K)> f) {
        f_binding = [f](K k) { return f(k) != 0; };
        return *this;
    }
    Taskflow& set_indegree(std::function<int(K)> f) { f_indegree = f; return *this; }
    Taskflow& set_name(std::function<std::string(K)> f) { f_name = f; return *this; }
    Taskflow& set_priority(std::function<double(K)> f) { f_prio = f; return *this; }

    std::string name(K k) { return f_name(k); }

    void fulfill_promise(K k) {
        const int indeg = f_indegree(k);
        if (indeg == 1) {
            const int node = new_node(k, 1);
            tp->capture_promise(node);
            tp->capture_ready(node);
            return;
        }
        auto it = dep_map.find(k);
        if (it == dep_map.end()) {
            if (indeg < 1) {
                printf("Error: indegree %d < 1 for %s\n", indeg, name(k).c_str());
                assert(false);
                return;
            }
            it = dep_map.emplace(k, std::make_pair(new_node(k, indeg), indeg)).first;
        }
        const int node = it->second.first;
        tp->capture_promise(node);
        const int count = --it->second.second;
        if (verb > 1) printf("%s count: %d\n", name(k).c_str(), count);
        if (count == 0) {
            dep_map.erase(it);
            tp->capture_ready(node);
        }
    }
};

}  // namespace ttor

#endif
