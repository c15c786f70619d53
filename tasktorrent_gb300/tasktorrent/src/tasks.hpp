// Task record: the same fields as the reference's tasktorrent/src/tasks.hpp
// (:13-29) — run and fulfill closures (always called one after the other), a
// priority (higher first) and a name.
#ifndef TTOR_GB300_TASKS_HPP
#define TTOR_GB300_TASKS_HPP

#include <functional>
#include <string>

struct Task {
    std::function<void()> run;
    std::function<void()> fulfill;
    double priority;
    std::string name;
    Task() : run([]() {}), fulfill([]() {}), priority(0), name("_") {}
    const char* c_name() { return name.c_str(); }
};

struct less_pTask {
    bool operator()(const Task* lhs, const Task* rhs) const { return lhs->priority < rhs->priority; }
};

#endif
