// ttor utilities: timers, event Logger and DepsLogger.
//
// Same interface and CSV formats as the reference's tasktorrent/src/util.hpp
// (:14-80) and util.cpp (:13-129): wctime/elapsed, a Logger of named
// start/end events with a fixed capacity and an overflow flag, and a
// DepsLogger of "src,dst" edges.  On this build the executor fills the Logger
// after join() from the device trace (one "<basename><worker>>run><task>"
// event per task).
#ifndef TTOR_GB300_UTIL_HPP
#define TTOR_GB300_UTIL_HPP

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <iomanip>
#include <iostream>
#include <memory>
#include <string>
#include <unistd.h>
#include <vector>

namespace ttor {

typedef std::chrono::time_point<std::chrono::high_resolution_clock> timer;

inline double elapsed(timer start, timer end) { return std::chrono::duration<double>(end - start).count(); }
inline double time(timer t) { return std::chrono::duration<double>(t.time_since_epoch()).count(); }
inline timer wctime() { return std::chrono::high_resolution_clock::now(); }
inline std::string get_name_me() {
    char name[64];
    return gethostname(name, sizeof(name)) == 0 ? std::string(name) : std::string("ErrorNoName");
}

struct Event {
    std::string name;
    timer start;
    timer end;
    explicit Event(std::string name_) : name(std::move(name_)), start(wctime()) {}
    Event() : name("_"), start(wctime()) {}
    void record() { end = wctime(); }
};

struct Logger {
   private:
    timer origin;
    std::atomic<bool> printed_warning;
    std::atomic<int> i;
    std::vector<std::unique_ptr<Event>> events;

   public:
    explicit Logger(int N) : origin(wctime()), printed_warning(false), i(0), events(N) {}
    Logger() : Logger(0) {}
    void add_event(std::unique_ptr<Event> e) {
        const int id = i++;
        if (id < (int)events.size()) {
            events[id] = std::move(e);
        } else if (!printed_warning.exchange(true)) {
            printf("Logger::add_event buffer full\n");
        }
    }
    void record(std::unique_ptr<Event> e) {
        e->record();
        add_event(std::move(e));
    }
    int n_events() const { return std::min((int)events.size(), i.load()); }
    bool was_full() const { return printed_warning.load(); }
    const std::vector<std::unique_ptr<Event>>& get_events() const { return events; }
    timer get_origin() const { return origin; }
};

struct DepsEvent {
    std::string self_name;
    std::string out_deps_name;
    DepsEvent(std::string s, std::string o) : self_name(std::move(s)), out_deps_name(std::move(o)) {}
    DepsEvent() {}
};

struct DepsLogger {
    std::atomic<int> i;
    std::atomic<bool> printed_warning;
    std::vector<std::unique_ptr<DepsEvent>> events;
    explicit DepsLogger(int N) : i(0), printed_warning(false), events(N) {}
    DepsLogger() : DepsLogger(0) {}
    void add_event(std::unique_ptr<DepsEvent> e) {
        const int id = i++;
        if (id < (int)events.size()) {
            events[id] = std::move(e);
        } else {
            printed_warning.store(true);
            printf("DepsLogger::add_event buffer full\n");
        }
    }
    bool was_full() const { return printed_warning.load(); }
};

inline std::ostream& operator<<(std::ostream& os, DepsLogger& t) {
    if (t.was_full()) printf("Warning: buffer was full at some point during the profiling\n");
    const int n = std::min((int)t.events.size(), t.i.load());
    for (int k = 0; k < n; ++k) os << t.events[k]->self_name << "," << t.events[k]->out_deps_name << "\n";
    return os;
}

inline std::ostream& operator<<(std::ostream& os, Logger& t) {
    if (t.was_full()) printf("Warning: buffer was full at some point during the profiling\n");
    os << std::setprecision(64);
    for (int k = 0; k < t.n_events(); ++k) {
        const auto& e = t.get_events()[k];
        os << e->name << "," << ttor::time(e->start) << "," << ttor::time(e->end) << "\n";
    }
    return os;
}

}  // namespace ttor

#endif
