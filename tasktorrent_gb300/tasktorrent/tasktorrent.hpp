// Public interface of the GB300 build of TaskTorrent's shared-memory core:
// the same umbrella header name as the reference (tasktorrent/tasktorrent.hpp)
// so a miniapp switches by changing its include path and linking libttg.so.
// The MPI half (Communicator, active messages, Threadpool_dist) is not part
// of this build; Threadpool is Threadpool_shared.
#ifndef TTOR_GB300_TASKTORRENT_HPP
#define TTOR_GB300_TASKTORRENT_HPP

#ifndef TTOR_SHARED
#define TTOR_SHARED
#endif

#include "src/util.hpp"
#include "src/tasks.hpp"
#include "src/threadpool_shared.hpp"
#include "src/taskflow.hpp"
#include "src/gpu_blas.hpp"

#endif
