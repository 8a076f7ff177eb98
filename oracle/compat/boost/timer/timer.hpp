// Boost-subset shim (self-written, test infrastructure): cpu_timer with
// elapsed().wall in nanoseconds, the only part the reference reads.
#ifndef KCNA_SHIM_BOOST_TIMER_HPP
#define KCNA_SHIM_BOOST_TIMER_HPP
#include <chrono>
#include <cstdint>
namespace boost {
namespace timer {
typedef int64_t nanosecond_type;
struct cpu_times {
    nanosecond_type wall, user, system;
};
struct cpu_timer {
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    cpu_times elapsed() const {
        nanosecond_type ns = std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count();
        cpu_times t;
        t.wall = ns;
        t.user = ns;
        t.system = 0;
        return t;
    }
    void start() { t0 = std::chrono::steady_clock::now(); }
};
} // namespace timer
} // namespace boost
#endif
