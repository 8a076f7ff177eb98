// Boost-subset shim (self-written, test infrastructure): a counter with the
// progress_display interface (no drawing).
#ifndef KCNA_SHIM_BOOST_PROGRESS_HPP
#define KCNA_SHIM_BOOST_PROGRESS_HPP
#include <ostream>
namespace boost {
struct progress_display {
    unsigned long n_, c_;
    progress_display(unsigned long n, std::ostream &) : n_(n), c_(0) {}
    unsigned long operator++() { return ++c_; }
    unsigned long operator+=(unsigned long k) { return c_ += k; }
    unsigned long count() const { return c_; }
    unsigned long expected_count() const { return n_; }
};
} // namespace boost
#endif
