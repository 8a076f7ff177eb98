// Boost-subset shim (self-written, test infrastructure): accumulator_set with
// the mean statistic only.  The sum is kept in the sample type and divided by
// the count converted to it, as the reference's float accumulators do.
#ifndef KCNA_SHIM_BOOST_ACCUMULATORS_HPP
#define KCNA_SHIM_BOOST_ACCUMULATORS_HPP
#include <cstddef>
namespace boost {
namespace accumulators {
namespace tag {
struct mean {};
struct moment_base {};
} // namespace tag
template <typename... Ts>
struct stats {};
template <typename T, typename Features>
struct accumulator_set {
    T sum_ = T();
    std::size_t n_ = 0;
    void operator()(T x) { sum_ += x; ++n_; }
};
template <typename T, typename F>
T mean(const accumulator_set<T, F> &a) { return a.sum_ / static_cast<T>(a.n_); }
} // namespace accumulators
} // namespace boost
#endif
