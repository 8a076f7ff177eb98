// Boost-subset shim (self-written, test infrastructure): the two assertion
// macros the reference uses.  BOOST_VERIFY always evaluates its argument.
#ifndef KCNA_SHIM_BOOST_ASSERT_HPP
#define KCNA_SHIM_BOOST_ASSERT_HPP
#include <cassert>
#include <cstdio>
#include <cstdlib>
#define BOOST_ASSERT(expr) assert(expr)
#define BOOST_VERIFY(expr)                                                          \
    do {                                                                            \
        if (!(expr)) {                                                              \
            std::fprintf(stderr, "BOOST_VERIFY failed: %s (%s:%d)\n", #expr, __FILE__, __LINE__); \
            std::abort();                                                           \
        }                                                                           \
    } while (0)
#endif
