// Boost-subset shim (self-written, test infrastructure): a copyable spin lock
// with lock / try_lock / unlock, zero-initialised = unlocked.
#ifndef KCNA_SHIM_BOOST_SPINLOCK_HPP
#define KCNA_SHIM_BOOST_SPINLOCK_HPP
namespace boost {
namespace detail {
struct spinlock {
    int v_ = 0;
    bool try_lock() { return __atomic_exchange_n(&v_, 1, __ATOMIC_ACQUIRE) == 0; }
    void lock() { while (!try_lock()) {} }
    void unlock() { __atomic_store_n(&v_, 0, __ATOMIC_RELEASE); }
};
} // namespace detail
} // namespace boost
#endif
