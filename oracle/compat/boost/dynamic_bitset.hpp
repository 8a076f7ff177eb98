// Boost-subset shim (self-written, test infrastructure): a resizable bitset
// with the members the reference uses: (n, value) construction, [] read and
// write through a proxy, set(), reset(), resize(), size().  Bit writes are
// atomic so that parallel writers of neighbouring bits do not lose updates.
#ifndef KCNA_SHIM_BOOST_DYNAMIC_BITSET_HPP
#define KCNA_SHIM_BOOST_DYNAMIC_BITSET_HPP
#include <cstddef>
#include <cstdint>
#include <vector>
namespace boost {
template <typename Block = unsigned long>
struct dynamic_bitset {
    typedef std::size_t size_type;
    std::vector<uint64_t> w_;
    size_type n_ = 0;
    struct reference {
        uint64_t *w;
        uint64_t m;
        operator bool() const { return (__atomic_load_n(w, __ATOMIC_RELAXED) & m) != 0; }
        reference &operator=(bool v) {
            if (v)
                __atomic_fetch_or(w, m, __ATOMIC_RELAXED);
            else
                __atomic_fetch_and(w, ~m, __ATOMIC_RELAXED);
            return *this;
        }
        reference &operator=(const reference &o) { return *this = bool(o); }
        bool operator~() const { return !bool(*this); }
    };
    dynamic_bitset() {}
    explicit dynamic_bitset(size_type n, unsigned long value = 0) { resize(n); if (n) w_[0] = value; trim(); }
    void trim() { if (n_ % 64 && !w_.empty()) w_.back() &= (~0ull >> (64 - n_ % 64)); }
    void resize(size_type n, bool v = false) {
        size_type old = n_;
        n_ = n;
        w_.resize((n + 63) / 64, 0);
        if (v) for (size_type i = old; i < n; ++i) (*this)[i] = true;
        trim();
    }
    size_type size() const { return n_; }
    reference operator[](size_type i) { return reference{&w_[i / 64], 1ull << (i % 64)}; }
    bool operator[](size_type i) const { return (w_[i / 64] >> (i % 64)) & 1; }
    bool test(size_type i) const { return (*this)[i]; }
    dynamic_bitset &set() { for (auto &x : w_) x = ~0ull; trim(); return *this; }
    dynamic_bitset &set(size_type i, bool v = true) { (*this)[i] = v; return *this; }
    dynamic_bitset &reset() { for (auto &x : w_) x = 0; return *this; }
    dynamic_bitset &reset(size_type i) { (*this)[i] = false; return *this; }
    size_type count() const { size_type c = 0; for (auto x : w_) c += __builtin_popcountll(x); return c; }
};
} // namespace boost
#endif
