// kcna_sort.cuh - shared-memory and warp sorting/merging primitives.
#pragma once
#include "kcna_common.cuh"

// Ascending bitonic sort of n (a power of two) 64-bit keys in shared memory by
// the whole thread block.  Ends with a __syncthreads.
__device__ __forceinline__ void kcna_cta_bitonic(uint64_t *s, int n) {
    for (int size = 2; size <= n; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            __syncthreads();
            for (int t = threadIdx.x; t < (n >> 1); t += blockDim.x) {
                int i = ((t & ~(stride - 1)) << 1) | (t & (stride - 1));
                int j = i + stride;
                bool asc = (i & size) == 0;
                uint64_t a = s[i], b = s[j];
                if ((a > b) == asc) {
                    s[i] = b;
                    s[j] = a;
                }
            }
        }
    }
    __syncthreads();
}

// Ascending bitonic sort of n (power of two, <= 32*E) keys in shared memory by
// one warp (no block barrier).
__device__ __forceinline__ void kcna_warp_bitonic(uint64_t *s, int n) {
    const int lane = kcna_lane();
    for (int size = 2; size <= n; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            __syncwarp();
            for (int t = lane; t < (n >> 1); t += 32) {
                int i = ((t & ~(stride - 1)) << 1) | (t & (stride - 1));
                int j = i + stride;
                bool asc = (i & size) == 0;
                uint64_t a = s[i], b = s[j];
                if ((a > b) == asc) {
                    s[i] = b;
                    s[j] = a;
                }
            }
        }
    }
    __syncwarp();
}

// Ascending bitonic sort of n (a power of two) keys in shared memory by one
// warp, each carrying a 16-bit value that moves with it (values of equal keys
// end in no particular order).
__device__ __forceinline__ void kcna_warp_bitonic_kv16(uint64_t *s, uint16_t *v, int n) {
    const int lane = kcna_lane();
    for (int size = 2; size <= n; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            __syncwarp();
            for (int t = lane; t < (n >> 1); t += 32) {
                int i = ((t & ~(stride - 1)) << 1) | (t & (stride - 1));
                int j = i + stride;
                bool asc = (i & size) == 0;
                uint64_t a = s[i], b = s[j];
                if ((a > b) == asc) {
                    s[i] = b;
                    s[j] = a;
                    const uint16_t va = v[i];
                    v[i] = v[j];
                    v[j] = va;
                }
            }
        }
    }
    __syncwarp();
}

// Ascending sort of s[0, n), any n >= 1, by one warp in shared memory: the
// bitonic network in its flip form (every comparator puts the smaller key at
// the lower index), padded to the next power of two with virtual +infinite
// keys.  A comparator that touches a virtual key leaves both in place, so
// only the comparators inside [0, n) run and nothing beyond n is read or
// written.  With KV every key carries a 16-bit value from v (values of equal
// keys end in no particular order).
template <bool KV>
__device__ __forceinline__ void kcna_warp_sort_n(uint64_t *s, uint16_t *v, int n) {
    const int lane = kcna_lane();
    int p2 = 1;
    while (p2 < n) p2 <<= 1;
    for (int size = 2; size <= p2; size <<= 1) {
        const int half = size >> 1;
        for (int stride = half; stride > 0; stride >>= 1) {
            __syncwarp();
            const bool flip = stride == half;
            // pairs are numbered in increasing order of their lower index i:
            // those with i < n come first
            const int tmax = (n / (2 * stride)) * stride + min(n % (2 * stride), stride);
            for (int t = lane; t < tmax; t += 32) {
                const int i = ((t & ~(stride - 1)) << 1) | (t & (stride - 1));
                const int j = flip ? (i ^ (size - 1)) : i + stride;
                if (j >= n) continue;
                const uint64_t a = s[i], b = s[j];
                if (b < a) {
                    s[i] = b;
                    s[j] = a;
                    if (KV) {
                        const uint16_t va = v[i];
                        v[i] = v[j];
                        v[j] = va;
                    }
                }
            }
        }
    }
    __syncwarp();
}

// Ascending bitonic sort of n (a power of two) (key, value) pairs in shared
// memory by the whole thread block, ordered by key then value: among equal
// keys the pair with the smallest value comes first.  Ends with a
// __syncthreads.
__device__ __forceinline__ void kcna_cta_bitonic_kv(uint64_t *s, uint32_t *v, int n) {
    for (int size = 2; size <= n; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            __syncthreads();
            for (int t = threadIdx.x; t < (n >> 1); t += blockDim.x) {
                int i = ((t & ~(stride - 1)) << 1) | (t & (stride - 1));
                int j = i + stride;
                bool asc = (i & size) == 0;
                uint64_t a = s[i], b = s[j];
                uint32_t va = v[i], vb = v[j];
                const bool gt = a > b || (a == b && va > vb);
                if (gt == asc) {
                    s[i] = b;
                    s[j] = a;
                    v[i] = vb;
                    v[j] = va;
                }
            }
        }
    }
    __syncthreads();
}

// Register bitonic sort of 32 keys, one per lane, ascending by lane.
__device__ __forceinline__ uint64_t kcna_warp_sort32(uint64_t v) {
    const int lane = kcna_lane();
#pragma unroll
    for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            uint64_t o = __shfl_xor_sync(KCNA_FULL, v, stride);
            bool up = (lane & size) == 0;
            bool lower = (lane & stride) == 0;
            uint64_t mn = v < o ? v : o, mx = v < o ? o : v;
            v = (up == lower) ? mn : mx;
        }
    }
    return v;
}

static inline int kcna_pow2_ceil(int x) {
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}
__device__ __forceinline__ int kcna_pow2_ceil_d(int x) {
    return x <= 1 ? 1 : 1 << (32 - __clz(x - 1));
}

// Number of elements of sorted a[0..na) strictly less than key (lower bound).
__device__ __forceinline__ int kcna_lower_bound(const uint64_t *a, int na, uint64_t key) {
    int lo = 0, hi = na;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] < key)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}
__device__ __forceinline__ int kcna_upper_bound(const uint64_t *a, int na, uint64_t key) {
    int lo = 0, hi = na;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] <= key)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}
