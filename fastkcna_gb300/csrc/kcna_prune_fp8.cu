// kcna_prune_fp8.cu - occlusion prune of float rows at high dimension on
// FP8 E4M3 tcgen05 Gram tiles with per-vector scales, every undecided pair
// recomputed in FP32.
//
// Same kept lists as prune_kernel (kcna_graph.cu; reference taumg_sync_prune
// src/kgraph.cpp:2833-2876 and nsg_sync_prune :1809-1851): the candidates of
// node q are its pool entries [first, lim) in order; the first is kept; a
// later candidate p is dropped when an already kept t occludes it, d(t,p) <
// d(q,p) - 3 tau (tau = 0: RNG), and the scan stops at range kept.  d(t,p) is
// the canonical FP32 distance (one FMA chain over the dimensions in order).
//
// Rows are encoded once per build (fp8_rows_kernel): x ~ s * c, c in E4M3 with
// the scale s = max|x| / 448, beside s the squared norm n = |s c|^2 and an
// upper bound e on the encoding error |x - s c|.  The tile kernel takes the
// first PC = 128 candidates of each node and forms their Gram matrix
// G = C C^T of codes on the tensor cores (kind::f8f6f4, K streamed in 128-byte
// blocks), so that D~ = n_t + n_p - 2 s_t s_p G estimates the squared distance
// of the encoded rows.  For every pair t < p it decides, from bounds that hold
// whatever the rounding, whether
//   * t certainly occludes p:      (1 + g)(sqrt(D~ + dl) + E)^2 < th_p
//   * t certainly does not:        (1 - g)(sqrt(D~ - dl) - E)^2 >= th_p
//   * otherwise the pair is undecided,
// with th_p = d(q,p) - 3 tau (FP32, as the reference computes it), E = e_t +
// e_p (the triangle inequality between |t - p| and |s_t c_t - s_p c_p|),
// dl = 2^-7 (n_t + n_p) (the FP32 products and sums of D~ and the tensor
// cores' accumulation; the GPU test measures the accumulation error to be
// far smaller), and g = (d + 2) 2^-24 + 1e-5 (the error of the canonical FP32
// chain against the real distance, and the rounding of the comparison
// itself).  The scan resolves the sequential rule on bit masks (certain
// occluders, undecided pairs) and computes the canonical FP32 distance only
// for undecided pairs between a kept t and a still live p.  A node whose scan
// reaches the end of the tile with fewer than range kept and more candidates
// left is finished by the FP32 warp prune (kcna_prune_resume, kcna_graph.cu),
// which continues from the kept list.
//
// The screen pays where the rule's margin is wide against the FP8 error: on
// the 960-dimensional C4 rows with tau = 10, every pair of the first 50
// candidates is decided "not occluded" by a wide margin, so the prune reads
// 128 one-byte rows per node and computes no FP32 distance at all.
//
// Block layout: persistent, one block per SM, warp-specialised, mbarrier
// hand-offs, every wait bounded (a wait that gives up sets the error word,
// lets in-flight copies and products finish, frees TMEM and returns):
//   warp 0       metadata: the node's pool prefix by one bulk copy (a node
//                ahead), ids, thresholds, the candidates' scales, norms and
//                error bounds, the initial dead set;
//   warps 11-14  loaders: the candidates' code rows, one 128-byte K block of
//                128 rows (16 KiB) at a time, by 16-byte cp.async into the
//                128-byte swizzled K-major layout, a ring of NS blocks;
//   warp 1       MMA issuer (one thread): G += A_kb A_kb^T for every K block
//                (four K = 32 steps each) into one of two 128-column TMEM
//                accumulators;
//   warps 2-9    mask builders: TMEM lane quarter (warp % 4) x column half;
//                64 pair decisions per thread into two bit planes;
//   warp 10      scan: the kept list, undecided pairs resolved in FP32.
#include <cuda_fp8.h>

#include <algorithm>

#include "kcna_internal.h"
#include "kcna_tc.cuh"

using namespace kcna_tc;

namespace {

constexpr int PC = 128;                    // candidates on the tile
constexpr int MWD = PC / 32;               // mask words per row
constexpr uint32_t KBB = 128;              // bytes (codes) of a row in one K block
constexpr uint32_t SLAB = PC * KBB;        // one K block of the tile's rows: 16 KiB
constexpr int NS = 8;                      // K-block ring
constexpr int NACC = 2;                    // 128-column TMEM accumulators
constexpr int NMASK = 8;                   // mask-building warps
constexpr int SCAN_W = 2 + NMASK;
constexpr int LOAD_W = SCAN_W + 1;
constexpr int NLOAD = 4;
constexpr int F8_THREADS = (LOAD_W + NLOAD) * 32;
constexpr float KAPPA = 1.0f / 128.0f;     // dl = KAPPA (n_t + n_p)

struct alignas(16) FMeta {
    uint64_t key[PC + 4]; // entries from an even index (16-byte bulk copy); candidate c at koff + c
    float th[PC];         // occlusion threshold: d(q,p) - 3 tau
    float rlo[PC];        // sqrt(th / (1 - g)): "certainly not" needs sqrt(D~ - dl) >= E + rlo
    float rhi[PC];        // sqrt(th / (1 + g)): "certainly" needs sqrt(D~ + dl) <= rhi - E
    float s[PC], n[PC], e[PC];
    uint32_t dead[MWD];
    uint32_t q, nc, ntot, koff;
};

struct FShared {
    uint64_t slab_full[NS], slab_empty[NS], acc_full[NACC], acc_empty[NACC];
    uint64_t keys_full[2], ids_ready[2], meta_full[2], mask_full[2], node_empty[2];
    uint32_t tmem;
    volatile int abort_flag;
    FMeta meta[2];
    uint32_t cm[2][MWD * PC]; // certain occlusion, word-major: word w of row t at w * PC + t
    uint32_t am[2][MWD * PC]; // undecided pairs
};

struct F8Args {
    uint32_t n_items;         // nodes (or list entries) to prune
    const uint32_t *nodes;    // list of nodes (null: item k is node k)
    const uint64_t *keys;     // candidate keys, row r = item (list) or node, `stride` apart
    uint64_t stride;
    const uint32_t *cnt;      // candidates of row r
    uint32_t n_oracle;        // ids at or beyond are skipped (the layer prefix), 0xFFFFFFFF: none
    const uint8_t *codes;     // E4M3 rows, ldq bytes apart (zero padded)
    uint32_t ldq;
    const float4 *qm;         // per row {s, n, e, 0}
    const float *X;           // FP32 rows (exact fallback), ld floats apart
    uint32_t ld;
    float t3, g;
    int range, maxc;
    uint32_t *g_ids;
    float *g_dist;
    uint32_t *g_deg;
    uint32_t W;
    uint32_t *resume;         // items left to the FP32 prune
    uint32_t *resume_cnt;
    unsigned long long *comps;
    unsigned long long *exact; // undecided pairs recomputed in FP32
    int *err;
};

__device__ __forceinline__ uint32_t idesc_e4m3(int M, int N) { // kind::f8f6f4, A/B E4M3, D FP32, K-major
    return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_e4m3(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_wait0() { asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory"); }

// Canonical FP32 distance of rows a and b (one FMA chain over the dimensions in order).
__device__ __noinline__ float exact_l2(const float *__restrict__ X, uint32_t ld, uint32_t a, uint32_t b) {
    return rows_l2(RowsF32{X, (int)ld}, a, b);
}

__global__ void __launch_bounds__(F8_THREADS, 1) prune_fp8_kernel(F8Args a) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t tiles_s = (smem_u32(smem_raw) + 1023u) & ~1023u;
    unsigned char *tiles = smem_raw + (tiles_s - smem_u32(smem_raw));
    FShared &S = *reinterpret_cast<FShared *>(tiles + NS * SLAB);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nkb = (int)(a.ldq / KBB);

    if (warp == 1) tmem_alloc(&S.tmem, NACC * PC);
    if (tid == 0) {
        for (int i = 0; i < NS; ++i) {
            mbar_init(&S.slab_full[i], NLOAD * 32);
            mbar_init(&S.slab_empty[i], 1);
        }
        for (int i = 0; i < NACC; ++i) {
            mbar_init(&S.acc_full[i], 1);
            mbar_init(&S.acc_empty[i], NMASK);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&S.keys_full[i], 1);
            mbar_init(&S.ids_ready[i], 1);
            mbar_init(&S.meta_full[i], 32);
            mbar_init(&S.mask_full[i], NMASK);
            mbar_init(&S.node_empty[i], 1 + NLOAD); // scan, loader warps
        }
        S.abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_proxy_async();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = S.tmem;
    bool ok = true;

    if (warp == 0) {
        // ------------------------------------------------------------ metadata
        uint32_t r_cnt[2] = {0u, 0u}, r_shift[2] = {0u, 0u};
        int pending = -1;
        // item k (the block's kk-th) into metadata slot kk & 1
        auto request = [&](uint32_t k, uint32_t kk) {
            if (k >= a.n_items) return;
            const int b = (int)(kk & 1u);
            const uint32_t q = a.nodes ? a.nodes[k] : k;
            const uint64_t row = a.nodes ? k : q;
            pending = (int)kk;
            const uint32_t cnt = a.cnt[a.nodes ? k : q];
            const uint64_t base = row * a.stride;
            const uint32_t shift = (uint32_t)(base & 1u);
            const uint32_t ncopy = min(cnt, (uint32_t)PC + 1u);
            const uint32_t nent = (shift + ncopy + 1u) & ~1u;
            r_cnt[b] = cnt;
            r_shift[b] = shift;
            if (lane == 0) {
                if (nent) {
                    fence_proxy_async();
                    mbar_arrive_expect_tx(&S.keys_full[b], nent * 8u);
                    bulk_copy_g2s(smem_u32(S.meta[b].key), a.keys + (base - shift), nent * 8u, &S.keys_full[b]);
                } else {
                    mbar_arrive(&S.keys_full[b]);
                }
            }
        };
        uint32_t kk = 0;
        request(blockIdx.x, 0u);
        for (uint32_t k = blockIdx.x; k < a.n_items; k += gridDim.x, ++kk) {
            const int sl = (int)(kk & 1u);
            if (!mbar_wait(&S.keys_full[sl], (kk >> 1) & 1u)) { ok = false; break; }
            pending = -1;
            if (S.abort_flag) { ok = false; break; }
            FMeta &M = S.meta[sl];
            const uint32_t q = a.nodes ? a.nodes[k] : k;
            const int cnt = (int)r_cnt[sl];
            const uint32_t shift = r_shift[sl];
            int first = 0;
            if (cnt > 0 && kcna_key_id(M.key[shift]) == q) first = 1;
            const int ntot = first < cnt ? max(min(cnt, a.maxc), first + 1) - first : 0;
            const int nc = min(ntot, PC);
            const uint32_t koff = shift + (uint32_t)first;
#pragma unroll
            for (int i = 0; i < MWD; ++i) {
                const int c = 32 * i + lane;
                const bool live = c < nc;
                uint32_t id = 0u, before = 0xFFFFFFFFu;
                float th = 0.f, pd = 0.f;
                float4 m4 = make_float4(1.f, 0.f, 0.f, 0.f);
                if (live) {
                    const uint64_t key = M.key[koff + c];
                    id = kcna_key_id(key);
                    pd = kcna_key_dist(key);
                    if (c > 0) before = kcna_key_id(M.key[koff + c - 1]);
                    if (id < a.n_oracle) m4 = __ldg(a.qm + id);
                }
                th = __fsub_rn(pd, a.t3); // src/kgraph.cpp:2859 (tau = 0: RNG's d(q,p))
                const float thp = fmaxf(th, 0.f);
                M.th[c] = th;
                M.rlo[c] = sqrtf(__fdiv_rn(thp, 1.f - a.g));
                M.rhi[c] = sqrtf(__fdiv_rn(thp, 1.f + a.g));
                M.s[c] = m4.x;
                M.n[c] = m4.y;
                M.e[c] = m4.z;
                // src/kgraph.cpp:1822: ids beyond the layer prefix are skipped; a
                // repeated id is occluded by its twin
                const bool dead = !live || (c > 0 && (id >= a.n_oracle || id == before));
                const unsigned dm = __ballot_sync(KCNA_FULL, dead);
                if (lane == 0) M.dead[i] = dm;
            }
            if (lane == 0) {
                M.q = q;
                M.nc = (uint32_t)nc;
                M.ntot = (uint32_t)ntot;
                M.koff = koff;
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.ids_ready[sl]);
            mbar_arrive(&S.meta_full[sl]);
            const uint32_t kn = k + gridDim.x;
            if (kn < a.n_items) {
                if (kk >= 1 && !mbar_wait(&S.node_empty[sl ^ 1], ((kk - 1) >> 1) & 1u)) { ok = false; break; }
                request(kn, kk + 1u);
            }
        }
        // a key copy still in flight lands before the block exits
        if (pending >= 0) (void)mbar_wait(&S.keys_full[pending & 1], ((uint32_t)pending >> 1) & 1u, 1u << 16);
        if (!ok) S.abort_flag = 1;
    } else if (warp >= LOAD_W) {
        // ------------------------------------------------------------- loaders
        const int lt = (warp - LOAD_W) * 32 + lane; // row of the tile
        uint32_t gsl = 0;
        int pend = -1;
        uint32_t kk = 0;
        for (uint32_t k = blockIdx.x; k < a.n_items; k += gridDim.x, ++kk) {
            const int sl = (int)(kk & 1u);
            if (!mbar_wait(&S.ids_ready[sl], (kk >> 1) & 1u) || S.abort_flag) { ok = false; break; }
            const FMeta &M = S.meta[sl];
            const bool row_live = lt < (int)M.nc;
            const uint8_t *src = a.codes;
            if (row_live) src += (uint64_t)kcna_key_id(M.key[M.koff + lt]) * a.ldq;
            for (int kb = 0; kb < nkb; ++kb, ++gsl) {
                const int s = (int)(gsl % NS);
                if (gsl >= (uint32_t)NS && !mbar_wait(&S.slab_empty[s], ((gsl / NS) - 1) & 1u)) { ok = false; break; }
                const uint32_t slab = tiles_s + (uint32_t)s * SLAB;
                if (row_live) {
#pragma unroll
                    for (int cc = 0; cc < 8; ++cc)
                        cp_async16(slab + sw128_off((uint32_t)lt, (uint32_t)cc), src + (uint32_t)kb * KBB + cc * 16);
                }
                cp_commit();
                if (pend >= 0) {
                    cp_wait1();
                    fence_proxy_async();
                    mbar_arrive(&S.slab_full[pend]);
                }
                pend = s;
            }
            if (pend >= 0) {
                cp_wait0();
                fence_proxy_async();
                mbar_arrive(&S.slab_full[pend]);
                pend = -1;
            }
            if (!ok) break;
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.node_empty[sl]);
        }
        cp_wait0();
        if (!ok) S.abort_flag = 1;
    } else if (warp == 1) {
        // ---------------------------------------------------------- MMA issuer
        if (lane == 0) {
            const uint32_t idesc = idesc_e4m3(PC, PC);
            uint32_t gsl = 0, kk = 0;
            for (uint32_t k = blockIdx.x; k < a.n_items && ok; k += gridDim.x, ++kk) {
                const int b = (int)(kk % NACC);
                if (S.abort_flag) { ok = false; break; }
                if (kk >= (uint32_t)NACC && !mbar_wait(&S.acc_empty[b], ((kk / NACC) - 1) & 1u)) { ok = false; break; }
                for (int kb = 0; kb < nkb; ++kb, ++gsl) {
                    const int s = (int)(gsl % NS);
                    if (!mbar_wait(&S.slab_full[s], (gsl / NS) & 1u)) { ok = false; break; }
                    fence_after();
                    const uint32_t slab = tiles_s + (uint32_t)s * SLAB;
#pragma unroll
                    for (int ks = 0; ks < 4; ++ks)
                        mma_e4m3(tmem + (uint32_t)(b * PC), desc_sw128(slab + ks * 32), desc_sw128(slab + ks * 32),
                                 idesc, (kb | ks) ? 1u : 0u);
                    mma_commit(&S.slab_empty[s]);
                }
                if (!ok) break;
                mma_commit(&S.acc_full[b]);
            }
            if (!ok) {
                S.abort_flag = 1;
                // products still in flight finish before TMEM is released: every K block
                // issued (of a node left half done too) was committed to its slab's
                // barrier, and the last commit tracks every product issued before it
                if (gsl > 0) {
                    const uint32_t last = gsl - 1u;
                    (void)mbar_wait(&S.slab_empty[last % NS], (last / NS) & 1u, 1u << 16);
                }
            }
        }
        __syncwarp();
    } else if (warp < SCAN_W) {
        // -------------------------------------------------------- mask builders
        const int qt = warp & 3, h = (warp - 2) >> 2; // TMEM lane quarter, column half
        const int t = 32 * qt + lane;
        uint32_t kk = 0;
        for (uint32_t k = blockIdx.x; k < a.n_items; k += gridDim.x, ++kk) {
            const int sl = (int)(kk & 1u), b = (int)(kk % NACC);
            bool mine = mbar_wait(&S.meta_full[sl], (kk >> 1) & 1u) && !S.abort_flag;
            mine = mine && mbar_wait(&S.acc_full[b], (kk / NACC) & 1u);
            if (!__all_sync(KCNA_FULL, mine)) { ok = false; break; }
            fence_after();
            const FMeta &M = S.meta[sl];
            uint32_t raw[64];
            const uint32_t ta = tmem + ((uint32_t)(32 * qt) << 16) + (uint32_t)(b * PC + 64 * h);
#pragma unroll
            for (int x = 0; x < 4; ++x) tmem_ld16_async(ta + 16 * x, raw + 16 * x);
#pragma unroll
            for (int x = 0; x < 4; ++x) tmem_wait_ld16(raw + 16 * x);
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.acc_empty[b]);
            const float s2 = -2.f * M.s[t], nt = M.n[t], et = M.e[t];
#pragma unroll
            for (int ww = 0; ww < 2; ++ww) {
                uint32_t cw = 0u, aw = 0u;
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const int p = 64 * h + 32 * ww + j;
                    const float nsum = nt + M.n[p];
                    const float dt = fmaf(s2 * M.s[p], __uint_as_float(raw[32 * ww + j]), nsum); // D~
                    const float dl = KAPPA * nsum;
                    const float E = et + M.e[p];
                    const float lo = E + M.rlo[p];
                    const float hi = M.rhi[p] - E;
                    const bool notocc = M.th[p] <= 0.f || dt - dl >= lo * lo;
                    const bool occ = hi > 0.f && dt + dl < hi * hi;
                    cw |= (occ ? 1u : 0u) << j;
                    aw |= (!notocc && !occ ? 1u : 0u) << j;
                }
                S.cm[sl][(2 * h + ww) * PC + t] = cw;
                S.am[sl][(2 * h + ww) * PC + t] = aw;
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.mask_full[sl]);
        }
        if (!ok) S.abort_flag = 1;
    } else {
        // ----------------------------------------------------------------- scan
        unsigned long long cc = 0, ex = 0;
        uint32_t kk = 0;
        for (uint32_t k = blockIdx.x; k < a.n_items; k += gridDim.x, ++kk) {
            const int sl = (int)(kk & 1u);
            const bool mine = mbar_wait(&S.mask_full[sl], (kk >> 1) & 1u) && !S.abort_flag;
            if (!__all_sync(KCNA_FULL, mine)) { ok = false; break; }
            const FMeta &M = S.meta[sl];
            const uint32_t *cm = S.cm[sl], *am = S.am[sl];
            const uint64_t *keys = M.key + M.koff;
            const int nc = (int)M.nc;
            uint32_t *gi = a.g_ids + (uint64_t)M.q * a.W;
            float *gd = a.g_dist + (uint64_t)M.q * a.W;
            int nk = 0;
            bool exhausted = false;
            if (nc > 0) {
                uint32_t dead = lane < MWD ? M.dead[lane] : 0xFFFFFFFFu;
                int t = 0;
                for (;;) {
                    const uint32_t tid_ = kcna_key_id(keys[t]);
                    if (lane == 0) {
                        gi[nk] = tid_;
                        gd[nk] = kcna_key_dist(keys[t]);
                        cc += (unsigned long long)nk;
                    }
                    ++nk;
                    if (nk >= a.range) break;
                    const int tw = t >> 5;
                    const uint32_t above = lane > tw ? 0xFFFFFFFFu : lane < tw ? 0u : ~((2u << (t & 31)) - 1u);
                    uint32_t o = 0u, u = 0u;
                    if (lane < MWD && lane >= tw) {
                        o = cm[lane * PC + t] & above;
                        u = am[lane * PC + t] & above & ~dead;
                    }
                    // undecided pairs with a live candidate: the canonical FP32 distance
#pragma unroll 1
                    for (int w = tw; w < MWD; ++w) {
                        const uint32_t bits = __shfl_sync(KCNA_FULL, u, w);
                        if (!bits) continue;
                        const bool mine = (bits >> lane) & 1u; // lane l takes candidate 32 w + l
                        bool hit = false;
                        if (mine) {
                            const int p = 32 * w + lane;
                            const float djk = exact_l2(a.X, a.ld, tid_, kcna_key_id(keys[p]));
                            hit = djk < M.th[p]; // src/kgraph.cpp:2859 (RNG: :1840)
                            ++ex;
                        }
                        const uint32_t hw = __ballot_sync(KCNA_FULL, hit);
                        if (lane == w) o |= hw;
                    }
                    cc += (unsigned long long)nk * __popc(o & ~dead); // dropped at the nk-th kept
                    dead |= o;
                    const uint32_t alive = ~dead & above;
                    const unsigned bal = __ballot_sync(KCNA_FULL, lane < MWD && alive != 0u);
                    if (!bal) {
                        exhausted = true;
                        break;
                    }
                    const int L = __ffs(bal) - 1;
                    t = 32 * L + __ffs(__shfl_sync(KCNA_FULL, alive, L)) - 1;
                }
            }
            const bool resume = exhausted && nk < a.range && M.ntot > (uint32_t)nc;
            __syncwarp();
            if (!resume)
                for (int j = nk + lane; j < (int)a.W; j += 32) {
                    gi[j] = KCNA_NONE;
                    gd[j] = 0.f;
                }
            if (lane == 0) {
                a.g_deg[M.q] = (uint32_t)nk;
                if (resume) a.resume[atomicAdd(a.resume_cnt, 1u)] = k;
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.node_empty[sl]);
        }
        cc = kcna_warp_sum(cc);
        ex = kcna_warp_sum(ex);
        if (lane == 0) {
            if (cc) atomicAdd(a.comps, cc);
            if (ex) atomicAdd(a.exact, ex);
        }
        if (!ok) S.abort_flag = 1;
    }
    fence_before();
    __syncthreads();
    if (warp == 1) tmem_free(tmem, NACC * PC);
    if (!ok) kcna_set_err(a.err, KCNA_DERR_SPIN);
}

size_t prune_fp8_smem() { return 1024 + (size_t)NS * SLAB + sizeof(FShared); }

// E4M3 codes with a per-row scale, the squared norm of the decoded row and
// a bound on the encoding error; warp per row.
__global__ void fp8_rows_kernel(const float *__restrict__ X, uint32_t n, uint32_t ld, uint32_t ldq,
                                uint8_t *__restrict__ codes, float4 *__restrict__ qm) {
    const uint64_t row = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    const float *x = X + row * ld;
    float amax = 0.f;
    for (uint32_t k = lane; k < ld; k += 32) amax = fmaxf(amax, fabsf(x[k]));
#pragma unroll
    for (int o = 16; o; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(KCNA_FULL, amax, o));
    const float s = amax > 0.f ? __fdiv_rn(amax, 448.f) : 1.f;
    float nn = 0.f, ee = 0.f;
    for (uint32_t k = lane; k < ldq; k += 32) {
        const float v = k < ld ? x[k] : 0.f;
        const __nv_fp8_storage_t c = __nv_cvt_float_to_fp8(__fdiv_rn(v, s), __NV_SATFINITE, __NV_E4M3);
        codes[row * ldq + k] = c;
        const __half_raw hr = __nv_cvt_fp8_to_halfraw(c, __NV_E4M3);
        const float dec = __half2float(__half(hr));
        const float xv = __fmul_rn(s, dec);
        nn = fmaf(xv, xv, nn);
        const float df = v - xv;
        ee = fmaf(df, df, ee);
    }
    nn = kcna_warp_sum(nn);
    ee = kcna_warp_sum(ee);
    if (lane == 0) {
        // the stored bound covers the FP32 sums and the rounding of s * c
        const float e = sqrtf(ee) * (1.f + 1.f / 1024.f) + sqrtf(nn) * (1.f / 4194304.f);
        qm[row] = make_float4(s, nn, e, 0.f);
    }
}

} // namespace

bool kcna_prune_fp8_ok(const kcna_ctx *c, int kind, int range, int maxc) {
    return kind == KCNA_TAUMNG && c->fp8_screen && c->Xq && c->qmeta && c->X && range >= 1 && maxc >= 1 &&
           prune_fp8_smem() <= 227 * 1024;
}

kcna_status kcna_fp8_rows(kcna_ctx *c) {
    const uint32_t ldq = (c->d + 127u) & ~127u;
    KCNA_TRY(kcna_alloc(c, &c->Xq, (size_t)c->n_total * ldq, "fp8 rows"));
    KCNA_TRY(kcna_alloc(c, &c->qmeta, c->n_total, "fp8 row scales"));
    c->ldq = ldq;
    fp8_rows_kernel<<<kcna_div_up((uint64_t)c->n_total * 32, 256), 256, 0, c->stream>>>(c->X, c->n_total, c->ld, ldq,
                                                                                       c->Xq, c->qmeta);
    KCNA_LAUNCHED(c);
    KCNA_TRY(kcna_cuda_check(c, cudaGetLastError(), "fp8_rows_kernel"));
    c->fp8_screen = true;
    return KCNA_OK;
}

kcna_status kcna_prune_fp8_launch(kcna_ctx *c, const uint64_t *keys, uint64_t stride, const uint32_t *cnt,
                                  const uint32_t *nodes, uint32_t n_items, uint32_t n_oracle, float t3, int range,
                                  int maxc, uint32_t *resume, uint32_t *resume_cnt, unsigned long long *comps,
                                  unsigned long long *exact) {
    if (n_items == 0) return KCNA_OK;
    F8Args a;
    a.n_items = n_items;
    a.nodes = nodes;
    a.keys = keys;
    a.stride = stride;
    a.cnt = cnt;
    a.n_oracle = n_oracle;
    a.codes = c->Xq;
    a.ldq = c->ldq;
    a.qm = c->qmeta;
    a.X = c->X;
    a.ld = c->ld;
    a.t3 = t3;
    a.g = (float)((c->d + 2) * (1.0 / 16777216.0) + 1e-5);
    a.range = range;
    a.maxc = maxc;
    a.g_ids = c->g_ids;
    a.g_dist = c->g_dist;
    a.g_deg = c->g_deg;
    a.W = c->W;
    a.resume = resume;
    a.resume_cnt = resume_cnt;
    a.comps = comps;
    a.exact = exact;
    a.err = c->d_err;
    const size_t sm = prune_fp8_smem();
    KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(prune_fp8_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)sm),
                             "prune_fp8 smem attr"));
    const uint32_t grid = (uint32_t)std::min<uint64_t>(n_items, (uint64_t)std::max(c->num_sms, 1));
    prune_fp8_kernel<<<grid, F8_THREADS, sm, c->stream>>>(a);
    KCNA_LAUNCHED(c);
    return kcna_cuda_check(c, cudaGetLastError(), "prune_fp8_kernel");
}
