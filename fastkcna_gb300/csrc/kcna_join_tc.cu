// kcna_join_tc.cu - NN-descent local join on tcgen05 Gram tiles.
//
// Same work as join_kernel (kcna_nnd.cu; reference join src/kgraph.cpp:1097-1117
// with Nhood::join :970-987): for node n, every pair of its new list A
// (i < j) and of A x old list B, each pair emitted to both endpoints'
// candidate buffers when within that endpoint's radius.  Here the distances
// come from Gram tiles: d(i, j) = (|x_i|^2 + |x_j|^2) - 2 <x_i, x_j>, with the
// dot products from tcgen05.mma on BF16 rows and FP32 accumulation in TMEM.
// The kernel runs only in Gram-exact mode (integer rows, squared norms below
// 2^23): every product and partial sum is then an integer below 2^24, so the
// tile distance is the canonical FMA-chain distance bit for bit and the join
// emits exactly the candidates of the FP32 kernel.
//
// Block layout (persistent; one node at a time per block, 8 warps):
//   set         A (na <= 128 new ids) followed by B (old ids), ncol entries.
//   operands    M side: the set in tiles of 128 rows; N side: A (NA = na
//               rounded up to 16 columns), staged once per node.  Every TMEM
//               lane (a set member) then meets only real new-list columns, so
//               the emission work is ncol x NA pair checks, not 128 x ncol.
//   staging     cp.async 16-byte gathers of BF16 rows into the 128-byte
//               swizzled K-major layout; tiles rotate through two slots, the
//               slot of tile r+2 being gathered while tile r is emitted.
//   MMA         one thread issues 4 (K=16) x 2 (64-element K blocks)
//               tcgen05.mma (M = 128, N = NA) per tile into one of two
//               128-column TMEM buffers and commits to that buffer's mbarrier.
//   emission    warp w reads TMEM lanes 32*(w%4).. (set members) and column
//               groups of 16 with parity w/4; a set member's candidates are
//               counted per thread, a new member's by warp ballots; one
//               atomicAdd per target and tile reserves a contiguous run in the
//               target's candidate buffer.
#include <algorithm>

#include "kcna_internal.h"
#include "kcna_join.cuh"
#include "kcna_tc.cuh"

using namespace kcna_tc;

namespace {

constexpr int TJ = 256;                      // threads per block
constexpr int TROWS = 128;                   // set rows per tile (MMA M), max new-list columns
constexpr uint32_t KBB = 128;                // bytes of a row inside one 64-element K block
constexpr uint32_t TILE = TROWS * KBB * 2;   // 128 rows, two K blocks (d <= 128): 32 KiB
constexpr uint32_t TILES = 3 * TILE;         // new-list rows + two rotating set tiles
constexpr uint32_t TMEM_COLS = 2 * TROWS;    // two accumulator buffers
constexpr int MAXG = TROWS / 16 / 2;         // column groups of 16 per warp half

// Gathers rows first..first+count-1 of the column list into rows 0..count-1 of
// a 128-row region (K block kb of row r at kb*128*128 + swizzle).
__device__ __forceinline__ void stage_rows(uint32_t region, const uint32_t *s_col, int first, int count,
                                           const uint16_t *__restrict__ Xh, int ldh, int nc16) {
    for (int idx = threadIdx.x; idx < count * nc16; idx += TJ) {
        const int r = idx / nc16, c = idx - r * nc16;
        const uint16_t *src = Xh + (uint64_t)s_col[first + r] * (uint64_t)ldh + c * 8;
        cp_async16(region + (uint32_t)(c >> 3) * TROWS * KBB + sw128_off((uint32_t)r, (uint32_t)(c & 7)), src);
    }
}

// D[128 x N] = rows(a) . rows(b)^T over nkb K blocks of 64 elements.
__device__ __forceinline__ void issue_tile(uint32_t tmem_d, uint32_t a_base, uint32_t b_base, uint32_t idesc,
                                           int nkb) {
    for (int kb = 0; kb < nkb; ++kb)
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
            mma_bf16(tmem_d, desc_sw128(a_base + kb * TROWS * KBB + kk * 32),
                     desc_sw128(b_base + kb * TROWS * KBB + kk * 32), idesc, (kb | kk) ? 1u : 0u);
}

__global__ void __launch_bounds__(TJ, 2) join_tc_kernel(JoinArgs a, const uint16_t *__restrict__ Xh, int ldh,
                                                        const float *__restrict__ norms, uint32_t colcap) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ uint64_t mbar[2];
    __shared__ uint32_t s_tmem, s_tmp;
    __shared__ unsigned s_emit;
    __shared__ uint8_t s_rcnt[2][TROWS], s_ccnt[4][TROWS];
    __shared__ uint32_t s_rbase[2][TROWS], s_cbase[4][TROWS];
    const uint32_t tiles_s = (smem_u32(smem_raw) + 1023u) & ~1023u; // swizzled tiles need 1024-byte alignment
    unsigned char *tiles = smem_raw + (tiles_s - smem_u32(smem_raw));
    uint32_t *s_col = reinterpret_cast<uint32_t *>(tiles + TILES); // set ids: A then B
    float *s_rad = reinterpret_cast<float *>(s_col + colcap);      // radius of each set id
    float *s_nrm = s_rad + colcap;                                 // squared norm of each set id
    const uint32_t tA = tiles_s, tS = tiles_s + TILE;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int q = warp & 3, h = warp >> 2; // TMEM lane quarter, column-group parity
    const int nc16 = ldh >> 3, nkb = (ldh + 63) >> 6;

    // K padding beyond ldh is never written by the gathers and must read as zero
    for (int i = tid; i < (int)(TILES / 16); i += TJ) reinterpret_cast<uint4 *>(tiles)[i] = make_uint4(0, 0, 0, 0);
    if (warp == 0) tmem_alloc(&s_tmem, TMEM_COLS);
    if (tid == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_emit = 0;
    }
    fence_proxy_async();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = s_tmem;
    uint32_t phase = 0u; // bit b: parity of the next completion of buffer b's mbarrier
    uint32_t pend = 0u;  // bit b: buffer b has a commit not yet waited for
    bool ok = true;
    unsigned long long pairs = 0, rows_g = 0, emitted = 0;

    for (uint32_t node = blockIdx.x; node < a.N && ok; node += gridDim.x) {
        // new list: forward new, then a random subset (<= R) of reverse new
        const uint32_t fn = min(a.fwd_new_cnt[node], a.fwd_new_cap);
        for (uint32_t i = tid; i < fn; i += TJ) s_col[i] = a.fwd_new[(uint64_t)node * a.fwd_new_cap + i];
        __syncthreads();
        uint32_t rn = 0;
        if (a.iter > 0) {
            take_reverse(a.rnew + (uint64_t)node * a.RB, a.rnew_cnt[node], a.RB, a.R, a.seed,
                         join_reverse_stream(a.iter, node, 0), s_col + fn, &s_tmp);
            rn = s_tmp;
        }
        const int na = (int)min(fn + rn, (uint32_t)TROWS);
        // old list after A: forward old, then a random subset of reverse old
        const uint32_t fo = min(a.fwd_old_cnt[node], a.fwd_old_cap);
        for (uint32_t i = tid; i < fo; i += TJ) s_col[na + i] = a.fwd_old[(uint64_t)node * a.fwd_old_cap + i];
        __syncthreads();
        uint32_t ro = 0;
        if (a.iter > 0) {
            take_reverse(a.rold + (uint64_t)node * a.RB, a.rold_cnt[node], a.RB, a.R, a.seed,
                         join_reverse_stream(a.iter, node, 1), s_col + na + fo, &s_tmp);
            ro = s_tmp;
        }
        const int nb = (int)(fo + ro), ncol = na + nb;
        if (na == 0) {
            __syncthreads();
            continue;
        }
        for (int j = tid; j < ncol; j += TJ) {
            const uint32_t id = s_col[j];
            s_rad[j] = __ldg(a.radius + id);
            s_nrm[j] = __ldg(norms + id);
        }
        if (tid == 0) {
            pairs += (unsigned long long)na * (na - 1) / 2 + (unsigned long long)na * nb;
            rows_g += (unsigned long long)ncol;
        }
        const int NA = (na + 15) & ~15, G = NA >> 4; // MMA N and its column groups
        const uint32_t idesc = idesc_bf16(TROWS, NA);
        const int ntile = (ncol + TROWS - 1) / TROWS;
        stage_rows(tA, s_col, 0, na, Xh, ldh, nc16);
        stage_rows(tS, s_col, 0, min(ncol, TROWS), Xh, ldh, nc16);
        if (ntile > 1) stage_rows(tS + TILE, s_col, TROWS, min(ncol - TROWS, TROWS), Xh, ldh, nc16);
        cp_async_wait_all();
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            fence_after();
            issue_tile(tmem, tS, tA, idesc, nkb);
            mma_commit(&mbar[0]);
            if (ntile > 1) {
                issue_tile(tmem + TROWS, tS + TILE, tA, idesc, nkb);
                mma_commit(&mbar[1]);
            }
        }
        pend = ntile > 1 ? 3u : 1u;
        for (int r = 0; r < ntile; ++r) {
            const int b = r & 1;
            if (mbar_wait(&mbar[b], (phase >> b) & 1u)) {
                phase ^= 1u << b;
                pend &= ~(1u << b);
            } else {
                ok = false;
            }
            fence_after();
            // tile r+2 goes to slot b, free now that tile r's products are done
            if (r + 2 < ntile) {
                const int first = (r + 2) * TROWS;
                stage_rows(tS + b * TILE, s_col, first, min(ncol - first, TROWS), Xh, ldh, nc16);
            }
            const int j = r * TROWS + 32 * q + lane; // this thread's set member
            const bool warp_live = r * TROWS + 32 * q < ncol;
            const bool rowv = j < ncol;
            const uint32_t id_j = rowv ? s_col[j] : 0u;
            const float rad_j = rowv ? s_rad[j] : -1.f;
            const float n_j = rowv ? s_nrm[j] : 0.f;
            const uint32_t trow = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * TROWS);
            uint64_t rmask = 0;
            uint32_t cmA = 0, cmB = 0; // ballot masks of this warp's local columns lane and lane+32
            if (warp_live) {
#pragma unroll 1
                for (int k = 0; k < MAXG; ++k) {
                    const int g = h + 2 * k;
                    if (g >= G) break;
                    uint32_t raw[16];
                    tmem_ld16_async(trow + 16 * g, raw);
                    tmem_wait_ld16(raw);
#pragma unroll
                    for (int t = 0; t < 16; ++t) {
                        const int i = 16 * g + t; // new-list column
                        const int ii = min(i, na - 1);
                        const float dd = __fsub_rn(__fadd_rn(n_j, s_nrm[ii]), 2.f * __uint_as_float(raw[t]));
                        const bool pv = rowv && i < na && (j >= na || i < j) && s_col[ii] != id_j;
                        rmask |= (uint64_t)(pv && dd <= rad_j) << (16 * k + t);
                        const unsigned m = __ballot_sync(KCNA_FULL, pv && dd <= s_rad[ii]);
                        const int c = 16 * k + t; // local column
                        if (lane == (c & 31)) {
                            if (c < 32)
                                cmA = m;
                            else
                                cmB = m;
                        }
                    }
                }
            }
            s_rcnt[h][32 * q + lane] = (uint8_t)__popcll(rmask);
            // column counts of this quarter: local column c = 16k + t <-> column 16(h + 2k) + t
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                const int c = lane + 32 * half, k = c >> 4;
                const int i = 16 * (h + 2 * k) + (c & 15);
                if (k < MAXG && h + 2 * k < G) s_ccnt[q][i] = (uint8_t)__popc(half ? cmB : cmA);
            }
            __syncthreads();
            // one reservation per target: set members by threads 0..127, new-list columns by 128..255
            if (tid < TROWS) {
                const uint32_t tot = (uint32_t)s_rcnt[0][tid] + s_rcnt[1][tid];
                if (tot) {
                    const uint32_t base = atomicAdd(a.cand_cnt + s_col[r * TROWS + tid], tot);
                    s_rbase[0][tid] = base;
                    s_rbase[1][tid] = base + s_rcnt[0][tid];
                    atomicAdd(&s_emit, tot);
                }
            } else {
                const int i = tid - TROWS;
                if (i < na) {
                    const uint32_t c0 = s_ccnt[0][i], c1 = s_ccnt[1][i], c2 = s_ccnt[2][i], c3 = s_ccnt[3][i];
                    const uint32_t tot = c0 + c1 + c2 + c3;
                    if (tot) {
                        const uint32_t base = atomicAdd(a.cand_cnt + s_col[i], tot);
                        s_cbase[0][i] = base;
                        s_cbase[1][i] = base + c0;
                        s_cbase[2][i] = base + c0 + c1;
                        s_cbase[3][i] = base + c0 + c1 + c2;
                        atomicAdd(&s_emit, tot);
                    }
                }
            }
            __syncthreads();
            if (warp_live) { // writes; the distances are read again from TMEM
                const uint32_t flags = (uint32_t)(KCNA_FLAG_NEW | KCNA_FLAG_ISNEW);
                uint32_t p = s_rbase[h][32 * q + lane];
                uint64_t *dst = a.cand + (uint64_t)id_j * a.CB;
#pragma unroll 1
                for (int k = 0; k < MAXG; ++k) {
                    const int g = h + 2 * k;
                    if (g >= G) break;
                    const uint32_t gm = (uint32_t)(rmask >> (16 * k)) & 0xFFFFu;
                    const uint32_t cm = k < 2 ? cmA : cmB;
                    if (!__any_sync(KCNA_FULL, gm != 0u || cm != 0u)) continue;
                    uint32_t raw[16];
                    tmem_ld16_async(trow + 16 * g, raw);
                    tmem_wait_ld16(raw);
#pragma unroll
                    for (int t = 0; t < 16; ++t) {
                        const int i = 16 * g + t;
                        const int ii = min(i, na - 1);
                        const float dd = __fsub_rn(__fadd_rn(n_j, s_nrm[ii]), 2.f * __uint_as_float(raw[t]));
                        if ((gm >> t) & 1u) {
                            if (p < a.CB) dst[p] = kcna_key(dd, s_col[ii], flags);
                            ++p;
                        }
                        const int c = 16 * k + t;
                        const unsigned m = __shfl_sync(KCNA_FULL, c < 32 ? cmA : cmB, c & 31);
                        if ((m >> lane) & 1u) {
                            const uint32_t pc = s_cbase[q][ii] + __popc(m & kcna_lanemask_lt());
                            if (pc < a.CB) a.cand[(uint64_t)s_col[ii] * a.CB + pc] = kcna_key(dd, id_j, flags);
                        }
                    }
                }
            }
            // slot b gathered and TMEM buffer b read by every thread: tile r+2 may start
            cp_async_wait_all();
            fence_proxy_async();
            fence_before();
            ok = __syncthreads_and(ok) != 0;
            if (ok && r + 2 < ntile) {
                if (tid == 0) {
                    fence_after();
                    issue_tile(tmem + b * TROWS, tS + b * TILE, tA, idesc, nkb);
                    mma_commit(&mbar[b]);
                }
                pend |= 1u << b;
            }
            if (!ok) break;
        }
        // found: this node's join emitted a candidate
        if (tid == 0) {
            a.found[node] = s_emit ? 1 : 0;
            emitted += s_emit;
            s_emit = 0;
        }
    }
    // after a wait gave up: wait (bounded) for the products still in flight
    // before the accumulator columns are released
    for (int b = 0; b < 2; ++b)
        if ((pend >> b) & 1u) (void)mbar_wait(&mbar[b], (phase >> b) & 1u);
    if (tid == 0) {
        atomicAdd(a.counters + 0, pairs);
        atomicAdd(a.counters + 5, rows_g);
        atomicAdd(a.counters + 6, emitted);
    }
    fence_before();
    __syncthreads();
    if (warp == 0) tmem_free(tmem, TMEM_COLS);
    if (!ok && tid == 0) kcna_set_err(a.err, KCNA_DERR_SPIN);
}

} // namespace

kcna_status kcna_join_tc_launch(kcna_ctx *c, const JoinArgs &a) {
    if (!c->gram_exact || !c->Xh || !c->norms || (c->ld & 7u) || c->ld > 128)
        return kcna_fail(c, KCNA_E_STATE, "Gram-tile join needs exact BF16 rows with d <= 128");
    const uint32_t colcap = std::max<uint32_t>(a.capA, TROWS + a.capB);
    const size_t sm = 1024 + TILES + (size_t)colcap * 12;
    KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(join_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm),
                             "join_tc smem attr"));
    // all of the unified L1 as shared memory, so that two blocks fit per SM
    KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(join_tc_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                                     (int)cudaSharedmemCarveoutMaxShared),
                             "join_tc carveout"));
    int per_sm = 0;
    KCNA_TRY(kcna_cuda_check(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, join_tc_kernel, TJ, sm),
                             "join_tc occupancy"));
    per_sm = std::min(std::max(per_sm, 1), 2); // 2 x 256 TMEM columns fill one SM's 512
    const uint32_t grid = (uint32_t)std::min<uint64_t>(a.N, (uint64_t)std::max(c->num_sms, 1) * per_sm);
    if (grid == 0) return KCNA_OK;
    join_tc_kernel<<<grid, TJ, sm, c->stream>>>(a, c->Xh, (int)c->ld, c->norms, colcap);
    KCNA_LAUNCHED(c);
    return kcna_cuda_check(c, cudaGetLastError(), "join_tc_kernel");
}
