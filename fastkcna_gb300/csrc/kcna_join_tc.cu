// kcna_join_tc.cu - NN-descent local join on tcgen05 Gram tiles, several
// nodes per tile.
//
// Same work as join_kernel (kcna_nnd.cu; reference join src/kgraph.cpp:1097-1117
// with Nhood::join :970-987): for node n, every pair of its new list A
// (i < j) and of A x old list B, each pair emitted to both endpoints'
// candidate buffers when within that endpoint's radius.  Here the distances
// come from Gram tiles: d(i, j) = (|x_i|^2 + |x_j|^2) - 2 <x_i, x_j>, with the
// dot products from tcgen05.mma on BF16 rows and FP32 accumulation in TMEM.
// Gram-exact mode (integer rows, squared norms below 2^23): every product and
// partial sum is an integer below 2^24, so the tile distance is the canonical
// FMA-chain distance bit for bit and the join emits exactly the candidates of
// the FP32 kernel.  Screen mode (rows not exact in BF16): the rows are
// rounded to BF16 and a pair is emitted when its Gram distance is below a
// bound on the rounding error; every emitted pair whose id is not already in
// the target's pool is recomputed in FP32 afterwards (rescore_kernel in
// kcna_nnd.cu; a repeat would be dropped by the merge anyway).
//
// A node's set (A then B) is ~20-60 rows and A ~10-30 columns, so one node
// per 128-row tile would leave most TMEM lanes idle.  Tiles are packed: the
// sets of consecutive nodes fill the 128 rows (M), their A lists fill up to
// 256 columns (N), and each row reads only its own node's columns - for a
// row of A with index j the columns i < j (each A pair once), for a row of B
// all of A.  A node with more than 128 rows spans several tiles, each with
// its full A list.
//
// Block layout: persistent, one block per SM, warp-specialised; the roles
// hand work to each other through mbarriers:
//   warp 0      packer: walks the block's range of nodes, copies row and
//               column ids into a tile stage (cp.async), marks each packed
//               node's found flag 0 (the merge credits it), then the radius and norm of every row and
//               column (cp.async); two stages;
//   warps 18-21 row loaders: the rows' and columns' BF16 rows by 16-byte
//               cp.async into the stage in the 128-byte swizzled K-major layout
//               the MMA descriptors read;
//   warp 1      MMA issuer (one thread): M = 128, N = columns rounded up to 16,
//               two accumulators of 256 TMEM columns;
//   warps 2-17  epilogue: warp w reads TMEM lane quarter w % 4 and every
//               fourth 16-column group of the span its rows cover; a count
//               pass (row and column emissions, column masks by ballots), one
//               atomicAdd per row and per column to reserve the runs in the
//               targets' candidate buffers, a write pass reading TMEM again
//               that stores every candidate's key and its joiner (the tile
//               row's node) for the merge's found credit.
// Every wait is bounded; a wait that gives up stops the block, sets the error
// word and lets in-flight copies and products finish before TMEM is released.
#include <algorithm>

#include "kcna_internal.h"
#include "kcna_join.cuh"
#include "kcna_tc.cuh"

using namespace kcna_tc;

namespace {

constexpr int EPI = 16;                        // epilogue warps: 4 lane quarters x 4 column phases
constexpr int LOAD_WARP = 2 + EPI;             // first row-loader warp
constexpr int NLOAD = 4;                       // row-loader warps
constexpr int JT_THREADS = (LOAD_WARP + NLOAD) * 32;
constexpr int PM = 128;                        // rows per tile (MMA M)
constexpr int PN = 256;                        // columns per tile (MMA N at most)
constexpr int NG = PN / 16;                    // 16-column groups
constexpr int GPW = NG / 4;                    // groups per epilogue warp at most
constexpr uint32_t KBB = 128;                  // bytes of a row inside one 64-element K block
constexpr uint32_t ROWS_R = PM * KBB * 2;      // 32 KiB
constexpr uint32_t ROWS_C = PN * KBB * 2;      // 64 KiB
constexpr uint32_t STAGE = ROWS_R + ROWS_C;    // 96 KiB
constexpr int TS = 2;                          // tile stages
constexpr int NACC = 2;                        // TMEM accumulators of PN columns

struct TileMeta {
    uint32_t rows, cols;
    uint32_t row_id[PM];
    uint32_t row_span[PM]; // the node's first column | end of the row's columns << 16
    uint32_t row_node[PM];
    float row_rad[PM], row_nrm[PM];
    uint32_t col_id[PN];
    float col_rad[PN], col_nrm[PN];
    // screening bound terms (screen mode): sqrt(radius (1 + 2^-15)) and the
    // norm of the rounded row
    float row_rr[PM], row_aa[PM], col_rr[PN], col_aa[PN];
};

struct JtShared {
    uint64_t ids_ready[TS], meta_full[TS], tile_full[TS], tile_empty[TS], acc_full[NACC], acc_empty[NACC];
    uint32_t tmem;
    volatile int abort_flag;
    TileMeta meta[TS];
};

// Screening bound of a rounded-row Gram distance (screen mode): with x~ the
// rows rounded to BF16 (relative error <= 2^-8 per element), a pair whose
// FP32 distance is <= radius has Gram distance
//   ds <= (sqrt(radius (1 + 2^-15)) + 2^-7 (|x~_i| + |x~_j|))^2 + 2^-14 (|x~_i|^2 + |x~_j|^2)
// (rounding of the rows, of the FP32 chain and of the FP32 accumulation, each
// bound doubled).  Pairs below the bound are emitted and recomputed in FP32.
constexpr float SCREEN_CE = 0.0078125f;       // 2^-7
constexpr float SCREEN_CG = 6.103515625e-05f; // 2^-14
__device__ __forceinline__ float screen_bound(float rr, float aa_sum, float nn_sum) {
    const float t = __fmaf_rn(SCREEN_CE, aa_sum, rr);
    return __fmaf_rn(t, t, SCREEN_CG * nn_sum);
}

// Commits this thread's outstanding cp.async copies as a group and waits for
// all of them (wait_group alone does not cover copies never committed).
__device__ __forceinline__ void cp_async_wait_0() {
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// The pair rule of one tile element: row (id_j, its radius / norm terms) and
// column i; rp: the column's id enters the row's buffer, cp: the row's id
// enters the column's buffer.
template <bool SCREEN>
__device__ __forceinline__ void pair_rule(const TileMeta &M, int i, float g, uint32_t id_j, float rad_j, float n_j,
                                          float rr_j, float aa_j, bool &rp, bool &cp, float &dd) {
    const float nn = __fadd_rn(n_j, M.col_nrm[i]);
    dd = __fsub_rn(nn, 2.f * g);
    if (SCREEN) {
        const float as = __fadd_rn(aa_j, M.col_aa[i]);
        rp = dd <= screen_bound(rr_j, as, nn);
        cp = dd <= screen_bound(M.col_rr[i], as, nn);
    } else {
        rp = dd <= rad_j;
        cp = dd <= M.col_rad[i];
    }
    if ((rp || cp) && M.col_id[i] == id_j) rp = cp = false; // an id in both lists
}

template <bool SCREEN>
__global__ void __launch_bounds__(JT_THREADS, 1) join_tc_kernel(JoinArgs a, const uint16_t *__restrict__ rowsb,
                                                                int ldh, const float *__restrict__ norms,
                                                                const float *__restrict__ rr,
                                                                const float *__restrict__ aa) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t tiles_s = (smem_u32(smem_raw) + 1023u) & ~1023u; // swizzled tiles need 1024-byte alignment
    unsigned char *tiles = smem_raw + (tiles_s - smem_u32(smem_raw));
    JtShared &S = *reinterpret_cast<JtShared *>(tiles + TS * STAGE);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nkb = (ldh + 63) >> 6;

    // K padding beyond ldh is never written by the loaders and must read as zero
    for (int i = tid; i < (int)(TS * STAGE / 16); i += JT_THREADS)
        reinterpret_cast<uint4 *>(tiles)[i] = make_uint4(0, 0, 0, 0);
    if (warp == 1) tmem_alloc(&S.tmem, NACC * PN);
    if (tid == 0) {
        for (int i = 0; i < TS; ++i) {
            mbar_init(&S.ids_ready[i], 1);        // packer lane 0 once the ids have landed
            mbar_init(&S.meta_full[i], 64);       // packer lanes: stores done, radius / norm copies landed
            mbar_init(&S.tile_full[i], NLOAD * 32); // every loader lane, after its copies and a proxy fence
            mbar_init(&S.tile_empty[i], 1 + EPI); // MMA commit + epilogue warps
        }
        for (int i = 0; i < NACC; ++i) {
            mbar_init(&S.acc_full[i], 1); // MMA commit
            mbar_init(&S.acc_empty[i], EPI);
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
    // this block's nodes
    const uint32_t per = (a.N + gridDim.x - 1) / gridDim.x;
    const uint32_t q0 = min(a.N, blockIdx.x * per), q1 = min(a.N, q0 + per);

    if (warp == 0) {
        // -------------------------------------------------------------- packer
        unsigned long long pairs = 0, rows_g = 0;
        uint32_t tcount = 0, rows = 0, cols = 0;
        int st = 0;
        TileMeta *M = &S.meta[0];
        auto open_tile = [&]() -> bool {
            st = (int)(tcount % TS);
            M = &S.meta[st];
            if (tcount >= (uint32_t)TS && !mbar_wait(&S.tile_empty[st], ((tcount / TS) - 1) & 1)) return false;
            rows = cols = 0;
            return true;
        };
        auto close_tile = [&]() {
            cp_async_wait_0(); // the ids have landed
            __syncwarp();
            if (lane == 0) {
                M->rows = rows;
                M->cols = cols;
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.ids_ready[st]);
            for (uint32_t i = lane; i < rows; i += 32) {
                const uint32_t u = M->row_id[i];
                cp_async4(smem_u32(&M->row_rad[i]), a.radius + u);
                cp_async4(smem_u32(&M->row_nrm[i]), norms + u);
                if (SCREEN) {
                    cp_async4(smem_u32(&M->row_rr[i]), rr + u);
                    cp_async4(smem_u32(&M->row_aa[i]), aa + u);
                }
            }
            for (uint32_t i = lane; i < cols; i += 32) {
                const uint32_t w = M->col_id[i];
                cp_async4(smem_u32(&M->col_rad[i]), a.radius + w);
                cp_async4(smem_u32(&M->col_nrm[i]), norms + w);
                if (SCREEN) {
                    cp_async4(smem_u32(&M->col_rr[i]), rr + w);
                    cp_async4(smem_u32(&M->col_aa[i]), aa + w);
                }
            }
            mbar_arrive_cp_async(&S.meta_full[st]); // when this lane's copies have landed
            mbar_arrive(&S.meta_full[st]);          // this lane's stores
            ++tcount;
        };
        ok = open_tile();
        for (uint32_t qb = q0; ok && qb < q1; qb += 32) {
            // the four list lengths of 32 nodes, one node per lane
            const uint32_t ql = qb + lane;
            uint32_t fn = 0, rn = 0, fo = 0, ro = 0;
            if (ql < q1) {
                fn = min(a.fwd_new_cnt[ql], a.fwd_new_cap);
                fo = min(a.fwd_old_cnt[ql], a.fwd_old_cap);
                if (a.iter > 0) { // the random subsets select_reverse_kernel left first
                    rn = min(a.rnew_cnt[ql], min(a.R, a.RB));
                    ro = min(a.rold_cnt[ql], min(a.R, a.RB));
                }
            }
            for (int jq = 0; jq < 32 && qb + jq < q1; ++jq) {
                const uint32_t q = qb + jq;
                const uint32_t nfn = __shfl_sync(KCNA_FULL, fn, jq), nrn = __shfl_sync(KCNA_FULL, rn, jq);
                const uint32_t nfo = __shfl_sync(KCNA_FULL, fo, jq), nro = __shfl_sync(KCNA_FULL, ro, jq);
                // A: forward new then reverse new, at most 128; B: forward old then reverse old
                const uint32_t na = min(nfn + nrn, (uint32_t)PM), nset = na + nfo + nro;
                if (na == 0) continue;
                pairs += (unsigned long long)na * (na - 1) / 2 + (unsigned long long)na * (nset - na);
                rows_g += nset;
                if (lane == 0) a.found[q] = 0; // set to 1 by the rows that emit
                const uint32_t *fnew = a.fwd_new + (uint64_t)q * a.fwd_new_cap;
                const uint32_t *fold = a.fwd_old + (uint64_t)q * a.fwd_old_cap;
                const uint32_t *rnw = a.rnew + (uint64_t)q * a.RB, *rod = a.rold + (uint64_t)q * a.RB;
                auto member = [&](uint32_t j) -> const uint32_t * {
                    if (j < na) return j < nfn ? fnew + j : rnw + (j - nfn);
                    j -= na;
                    return j < nfo ? fold + j : rod + (j - nfo);
                };
                for (uint32_t done = 0; done < nset;) {
                    if (rows == PM || cols + na > PN) {
                        close_tile();
                        if (!(ok = open_tile())) break;
                    }
                    const uint32_t take = min(nset - done, PM - rows);
                    for (uint32_t i = lane; i < na; i += 32) cp_async4(smem_u32(&M->col_id[cols + i]), member(i));
                    for (uint32_t i = lane; i < take; i += 32) {
                        const uint32_t j = done + i;
                        cp_async4(smem_u32(&M->row_id[rows + i]), member(j));
                        M->row_span[rows + i] = cols | ((cols + (j < na ? j : na)) << 16);
                        M->row_node[rows + i] = q;
                    }
                    rows += take;
                    cols += na;
                    done += take;
                }
                if (!ok) break;
            }
        }
        if (ok) {
            if (rows > 0) {
                close_tile();
                ok = open_tile();
            }
            if (ok) close_tile(); // a tile without rows ends the stream
        }
        cp_async_wait_0();
        if (!ok) S.abort_flag = 1;
        if (lane == 0) {
            atomicAdd(a.counters + 0, pairs);
            atomicAdd(a.counters + 5, rows_g);
        }
    } else if (warp >= LOAD_WARP) {
        // --------------------------------------------------------- row loaders
        const int lw = warp - LOAD_WARP;
        const int nseg = ldh >> 3; // 16-byte segments per row
        const int seg = lane & 15;
        for (uint32_t t = 0;; ++t) {
            const int st = (int)(t % TS);
            if (!mbar_wait(&S.ids_ready[st], (t / TS) & 1) || S.abort_flag) { ok = false; break; }
            const TileMeta &M = S.meta[st];
            const int rows = (int)M.rows, cols = (int)M.cols;
            const uint32_t base = tiles_s + (uint32_t)st * STAGE;
            if (seg < nseg) {
                // rows: 32 per loader warp, two per instruction
                for (int k = 0; k < 16; ++k) {
                    const int r = 32 * lw + 2 * k + (lane >> 4);
                    if (r < rows)
                        cp_async16(base + (uint32_t)(seg >> 3) * PM * KBB + sw128_off((uint32_t)r, (uint32_t)(seg & 7)),
                                   rowsb + (uint64_t)M.row_id[r] * ldh + seg * 8);
                }
                // columns: 64 per loader warp
                for (int k = 0; k < 32; ++k) {
                    const int c = 64 * lw + 2 * k + (lane >> 4);
                    if (c < cols)
                        cp_async16(base + ROWS_R + (uint32_t)(seg >> 3) * PN * KBB +
                                       sw128_off((uint32_t)c, (uint32_t)(seg & 7)),
                                   rowsb + (uint64_t)M.col_id[c] * ldh + seg * 8);
                }
            }
            cp_async_wait_0();
            fence_proxy_async(); // the copies, for the tensor cores' reads
            mbar_arrive(&S.tile_full[st]);
            if (rows == 0) break;
        }
        cp_async_wait_0();
        if (!ok) S.abort_flag = 1;
    } else if (warp == 1) {
        // ---------------------------------------------------------- MMA issuer
        if (lane == 0) {
            for (uint32_t t = 0;; ++t) {
                const int st = (int)(t % TS), b = (int)(t % NACC);
                if (!mbar_wait(&S.tile_full[st], (t / TS) & 1) || S.abort_flag) { ok = false; break; }
                const uint32_t rows = S.meta[st].rows, cols = S.meta[st].cols;
                if (rows == 0) break;
                if (t >= (uint32_t)NACC && !mbar_wait(&S.acc_empty[b], ((t / NACC) - 1) & 1)) { ok = false; break; }
                fence_after();
                const uint32_t base = tiles_s + st * STAGE;
                const uint32_t idesc = idesc_bf16(PM, (int)((cols + 15) & ~15u));
                const uint32_t d = tmem + (uint32_t)(b * PN);
                for (int kb = 0; kb < nkb; ++kb)
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk)
                        mma_bf16(d, desc_sw128(base + kb * PM * KBB + kk * 32),
                                 desc_sw128(base + ROWS_R + kb * PN * KBB + kk * 32), idesc, (kb | kk) ? 1u : 0u);
                mma_commit(&S.acc_full[b]);
                mma_commit(&S.tile_empty[st]);
            }
            if (!ok) S.abort_flag = 1;
        }
        __syncwarp();
    } else {
        // ------------------------------------------------------------ epilogue
        const int q = warp & 3, h = (warp - 2) >> 2; // TMEM lane quarter, column phase
        const int r = 32 * q + lane;                 // this thread's row of a tile
        const uint32_t flags = (uint32_t)(KCNA_FLAG_NEW | KCNA_FLAG_ISNEW);
        unsigned long long emitted = 0;
        for (uint32_t t = 0;; ++t) {
            const int st = (int)(t % TS), b = (int)(t % NACC);
            bool mine = mbar_wait(&S.meta_full[st], (t / TS) & 1) && !S.abort_flag;
            if (!__all_sync(KCNA_FULL, mine)) { ok = false; break; }
            const TileMeta &M = S.meta[st];
            const uint32_t rows = M.rows;
            if (rows == 0) break;
            mine = mbar_wait(&S.acc_full[b], (t / NACC) & 1);
            if (!__all_sync(KCNA_FULL, mine)) { ok = false; break; }
            fence_after();
            const bool rowv = (uint32_t)r < rows;
            const uint32_t id_j = rowv ? M.row_id[r] : 0u;
            const uint32_t span = rowv ? M.row_span[r] : 0u;
            const int cs = (int)(span & 0xFFFFu), ce = (int)(span >> 16);
            const float rad_j = rowv ? M.row_rad[r] : 0.f, n_j = rowv ? M.row_nrm[r] : 0.f;
            const float rr_j = SCREEN && rowv ? M.row_rr[r] : 0.f, aa_j = SCREEN && rowv ? M.row_aa[r] : 0.f;
            // the 16-column groups this warp's rows touch
            int gl = ce > cs ? cs >> 4 : 1 << 20, gh = ce > cs ? (ce - 1) >> 4 : -1;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                gl = min(gl, __shfl_xor_sync(KCNA_FULL, gl, o));
                gh = max(gh, __shfl_xor_sync(KCNA_FULL, gh, o));
            }
            const uint32_t trow = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * PN);
            // count pass: the row's emissions as bits, the columns' as ballots
            uint64_t rmask = 0;
            uint32_t cm[GPW] = {0u, 0u, 0u, 0u}; // lane x: rows emitting into column 16 g_k + x
#pragma unroll
            for (int k = 0; k < GPW; ++k) {
                const int g = gl + h + 4 * k;
                if (g > gh) break;
                uint32_t raw[16];
                tmem_ld16_async(trow + 16 * g, raw);
                tmem_wait_ld16(raw);
#pragma unroll
                for (int x = 0; x < 16; ++x) {
                    const int i = 16 * g + x;
                    bool rp = false, cp = false;
                    if (i >= cs && i < ce) {
                        float dd;
                        pair_rule<SCREEN>(M, i, __uint_as_float(raw[x]), id_j, rad_j, n_j, rr_j, aa_j, rp, cp, dd);
                    }
                    rmask |= (uint64_t)rp << (16 * k + x);
                    const unsigned m = __ballot_sync(KCNA_FULL, cp);
                    if (lane == x) cm[k] = m;
                }
            }
            // reservations, without barriers between warps: the row's run for
            // this warp's columns, lane x the run of column 16 g_k + x for this
            // lane quarter
            const int nr = __popcll(rmask);
            uint32_t p = nr ? atomicAdd(a.cand_cnt + id_j, (uint32_t)nr) : 0u;
            uint32_t cb[GPW] = {0u, 0u, 0u, 0u};
            int nct = 0;
#pragma unroll
            for (int k = 0; k < GPW; ++k) {
                const int g = gl + h + 4 * k;
                if (g > gh) break;
                if (lane < 16 && cm[k]) {
                    cb[k] = atomicAdd(a.cand_cnt + M.col_id[16 * g + lane], (uint32_t)__popc(cm[k]));
                    nct += __popc(cm[k]);
                }
            }
            emitted += (unsigned long long)(nr + nct);
            if (__any_sync(KCNA_FULL, nr > 0 || nct > 0)) { // write pass; the distances are read again from TMEM
                const uint64_t s0 = (uint64_t)id_j * a.CB;
                const uint32_t joiner = rowv ? M.row_node[r] : 0u; // the node whose join made this tile row
#pragma unroll
                for (int k = 0; k < GPW; ++k) {
                    const int g = gl + h + 4 * k;
                    if (g > gh) break;
                    const uint32_t gm = (uint32_t)(rmask >> (16 * k)) & 0xFFFFu;
                    if (!__any_sync(KCNA_FULL, gm != 0u || (lane < 16 && cm[k] != 0u))) continue;
                    uint32_t raw[16];
                    tmem_ld16_async(trow + 16 * g, raw);
                    tmem_wait_ld16(raw);
#pragma unroll
                    for (int x = 0; x < 16; ++x) {
                        const int i = 16 * g + x;
                        const unsigned m = __shfl_sync(KCNA_FULL, cm[k], x);
                        const uint32_t cbx = __shfl_sync(KCNA_FULL, cb[k], x);
                        if (((gm >> x) & 1u) || ((m >> lane) & 1u)) {
                            // emitted with the Gram distance (exact in Gram-exact mode;
                            // recomputed in FP32 by the rescore in screen mode)
                            const float dd = fmaxf(
                                __fsub_rn(__fadd_rn(n_j, M.col_nrm[i]), 2.f * __uint_as_float(raw[x])), 0.f);
                            if ((gm >> x) & 1u) {
                                if (p < a.CB) kcna_cand_put(a.cand, s0 + p, kcna_key(dd, M.col_id[i], flags), joiner);
                                ++p;
                            }
                            if ((m >> lane) & 1u) {
                                const uint32_t pc = cbx + __popc(m & kcna_lanemask_lt());
                                if (pc < a.CB)
                                    kcna_cand_put(a.cand, (uint64_t)M.col_id[i] * a.CB + pc, kcna_key(dd, id_j, flags),
                                                  joiner);
                            }
                        }
                    }
                }
            }
            // accumulator and stage released by each epilogue warp
            fence_before();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&S.acc_empty[b]);
                mbar_arrive(&S.tile_empty[st]);
            }
        }
        if (!ok) S.abort_flag = 1;
        emitted = kcna_warp_sum(emitted);
        if (lane == 0 && emitted) atomicAdd(a.counters + 6, emitted);
    }
    fence_before();
    __syncthreads();
    if (warp == 1) tmem_free(tmem, NACC * PN);
    if (!ok) kcna_set_err(a.err, KCNA_DERR_SPIN);
}

constexpr size_t join_tc_smem() { return 1024 + (size_t)TS * STAGE + sizeof(JtShared); }

} // namespace

bool kcna_join_tc_fits(const JoinArgs &a) {
    (void)a;
    return join_tc_smem() <= 227 * 1024;
}

// sqrt(radius (1 + 2^-15)) and sqrt(norm) for the screening bound
__global__ void screen_terms_kernel(const float *__restrict__ radius, const float *__restrict__ norms, uint32_t n,
                                    float *__restrict__ rr, float *__restrict__ aa) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    rr[i] = __fsqrt_ru(__fmul_ru(radius[i], 1.000030517578125f));
    aa[i] = __fsqrt_ru(norms[i]);
}

kcna_status kcna_join_tc_launch(kcna_ctx *c, const JoinArgs &a) {
    if (!(c->gram_exact || c->bf16_screen) || !c->Xh || !c->norms || (c->ld & 7u) || c->ld > 128)
        return kcna_fail(c, KCNA_E_STATE, "Gram-tile join needs BF16 rows with d <= 128");
    if (!kcna_join_tc_fits(a)) return kcna_fail(c, KCNA_E_STATE, "Gram-tile join: shared memory");
    const size_t sm = join_tc_smem();
    KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(join_tc_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)sm),
                             "join_tc smem attr"));
    KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(join_tc_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)sm),
                             "join_tc smem attr"));
    const uint32_t grid = (uint32_t)std::min<uint64_t>(a.N, (uint64_t)std::max(c->num_sms, 1));
    if (grid == 0) return KCNA_OK;
    if (c->bf16_screen) {
        float *rr = nullptr, *aa = nullptr;
        KCNA_TRY(kcna_scratch(c, (size_t)c->n * 8, reinterpret_cast<void **>(&rr)));
        aa = rr + c->n;
        screen_terms_kernel<<<kcna_div_up(c->n, 256), 256, 0, c->stream>>>(a.radius, c->norms, c->n, rr, aa);
        KCNA_LAUNCHED(c);
        join_tc_kernel<true><<<grid, JT_THREADS, sm, c->stream>>>(a, c->Xh, (int)c->ld, c->norms, rr, aa);
    } else {
        join_tc_kernel<false><<<grid, JT_THREADS, sm, c->stream>>>(a, c->Xh, (int)c->ld, c->norms, nullptr, nullptr);
    }
    KCNA_LAUNCHED(c);
    return kcna_cuda_check(c, cudaGetLastError(), "join_tc_kernel");
}
