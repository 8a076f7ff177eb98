// kcna_p2k_tc.cu - P2K (BridgeView) join on tcgen05 Gram tiles.
//
// Same work as p2k_join_kernel (kcna_graph.cu; reference BridgeView_join,
// src/kgraph.cpp:2634-2648): for every node q, every pusher u of q (the
// entries of rnn(q), with u's isnew flag) meets every graph neighbour w of q;
// the pair is skipped when u == w or both are old, counted otherwise, and w
// becomes a candidate of u when d(u, w) <= radius(u).  Distances come from
// Gram tiles, (|u|^2 + |w|^2) - 2 <u, w> with tcgen05.mma on BF16 rows and
// FP32 accumulation in TMEM; the kernel runs only in Gram-exact mode (integer
// rows, squared norms below 2^23), where that is the canonical FMA-chain
// distance bit for bit.
//
// A node has ~10 pushers and ~26 neighbours, so one node alone would fill a
// 128-row tile by a tenth.  Tiles are packed instead: the pushers of several
// consecutive nodes fill the 128 rows (M), their neighbour lists fill up to 256
// columns (N), and each row only reads the column range of its own node.  A
// node with more than 128 pushers spans several tiles, each with its full
// neighbour list.
//
// Block layout: persistent, one block per SM, warp-specialised like the local
// join (kcna_join_tc.cu):
//   warp 0      producer: walks the block's range of nodes, packs tiles, copies
//               pusher / neighbour ids into the tile stage with cp.async, then
//               radius, norm and isnew flags; a tile with no rows ends the
//               stream.
//   warps 18-21 row loaders: the pushers' and neighbours' BF16 rows by 16-byte
//               cp.async in the 128-byte swizzled K-major layout.
//   warp 1      MMA issuer: M = 128, N = columns used rounded up to 16.
//   warps 2-17  epilogue: warp w reads TMEM lanes 32*(w%4).. (pushers) and
//               every fourth 16-column group of the span its lanes' nodes
//               cover; per thread a count pass, one atomicAdd on the pusher's
//               candidate count, and a write pass reading TMEM again.
#include <algorithm>

#include "kcna_internal.h"
#include "kcna_tc.cuh"

using namespace kcna_tc;

namespace {

constexpr int EPI = 16;       // epilogue warps: 4 lane quarters x 4 column phases
constexpr int LOAD_WARP = 2 + EPI; // first row-loader warp
constexpr int NLOAD = 4;      // row-loader warps
constexpr int PW_WARPS = LOAD_WARP + NLOAD;
constexpr int PW_THREADS = PW_WARPS * 32;
constexpr int PM = 128;                      // pusher rows per tile (MMA M)
constexpr int PN = 256;                      // neighbour columns per tile (MMA N at most)
constexpr uint32_t KBB = 128;                // bytes of a row inside one 64-element K block
constexpr uint32_t ROWS_A = PM * KBB * 2;    // 32 KiB
constexpr uint32_t ROWS_B = PN * KBB * 2;    // 64 KiB
constexpr uint32_t STAGE = ROWS_A + ROWS_B;  // 96 KiB
constexpr int TS = 2;                        // tile stages
constexpr int NACC = 2;                      // TMEM accumulators of PN columns

struct StageMeta {
    uint32_t rows, cols;
    uint32_t row_id[PM];   // pusher id | isnew << 31
    uint32_t row_span[PM]; // column range of the row's node: begin | end << 16
    float row_rad[PM], row_nrm[PM];
    uint16_t row_nn[PM];   // new neighbours of the row's node: an old pusher's row spans only them
    uint32_t col_id[PN];
    uint32_t col_gidx[PN]; // q * W + j: where the column's isnew flag lives
    float col_nrm[PN];
    uint8_t col_new[PN];
};

struct PwShared {
    uint64_t ids_ready[TS], meta_full[TS], tile_full[TS], tile_empty[TS], acc_full[NACC], acc_empty[NACC];
    uint32_t tmem;
    volatile int abort_flag;
    StageMeta meta[TS];
};

struct P2kArgs {
    uint32_t N, W;
    const uint64_t *off;
    const uint32_t *rnn;
    const uint32_t *g_ids, *g_deg;
    const uint8_t *g_isnew;
    const float *radius, *norms;
    const uint16_t *Xh;
    int ldh;
    uint64_t *cand;
    uint32_t *cand_cnt;
    uint32_t CB;
    const uint16_t *nnew; // per node: graph neighbours flagged new
    const uint8_t *pnew;  // per node: 1 when one of its pushers this round is new
    unsigned long long *comps;
    int *err;
};

__global__ void __launch_bounds__(PW_THREADS, 1) p2k_tc_kernel(P2kArgs a) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t tiles_s = (smem_u32(smem_raw) + 1023u) & ~1023u;
    unsigned char *tiles = smem_raw + (tiles_s - smem_u32(smem_raw));
    PwShared &S = *reinterpret_cast<PwShared *>(tiles + TS * STAGE);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nkb = (a.ldh + 63) >> 6;

    for (int i = tid; i < (int)(TS * STAGE / 16); i += PW_THREADS)
        reinterpret_cast<uint4 *>(tiles)[i] = make_uint4(0, 0, 0, 0);
    if (warp == 1) tmem_alloc(&S.tmem, NACC * PN);
    if (tid == 0) {
        for (int i = 0; i < TS; ++i) {
            mbar_init(&S.ids_ready[i], 1);          // producer lane 0 once the ids have landed
            mbar_init(&S.meta_full[i], 64);         // producer lanes: stores done, radius / norm copies landed
            mbar_init(&S.tile_full[i], NLOAD * 32); // every loader lane, after its copies and a proxy fence
            mbar_init(&S.tile_empty[i], 1 + EPI); // MMA commit + epilogue warps
        }
        for (int i = 0; i < NACC; ++i) {
            mbar_init(&S.acc_full[i], 1);
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
        // ------------------------------------------------------------ producer
        uint32_t tcount = 0, rows = 0, cols = 0;
        int st = 0;
        StageMeta *M = &S.meta[0];
        auto open_tile = [&]() -> bool {
            st = (int)(tcount % TS);
            M = &S.meta[st];
            if (tcount >= (uint32_t)TS && !mbar_wait(&S.tile_empty[st], ((tcount / TS) - 1) & 1)) return false;
            rows = cols = 0;
            return true;
        };
        auto close_tile = [&]() {
            // ids landed: announce them to the loaders, then radius, norms and flags
            asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
            __syncwarp();
            if (lane == 0) {
                M->rows = rows;
                M->cols = cols;
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.ids_ready[st]);
            for (uint32_t i = lane; i < rows; i += 32) {
                const uint32_t u = M->row_id[i] & 0x7FFFFFFFu;
                cp_async4(smem_u32(&M->row_rad[i]), a.radius + u);
                cp_async4(smem_u32(&M->row_nrm[i]), a.norms + u);
            }
            for (uint32_t i = lane; i < cols; i += 32) cp_async4(smem_u32(&M->col_nrm[i]), a.norms + M->col_id[i]);
            uint8_t fl[PN / 32]; // isnew flags: all loads first, one round trip
#pragma unroll
            for (int k2 = 0; k2 < PN / 32; ++k2) {
                const uint32_t i = lane + 32 * k2;
                fl[k2] = i < cols ? a.g_isnew[M->col_gidx[i]] : (uint8_t)0;
            }
#pragma unroll
            for (int k2 = 0; k2 < PN / 32; ++k2)
                if (lane + 32 * k2 < cols) M->col_new[lane + 32 * k2] = fl[k2];
            mbar_arrive_cp_async(&S.meta_full[st]); // when this lane's copies have landed
            mbar_arrive(&S.meta_full[st]);          // this lane's stores
            ++tcount;
        };
        ok = open_tile();
        for (uint32_t qb = q0; ok && qb < q1; qb += 32) {
            const uint32_t ql = qb + lane;
            uint64_t o0 = 0, o1 = 0;
            uint32_t dl = 0, nl = 0, al = 0;
            if (ql < q1) {
                o0 = a.off[ql];
                o1 = a.off[ql + 1];
                dl = min(a.g_deg[ql], a.W);
                nl = a.nnew[ql];
                al = a.pnew[ql];
            }
            for (int jq = 0; jq < 32 && qb + jq < q1; ++jq) {
                const uint32_t q = qb + jq;
                const uint64_t ob = __shfl_sync(KCNA_FULL, o0, jq), oe = __shfl_sync(KCNA_FULL, o1, jq);
                const uint32_t deg = __shfl_sync(KCNA_FULL, dl, jq);
                const uint32_t nn = min(__shfl_sync(KCNA_FULL, nl, jq), deg);
                const bool an = __shfl_sync(KCNA_FULL, al, jq) != 0u;
                const uint32_t nu = (uint32_t)(oe - ob);
                if (nu == 0 || deg == 0) continue;
                // a pair of an old pusher and an old neighbour is skipped
                // (src/kgraph.cpp:2639-2641): a node whose pushers and neighbours
                // are all old has nothing to join; otherwise its new neighbours
                // come first among its columns, an old pusher's row spans only
                // them, and without new pushers only they are packed
                if (!an && nn == 0) continue;
                const uint32_t cl = an ? deg : nn; // columns the node needs
                const bool reorder = nn > 0 && nn < deg;
                for (uint32_t done = 0; done < nu;) {
                    if (rows == PM || cols + cl > PN) {
                        close_tile();
                        if (!(ok = open_tile())) break;
                    }
                    const uint32_t take = min(nu - done, PM - rows);
                    const uint32_t span = cols | ((cols + cl) << 16);
                    for (uint32_t i = lane; i < take; i += 32) {
                        cp_async4(smem_u32(&M->row_id[rows + i]), a.rnn + ob + done + i);
                        M->row_span[rows + i] = span;
                        M->row_nn[rows + i] = (uint16_t)nn;
                    }
                    if (!reorder) { // all new, all old (new pushers only), or no reordering to do
                        for (uint32_t j = lane; j < deg; j += 32) {
                            cp_async4(smem_u32(&M->col_id[cols + j]), a.g_ids + (uint64_t)q * a.W + j);
                            M->col_gidx[cols + j] = q * a.W + j;
                        }
                    } else {
                        const uint8_t *fq = a.g_isnew + (uint64_t)q * a.W;
                        uint32_t an_ = 0, ao = 0;
                        for (uint32_t j0 = 0; j0 < deg; j0 += 32) {
                            const uint32_t j = j0 + lane;
                            const bool f = j < deg && fq[j];
                            const unsigned mn = __ballot_sync(KCNA_FULL, f);
                            const unsigned mo = __ballot_sync(KCNA_FULL, j < deg && !f);
                            if (j < deg && (f || an)) {
                                const uint32_t c = cols + (f ? an_ + __popc(mn & kcna_lanemask_lt())
                                                             : nn + ao + __popc(mo & kcna_lanemask_lt()));
                                cp_async4(smem_u32(&M->col_id[c]), a.g_ids + (uint64_t)q * a.W + j);
                                M->col_gidx[c] = q * a.W + j;
                            }
                            an_ += __popc(mn);
                            ao += __popc(mo);
                        }
                    }
                    rows += take;
                    cols += cl;
                    done += take;
                }
            }
        }
        if (ok) {
            if (rows > 0) {
                close_tile();
                ok = open_tile();
            }
            if (ok) close_tile(); // a tile without rows ends the stream
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        if (!ok) S.abort_flag = 1;
    } else if (warp >= LOAD_WARP) {
        // --------------------------------------------------------- row loaders
        // pushers' and neighbours' BF16 rows by 16-byte cp.async into the
        // stage's 128-byte swizzled K-major regions
        const int lw = warp - LOAD_WARP;
        const int nseg = a.ldh >> 3, seg = lane & 15;
        for (uint32_t t = 0;; ++t) {
            const int st = (int)(t % TS);
            if (!mbar_wait(&S.ids_ready[st], (t / TS) & 1) || S.abort_flag) { ok = false; break; }
            const StageMeta &M = S.meta[st];
            const int rows = (int)M.rows, cols = (int)M.cols;
            const uint32_t base = tiles_s + (uint32_t)st * STAGE;
            if (seg < nseg) {
                for (int k = 0; k < PM / (2 * NLOAD); ++k) {
                    const int r = PM / NLOAD * lw + 2 * k + (lane >> 4);
                    if (r < rows)
                        cp_async16(base + (uint32_t)(seg >> 3) * PM * KBB + sw128_off((uint32_t)r, (uint32_t)(seg & 7)),
                                   a.Xh + (uint64_t)(M.row_id[r] & 0x7FFFFFFFu) * a.ldh + seg * 8);
                }
                for (int k = 0; k < PN / (2 * NLOAD); ++k) {
                    const int cc = PN / NLOAD * lw + 2 * k + (lane >> 4);
                    if (cc < cols)
                        cp_async16(base + ROWS_A + (uint32_t)(seg >> 3) * PN * KBB +
                                       sw128_off((uint32_t)cc, (uint32_t)(seg & 7)),
                                   a.Xh + (uint64_t)M.col_id[cc] * a.ldh + seg * 8);
                }
            }
            asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
            fence_proxy_async(); // the copies, for the tensor cores' reads
            mbar_arrive(&S.tile_full[st]);
            if (rows == 0) break;
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        if (!ok) S.abort_flag = 1;
    } else if (warp == 1) {
        // ---------------------------------------------------------- MMA issuer
        if (lane == 0) {
            for (uint32_t t = 0;; ++t) {
                const int st = (int)(t % TS), b = (int)(t % NACC);
                if (!mbar_wait(&S.tile_full[st], (t / TS) & 1) || S.abort_flag) { ok = false; break; }
                const uint32_t cols = S.meta[st].cols;
                if (S.meta[st].rows == 0) break;
                if (t >= (uint32_t)NACC && !mbar_wait(&S.acc_empty[b], ((t / NACC) - 1) & 1)) { ok = false; break; }
                fence_after();
                const uint32_t base = tiles_s + st * STAGE;
                const uint32_t idesc = idesc_bf16(PM, (int)((cols + 15) & ~15u));
                const uint32_t d = tmem + (uint32_t)(b * PN);
                for (int kb = 0; kb < nkb; ++kb)
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk)
                        mma_bf16(d, desc_sw128(base + kb * PM * KBB + kk * 32),
                                 desc_sw128(base + ROWS_A + kb * PN * KBB + kk * 32), idesc, (kb | kk) ? 1u : 0u);
                mma_commit(&S.acc_full[b]);
                mma_commit(&S.tile_empty[st]);
            }
            if (!ok) S.abort_flag = 1;
        }
        __syncwarp();
    } else {
        // ------------------------------------------------------------ epilogue
        const int q = warp & 3, h = (warp - 2) >> 2;
        const int rr = 32 * q + lane;
        unsigned long long cc = 0;
        for (uint32_t t = 0;; ++t) {
            const int st = (int)(t % TS), b = (int)(t % NACC);
            bool mine = mbar_wait(&S.meta_full[st], (t / TS) & 1) && !S.abort_flag;
            if (!__all_sync(KCNA_FULL, mine)) { ok = false; break; }
            const StageMeta &M = S.meta[st];
            const uint32_t rows = M.rows;
            if (rows == 0) break;
            mine = mbar_wait(&S.acc_full[b], (t / NACC) & 1);
            if (!__all_sync(KCNA_FULL, mine)) { ok = false; break; }
            fence_after();
            const bool rowv = (uint32_t)rr < rows;
            const uint32_t uw = rowv ? M.row_id[rr] : 0u;
            const uint32_t u = uw & 0x7FFFFFFFu;
            const bool unew = (uw >> 31) != 0u;
            const uint32_t span = rowv ? M.row_span[rr] : 0u;
            const int cs = (int)(span & 0xFFFFu);
            // an old pusher meets only its node's new neighbours (the first ones)
            const int ce = unew ? (int)(span >> 16) : min((int)(span >> 16), cs + (rowv ? (int)M.row_nn[rr] : 0));
            const float rad = rowv ? M.row_rad[rr] : -1.f, nu2 = rowv ? M.row_nrm[rr] : 0.f;
            // 16-column groups this warp's rows touch
            const bool rowe = rowv && ce > cs;
            int gl = rowe ? cs >> 4 : 1 << 20, gh = rowe ? (ce - 1) >> 4 : -1;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                gl = min(gl, __shfl_xor_sync(KCNA_FULL, gl, o));
                gh = max(gh, __shfl_xor_sync(KCNA_FULL, gh, o));
            }
            const uint32_t trow = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * PN);
            uint32_t cnt = 0;
            for (int g = gl + h; g <= gh; g += 4) { // count pass
                uint32_t raw[16];
                tmem_ld16_async(trow + 16 * g, raw);
                tmem_wait_ld16(raw);
#pragma unroll
                for (int x = 0; x < 16; ++x) {
                    const int col = 16 * g + x;
                    if (col >= cs && col < ce) {
                        const uint32_t w = M.col_id[col];
                        if (w != u && (unew || M.col_new[col])) {
                            ++cc;
                            const float dd = __fsub_rn(__fadd_rn(nu2, M.col_nrm[col]), 2.f * __uint_as_float(raw[x]));
                            cnt += dd <= rad ? 1u : 0u;
                        }
                    }
                }
            }
            uint32_t p = cnt ? atomicAdd(a.cand_cnt + u, cnt) : 0u;
            if (__any_sync(KCNA_FULL, cnt != 0u)) { // write pass
                const uint64_t s0 = (uint64_t)u * a.CB; // whole slots, joiner 0 (no credit)
                for (int g = gl + h; g <= gh; g += 4) {
                    uint32_t raw[16];
                    tmem_ld16_async(trow + 16 * g, raw);
                    tmem_wait_ld16(raw);
                    if (!cnt) continue;
#pragma unroll
                    for (int x = 0; x < 16; ++x) {
                        const int col = 16 * g + x;
                        if (col >= cs && col < ce) {
                            const uint32_t w = M.col_id[col];
                            if (w != u && (unew || M.col_new[col])) {
                                const float dd =
                                    __fsub_rn(__fadd_rn(nu2, M.col_nrm[col]), 2.f * __uint_as_float(raw[x]));
                                if (dd <= rad) {
                                    if (p < a.CB)
                                        kcna_cand_put(a.cand, s0 + p,
                                                      kcna_key(dd, w, (uint32_t)(KCNA_FLAG_NEW | KCNA_FLAG_ISNEW)), 0u);
                                    ++p;
                                }
                            }
                        }
                    }
                }
            }
            fence_before();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&S.acc_empty[b]);
                mbar_arrive(&S.tile_empty[st]);
            }
        }
        cc = kcna_warp_sum(cc);
        if (lane == 0 && cc) atomicAdd(a.comps, cc);
        if (!ok) S.abort_flag = 1;
    }
    fence_before();
    __syncthreads();
    if (warp == 1) tmem_free(tmem, NACC * PN);
    if (!ok) kcna_set_err(a.err, KCNA_DERR_SPIN);
}

} // namespace

kcna_status kcna_p2k_tc_launch(kcna_ctx *c, const uint64_t *off, const uint32_t *rnn, const uint16_t *nnew,
                               const uint8_t *pnew, unsigned long long *comps) {
    if (!c->gram_exact || !c->Xh || !c->norms || (c->ld & 7u) || c->ld > 128 || c->W > (uint32_t)PN)
        return kcna_fail(c, KCNA_E_STATE, "Gram-tile P2K needs exact BF16 rows with d <= 128 and width <= 256");
    P2kArgs a;
    a.N = c->n;
    a.W = c->W;
    a.off = off;
    a.rnn = rnn;
    a.g_ids = c->g_ids;
    a.g_deg = c->g_deg;
    a.g_isnew = c->g_isnew;
    a.radius = c->radius;
    a.norms = c->norms;
    a.Xh = c->Xh;
    a.ldh = (int)c->ld;
    a.cand = c->cand;
    a.cand_cnt = c->cand_cnt;
    a.CB = c->CB;
    a.nnew = nnew;
    a.pnew = pnew;
    a.comps = comps;
    a.err = c->d_err;
    const size_t sm = 1024 + (size_t)TS * STAGE + sizeof(PwShared);
    KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(p2k_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm),
                             "p2k_tc smem attr"));
    const uint32_t grid = (uint32_t)std::max(c->num_sms, 1);
    p2k_tc_kernel<<<grid, PW_THREADS, sm, c->stream>>>(a);
    KCNA_LAUNCHED(c);
    return kcna_cuda_check(c, cudaGetLastError(), "p2k_tc_kernel");
}
