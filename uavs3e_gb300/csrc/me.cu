// Batched motion search of every block of a frame (8x8 .. 64x64 including 2:1 shapes on the
// 64x64 CTU grid), bit-exact with the per-candidate costs of uavs3e's motion search:
//   integer stage: cost = (SAD << 16) + (mvbits(4dx) + mvbits(4dy)) * lambda_mv over the full
//     clipped window, strict '<' in raster order (cost_sad + GET_MVBITS_IPEL_*,
//     src/me.c:103-197 and src/com_cost.c:40-115; window limits as get_max_search_range,
//     src/me.c:502-527, with is_padding = 1 and mvp = 0);
//   fractional stage: me_sub_pel_search with SATD cost (src/me.c:366-500): centre, 8
//     half-sample and 8 quarter-sample neighbours, com_had on the interpolated planes.
//
// Integer stage layout: one CTA per (CTU, reference).  Its search window is staged once into
// shared memory.  A half-warp covers the CTU as a 4x4 grid of 16x16 sub-blocks (one lane
// each, org samples in registers) and sweeps NDY vertically adjacent candidates at one dx,
// so every byte-aligned reference word is reused by up to NDY rows of the block.  The four
// 8x8 tile SADs of a lane give the 8x8/16x8/8x16/16x16 blocks; warp shuffles give the
// 32x16 .. 64x64 ones.  Each block keeps a 32-bit running minimum of
//     ((SAD + q) << 11) | rank,   q = mvcost >> 16,
// where rank orders this lane group's candidates by (mvcost & 0xffff, raster index): the
// minimum is then exactly the (cost, raster) minimum, so a block update is one LEA + one
// IMNMX.  Per-group winners are merged into a 64-bit (cost << 15 | raster) key.
#include "common.cuh"
#include "uavs3e_cuda_internal.h"
#include <algorithm>
#include <vector>

namespace uc {

void ctu_block_table(CtuBlock o[ME_BLOCKS_PER_CTU])
{
    static const int shapes[10][2] = { { 8, 8 }, { 16, 8 }, { 8, 16 }, { 16, 16 }, { 32, 16 },
                                       { 16, 32 }, { 32, 32 }, { 64, 32 }, { 32, 64 }, { 64, 64 } };
    int n = 0;
    for (int s = 0; s < 10; s++) {
        int w = shapes[s][0], h = shapes[s][1];
        for (int y = 0; y < ME_CTU; y += h)
            for (int x = 0; x < ME_CTU; x += w) o[n++] = CtuBlock{ (u8)x, (u8)y, (u8)w, (u8)h };
    }
}

// MV bits of a quarter-sample component (inter_search_create, src/inter.c:2029-2057):
// 1 for 0, else 2 * (floor(log2(|v| + 1)) + 1)
__host__ __device__ __forceinline__ u32 mvbits(int v)
{
    if (v == 0) return 1;
    u32 a = (u32)(v < 0 ? -v : v) + 1;
#ifdef __CUDA_ARCH__
    return 2u * (32u - __clz(a));
#else
    u32 r = 0;
    while (a) { r++; a >>= 1; }
    return 2u * r;
#endif
}

u32 me_mvbits(int v) { return mvbits(v); }

size_t me_q2_entries(int range, int ndy_per_item)
{
    int nd = 2 * range + 1;
    int nchunk = (nd + ndy_per_item - 1) / ndy_per_item;
    return (size_t)nd * nchunk * ndy_per_item;
}

size_t me_sub_scratch_bytes(int W, int H, int n_refs)
{
    size_t nctu = (size_t)((W + 63) / 64) * ((H + 63) / 64);
    return nctu * n_refs * ME_BLOCKS_PER_CTU * 17 * sizeof(u32);
}

size_t me_key_scratch_bytes(int W, int H, int n_refs)
{
    size_t nctu = (size_t)((W + 63) / 64) * ((H + 63) / 64);
    return nctu * n_refs * ME_BLOCKS_PER_CTU * sizeof(u64);
}

int me_build_tables(int W, int H, int range, u32 lambda_mv, int ndy, MeTables *t, u32 *q2tab, u16 *rank2mv,
                    size_t q2cap)
{
    int M = std::max(W, H);
    t->lo_x = t->lo_y = std::max(-range, -M + 4);
    t->hi_x = t->hi_y = std::min(range, M - 4);
    t->ndx = t->hi_x - t->lo_x + 1;
    t->ndy = t->hi_y - t->lo_y + 1;
    t->ndy_per_item = ndy;
    t->nchunk = (t->ndy + ndy - 1) / ndy;
    t->n_items = t->ndx * t->nchunk;
    t->lambda_mv = lambda_mv;
    if (t->ndx <= 0 || (size_t)t->n_items * ndy > q2cap || t->ndx * t->ndy > (1 << 15)) return UC_ERR_ARG;
    // per lane group: its candidates sorted by (mvcost & 0xffff, raster)
    for (int g = 0; g < ME_GROUPS; g++) {
        std::vector<std::pair<u32, u32>> c;   // (r, raster) -> position in the table
        std::vector<std::pair<std::pair<u32, u32>, size_t>> v;
        for (int it = g; it < t->n_items; it += ME_GROUPS) {
            int dx = t->lo_x + it % t->ndx, dy0 = t->lo_y + (it / t->ndx) * ndy;
            for (int j = 0; j < ndy; j++) {
                int dy = dy0 + j;
                size_t pos = (size_t)it * ndy + j;
                if (dy > t->hi_y) { q2tab[pos] = 0xFFFFFFFFu; continue; }
                u32 mvc = (mvbits(4 * dx) + mvbits(4 * dy)) * lambda_mv;
                u32 raster = (u32)((dy - t->lo_y) * t->ndx + (dx - t->lo_x));
                v.push_back({ { mvc & 0xFFFFu, raster }, pos });
            }
        }
        if (v.size() > (size_t)ME_MAX_GROUP) return UC_ERR_ARG;
        std::sort(v.begin(), v.end());
        for (size_t k = 0; k < v.size(); k++) {
            size_t pos = v[k].second;
            int it = (int)(pos / ndy), j = (int)(pos % ndy);
            int dx = t->lo_x + it % t->ndx, dy = t->lo_y + (it / t->ndx) * ndy + j;
            u32 mvc = (mvbits(4 * dx) + mvbits(4 * dy)) * lambda_mv;
            q2tab[pos] = ((mvc >> 16) << ME_RANK_BITS) | (u32)k;
            rank2mv[g * ME_MAX_GROUP + k] = (u16)v[k].first.second;
        }
    }
    return UC_OK;
}

struct MeIntParams {
    const pel *org; int i_org;
    const pel *ref[ME_MAX_REFS]; int i_ref;
    int W, H, ctus_w;
    int lo_x, hi_x, lo_y, hi_y, ndx, nchunk, n_items;
    u32 lambda_mv;
    const u32 *q2tab; const u16 *rank2mv;
    u64 *keys;             // [ctu][ref][169]
    int n_refs;
    int win_h, win_ww;     // window rows, words per stored row (incl. skew room)
    int win_cols;          // window data bytes per row
    int pad;               // reference padding (samples)
    int edge, nx_int, ny_int, ctus_h;   // CTU subset of this launch (see ctu_of)
};

// CTU of this CTA: interior launches cover the nx_int x ny_int rectangle of CTUs whose blocks
// can never reach the right/bottom MV limit; edge launches cover the rest (right strip, then
// bottom strip)
__device__ __forceinline__ void ctu_of(const MeIntParams &P, int i, int *col, int *row)
{
    if (!P.edge) { *col = i % P.nx_int; *row = i / P.nx_int; return; }
    const int rw = P.ctus_w - P.nx_int;
    if (i < rw * P.ctus_h) { *col = P.nx_int + i % rw; *row = i / rw; return; }
    i -= rw * P.ctus_h;
    *col = i % P.nx_int; *row = P.ny_int + i / P.nx_int;
}

// word skew of window row r: rows 16 apart (the four sub-block rows of a half-warp) land on
// bank offsets 0, 16, 2, 18, which with the 4-word column steps of the sub-block columns
// gives 16 distinct even banks per half-warp
__device__ __forceinline__ int win_skew(int r)
{
    int t = (r >> 4) & 3;
    return ((t & 1) << 4) | ((t >> 1) << 1);
}

__device__ __forceinline__ void upd(u32 &b, u32 v, bool ok)
{
    if (ok) b = min(b, v);
}

template <int NDY, bool EDGE>
__global__ void __launch_bounds__(256, 2) k_me_int(MeIntParams P)
{
    extern __shared__ __align__(16) u32 win[];
    __shared__ unsigned long long skey[ME_BLOCKS_PER_CTU];

    const int ref = blockIdx.y;
    int ccol, crow;
    ctu_of(P, blockIdx.x, &ccol, &crow);
    const int ctu = crow * P.ctus_w + ccol;
    const int cx = ccol * ME_CTU, cy = crow * ME_CTU;
    const int tid = threadIdx.x;
    const pel *rp = P.ref[ref];

    // ---- stage the search window: rows cy+lo_y .., columns from a 16-byte boundary.
    // Row r is stored at word r*win_ww + skew(r): the 16 lanes of a half-warp read rows 16
    // apart, and the skew spreads them over distinct banks.
    const pel *g0 = rp + (long long)(cy + P.lo_y) * P.i_ref + (cx + P.lo_x);
    const int off = (int)(((uintptr_t)g0) & 15);
    const pel *gw = g0 - off;
    const int wwords = P.win_cols >> 2;                 // words of window data per row
    // columns past the right padding are never read by a valid candidate: filled with 0
    const int gcol0 = cx + P.lo_x - off, gcol_end = P.W + P.pad;
    if ((P.i_ref & 15) == 0) {
        const int nv = wwords >> 2;
        for (int i = tid; i < P.win_h * nv; i += blockDim.x) {
            int r = i / nv, c = i % nv;
            uint4 v;
            if (gcol0 + c * 16 + 15 < gcol_end) {
                v = __ldg(reinterpret_cast<const uint4 *>(gw + (long long)r * P.i_ref) + c);
            } else {
                u32 wv[4];
                for (int q = 0; q < 4; q++) {
                    wv[q] = 0;
                    for (int b = 0; b < 4; b++) {
                        int col = c * 16 + q * 4 + b;
                        if (gcol0 + col < gcol_end) wv[q] |= (u32)gw[(long long)r * P.i_ref + col] << (8 * b);
                    }
                }
                v = make_uint4(wv[0], wv[1], wv[2], wv[3]);
            }
            u32 *d = win + r * P.win_ww + win_skew(r) + 4 * c;
            d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w;
        }
    } else {
        for (int i = tid; i < P.win_h * wwords; i += blockDim.x) {
            int r = i / wwords, c = i % wwords;
            u32 v = 0;
            for (int b = 0; b < 4; b++) {
                int col = 4 * c + b;
                if (gcol0 + col < gcol_end) v |= (u32)gw[(long long)r * P.i_ref + col] << (8 * b);
            }
            win[r * P.win_ww + win_skew(r) + c] = v;
        }
    }
    for (int i = tid; i < ME_BLOCKS_PER_CTU; i += blockDim.x) skey[i] = ~0ull;

    const int lane = tid & 31, warp = tid >> 5;
    const int s = lane & 15, g = warp * 2 + (lane >> 4);
    const int sx = s & 3, sy = s >> 2;

    // ---- org 16x16 sub-block in registers (reads clamped to the picture)
    u32 o[16][4];
    {
        const int ox = cx + 16 * sx, oy = cy + 16 * sy;
#pragma unroll
        for (int r = 0; r < 16; r++) {
            const pel *orow = P.org + (long long)min(oy + r, P.H - 1) * P.i_org;
#pragma unroll
            for (int w = 0; w < 4; w++) {
                u32 v = 0;
#pragma unroll
                for (int b = 0; b < 4; b++) v |= (u32)orow[min(ox + 4 * w + b, P.W - 1)] << (8 * b);
                o[r][w] = v;
            }
        }
    }
    __syncthreads();

    // block-validity limits at the right/bottom picture edge (max_mv = pic - 1 - pos)
    const int lim_x0 = P.W - 1 - (cx + 16 * sx), lim_x1 = lim_x0 - 8;
    const int lim_y0 = P.H - 1 - (cy + 16 * sy), lim_y1 = lim_y0 - 8;

    u32 best[15];
#pragma unroll
    for (int i = 0; i < 15; i++) best[i] = 0xFFFFFFFFu;

    const int n_iter = (P.n_items + ME_GROUPS - 1) / ME_GROUPS;   // warp-uniform trip count
    for (int k = 0; k < n_iter; k++) {
        const int it = g + k * ME_GROUPS;
        const bool item_ok = it < P.n_items;
        const int iti = item_ok ? it : 0;
        const int dxi = iti % P.ndx, dyc = iti / P.ndx;
        const int dx = P.lo_x + dxi, dy0 = P.lo_y + dyc * NDY;
        const int bx = off + 16 * sx + dxi;
        const int sh = bx & 3;
        // rows R0 .. R0+15+NDY-1 of the window; the skew changes once, at the same row for
        // every lane (16*sy is a multiple of 16), so two base pointers cover the item
        const int R0 = 16 * sy + dyc * NDY;
        const int rr_c = 16 - (R0 & 15);
        const u32 *p0 = win + R0 * P.win_ww + win_skew(R0) + (bx >> 2);
        const u32 *p1 = p0 + (win_skew(R0 + 16) - win_skew(R0));

        u32 acc[NDY][4];
#pragma unroll
        for (int j = 0; j < NDY; j++)
#pragma unroll
            for (int t = 0; t < 4; t++) acc[j][t] = 0;

#pragma unroll
        for (int rr = 0; rr < 16 + NDY - 1; rr++) {
            const u32 *wp = (rr < rr_c ? p0 : p1) + rr * P.win_ww;
            const u32 w0 = wp[0], w1 = wp[1], w2 = wp[2], w3 = wp[3], w4 = wp[4];
            const u32 a0 = align4(w0, w1, sh), a1 = align4(w1, w2, sh);
            const u32 a2 = align4(w2, w3, sh), a3 = align4(w3, w4, sh);
#pragma unroll
            for (int j = 0; j < NDY; j++) {
                const int r = rr - j;
                if (r < 0 || r >= 16) continue;
                const int t = (r >> 3) * 2;
                acc[j][t] = sad4(o[r][0], a0, acc[j][t]);
                acc[j][t] = sad4(o[r][1], a1, acc[j][t]);
                acc[j][t + 1] = sad4(o[r][2], a2, acc[j][t + 1]);
                acc[j][t + 1] = sad4(o[r][3], a3, acc[j][t + 1]);
            }
        }

        const u32 *q2p = P.q2tab + (size_t)iti * NDY;
#pragma unroll
        for (int j = 0; j < NDY; j++) {
            const int dy = dy0 + j;
            const u32 q2 = __ldg(q2p + j);
            const bool ok = item_ok && q2 != 0xFFFFFFFFu;
            bool vx0 = true, vx1 = true, vy0 = true, vy1 = true;
            if (EDGE) { vx0 = dx <= lim_x0; vx1 = dx <= lim_x1; vy0 = dy <= lim_y0; vy1 = dy <= lim_y1; }
            const u32 t00 = acc[j][0], t01 = acc[j][1], t10 = acc[j][2], t11 = acc[j][3];
            // keys (sad << 11) + q2, sums of keys formed as a + b - q2 (exact modulo 2^32)
            const u32 v00 = (t00 << ME_RANK_BITS) + q2, v01 = (t01 << ME_RANK_BITS) + q2;
            const u32 v10 = (t10 << ME_RANK_BITS) + q2, v11 = (t11 << ME_RANK_BITS) + q2;
            const u32 vt = v00 + (t01 << ME_RANK_BITS), vb = v10 + (t11 << ME_RANK_BITS);
            const u32 vl = v00 + (t10 << ME_RANK_BITS), vr = v01 + (t11 << ME_RANK_BITS);
            const u32 v16 = vt + vb - q2;
            const bool v00ok = ok && vx0 && vy0;
            upd(best[0], v00, v00ok);
            upd(best[1], v01, ok && vx1 && vy0);
            upd(best[2], v10, ok && vx0 && vy1);
            upd(best[3], v11, ok && vx1 && vy1);
            upd(best[4], vt, v00ok);                  // 16x8 top
            upd(best[5], vb, ok && vx0 && vy1);       // 16x8 bottom
            upd(best[6], vl, v00ok);                  // 8x16 left
            upd(best[7], vr, ok && vx1 && vy0);       // 8x16 right
            upd(best[8], v16, v00ok);
            const u32 v32x16 = v16 + __shfl_xor_sync(0xFFFFFFFFu, v16, 1) - q2;
            const u32 v16x32 = v16 + __shfl_xor_sync(0xFFFFFFFFu, v16, 4) - q2;
            const u32 v32 = v32x16 + __shfl_xor_sync(0xFFFFFFFFu, v32x16, 4) - q2;
            const u32 v64x32 = v32 + __shfl_xor_sync(0xFFFFFFFFu, v32, 2) - q2;
            const u32 v32x64 = v32 + __shfl_xor_sync(0xFFFFFFFFu, v32, 8) - q2;
            const u32 v64 = v64x32 + __shfl_xor_sync(0xFFFFFFFFu, v64x32, 8) - q2;
            upd(best[9], v32x16, v00ok);
            upd(best[10], v16x32, v00ok);
            upd(best[11], v32, v00ok);
            upd(best[12], v64x32, v00ok);
            upd(best[13], v32x64, v00ok);
            upd(best[14], v64, v00ok);
        }
    }

    // ---- decode the lane group's winners and merge into the CTU's 64-bit keys
    {
        int ids[15];
#pragma unroll
        for (int i = 0; i < 2; i++)
#pragma unroll
            for (int j = 0; j < 2; j++) ids[j * 2 + i] = (2 * sy + j) * 8 + 2 * sx + i;
        ids[4] = 64 + (2 * sy) * 4 + sx;
        ids[5] = 64 + (2 * sy + 1) * 4 + sx;
        ids[6] = 96 + sy * 8 + 2 * sx;
        ids[7] = 96 + sy * 8 + 2 * sx + 1;
        ids[8] = 128 + sy * 4 + sx;
        ids[9] = (sx & 1) ? -1 : 144 + sy * 2 + (sx >> 1);
        ids[10] = (sy & 1) ? -1 : 152 + (sy >> 1) * 4 + sx;
        ids[11] = ((sx | sy) & 1) ? -1 : 160 + (sy >> 1) * 2 + (sx >> 1);
        ids[12] = (sx == 0 && !(sy & 1)) ? 164 + (sy >> 1) : -1;
        ids[13] = (sy == 0 && !(sx & 1)) ? 166 + (sx >> 1) : -1;
        ids[14] = (sx == 0 && sy == 0) ? 168 : -1;
        const u16 *r2m = P.rank2mv + g * ME_MAX_GROUP;
#pragma unroll
        for (int i = 0; i < 15; i++) {
            const u32 b = best[i];
            if (ids[i] < 0 || b == 0xFFFFFFFFu) continue;
            const u32 raster = r2m[b & (ME_MAX_GROUP - 1)];
            const int dx = P.lo_x + (int)(raster % P.ndx), dy = P.lo_y + (int)(raster / P.ndx);
            const u32 mvc = (mvbits(4 * dx) + mvbits(4 * dy)) * P.lambda_mv;
            const u64 cost = ((u64)(b >> ME_RANK_BITS) << 16) + (mvc & 0xFFFFu);
            atomicMin(&skey[ids[i]], (unsigned long long)((cost << 15) | raster));
        }
    }
    __syncthreads();
    u64 *dst = P.keys + ((size_t)ctu * P.n_refs + ref) * ME_BLOCKS_PER_CTU;
    for (int i = tid; i < ME_BLOCKS_PER_CTU; i += blockDim.x) dst[i] = skey[i];
}

// ---------------------------------------------------------------- fractional refinement
//
// Task grid: one thread per (block, reference, candidate, com_had tile).  Stage 1 evaluates
// the centre and the 8 half-sample points, stage 2 the 8 quarter-sample points around the
// stage-1 winner (each stage-2 thread re-derives that winner from the stage-1 sums), and a
// final pass picks the stage-2 winner.  Tile SATDs are summed per (block, reference,
// candidate) with global atomics; candidate order and the strict '<' of me_sub_pel_search
// are applied in the selection.

struct MeSubParams {
    const pel *org; int i_org;
    const pel *planes[ME_MAX_REFS][16]; int i_ref;
    int W, H, ctus_w, n_ctu, n_refs;
    int lo_x, lo_y, ndx;
    u32 lambda_mv;
    double sq32, sq128;
    const u64 *keys;
    u32 *satd1;          // [item][9]
    u32 *satd2;          // [item][8]
    MeResult *out;
    long long task_base[11];   // prefix of tasks per shape class
};

__constant__ s8 kHalfPat[8][2] = { { -2, 0 }, { -2, 2 }, { 0, 2 }, { 2, 2 }, { 2, 0 }, { 2, -2 }, { 0, -2 }, { -2, -2 } };
__constant__ s8 kQuarPat[8][2] = { { -1, 0 }, { 0, 1 }, { 1, 0 }, { 0, -1 }, { -1, 1 }, { 1, 1 }, { -1, -1 }, { 1, -1 } };
__constant__ CtuBlock kCtuBlocks[ME_BLOCKS_PER_CTU];
// shape classes of the CTU block table: first block index, count, width, height
__constant__ int kShapeFirst[11] = { 0, 64, 96, 128, 144, 152, 160, 164, 166, 168, 169 };
__constant__ u8 kShapeWH[10][2] = { { 8, 8 }, { 16, 8 }, { 8, 16 }, { 16, 16 }, { 32, 16 }, { 16, 32 }, { 32, 32 },
                                   { 64, 32 }, { 32, 64 }, { 64, 64 } };

// com_mc_blk_luma_pointer (src/com_mc.c:89-101) for a block at (x, y) with qpel MV (mvx, mvy)
__device__ __forceinline__ const pel *mc_ptr(const MeSubParams &P, int ref, int x, int y, int mvx, int mvy)
{
    int qx = (x << 2) + mvx, qy = (y << 2) + mvy;
    int px = min(max(qx >> 2, -128 - 4), P.W + 4), py = min(max(qy >> 2, -128 - 4), P.H + 4);
    return P.planes[ref][(qy & 3) * 4 + (qx & 3)] + (long long)py * P.i_ref + px;
}

// 8 samples at p (any alignment) as two little-endian words; reads only words that hold
// requested samples
__device__ __forceinline__ void load8(const pel *p, u32 &lo, u32 &hi)
{
    const uintptr_t a = (uintptr_t)p;
    const u32 *q = (const u32 *)(a & ~(uintptr_t)3);
    const u32 sh = (u32)(a & 3) * 8;
    const u32 w0 = __ldg(q), w1 = __ldg(q + 1);
    const u32 w2 = sh ? __ldg(q + 2) : 0u;
    lo = __funnelshift_r(w0, w1, sh);
    hi = __funnelshift_r(w1, w2, sh);
}

// magnitude sum of the 2-D WHT of the 8x8 difference org - pred; with o2/p2 the second 8x8
// half of a 16x8 / 8x16 tile is folded in as first + sgn * second (the first stage of the
// 16-point transform).  Rows are transformed as they are loaded.
__device__ __noinline__ int satd8x8_raw(const pel *o, int io, const pel *p, int ip, const pel *o2, const pel *p2,
                                           int sgn)
{
    int d[64];
#pragma unroll
    for (int r = 0; r < 8; r++) {
        u32 ol, oh, pl, ph;
        load8(o + r * io, ol, oh);
        load8(p + r * ip, pl, ph);
        int v[8];
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const u32 ow = c < 4 ? ol : oh, pw = c < 4 ? pl : ph;
            v[c] = (int)((ow >> (8 * (c & 3))) & 255) - (int)((pw >> (8 * (c & 3))) & 255);
        }
        if (o2) {
            load8(o2 + r * io, ol, oh);
            load8(p2 + r * ip, pl, ph);
#pragma unroll
            for (int c = 0; c < 8; c++) {
                const u32 ow = c < 4 ? ol : oh, pw = c < 4 ? pl : ph;
                v[c] += sgn * ((int)((ow >> (8 * (c & 3))) & 255) - (int)((pw >> (8 * (c & 3))) & 255));
            }
        }
        wht<8>(v);
#pragma unroll
        for (int c = 0; c < 8; c++) d[r * 8 + c] = v[c];
    }
    int s = 0;
#pragma unroll
    for (int c = 0; c < 8; c++) {
        int col[8];
#pragma unroll
        for (int r = 0; r < 8; r++) col[r] = d[r * 8 + c];
        wht<8>(col);
#pragma unroll
        for (int r = 0; r < 8; r++) s += abs(col[r]);
    }
    return s;
}

// com_had tile SATD for the ME tile shapes 8x8 / 16x8 / 8x16.  For 16x8 (8x16) the 16-point
// transform's first stage forms left+right and left-right (top+bottom, top-bottom); the
// magnitude sum is the sum of the two 8x8 transforms of those.
__device__ __forceinline__ u32 me_tile_satd(int tw, int th, const pel *o, int io, const pel *p, int ip, double sq128)
{
    if (tw == 8 && th == 8) return (u32)((satd8x8_raw(o, io, p, ip, nullptr, nullptr, 0) + 2) >> 2);
    const int bo = tw == 16 ? 8 : 8 * io, bp = tw == 16 ? 8 : 8 * ip;
    int s = satd8x8_raw(o, io, p, ip, o + bo, p + bp, 1);
    s += satd8x8_raw(o, io, p, ip, o + bo, p + bp, -1);
    return (u32)(int)((double)s / sq128 * 2.0);
}

struct SubTask { int item, ctu, b, ref, cand, tile, x, y, w, h, tw, th; };

__device__ __forceinline__ bool decode_task(const MeSubParams &P, long long t, int ncand, SubTask &k)
{
    int s = 0;
    while (s < 9 && t >= P.task_base[s + 1]) s++;
    long long l = t - P.task_base[s];
    const int w = kShapeWH[s][0], h = kShapeWH[s][1];
    int tw, th;
    had_tile_shape(w, h, &tw, &th);
    const int ntiles = (w * h) / (tw * th);
    const int cnt = kShapeFirst[s + 1] - kShapeFirst[s];
    k.tile = (int)(l % ntiles); l /= ntiles;
    k.cand = (int)(l % ncand); l /= ncand;
    k.ref = (int)(l % P.n_refs); l /= P.n_refs;
    k.b = kShapeFirst[s] + (int)(l % cnt);
    k.ctu = (int)(l / cnt);
    k.item = (k.ctu * ME_BLOCKS_PER_CTU + k.b) * P.n_refs + k.ref;
    const CtuBlock cb = kCtuBlocks[k.b];
    k.x = (k.ctu % P.ctus_w) * ME_CTU + cb.x;
    k.y = (k.ctu / P.ctus_w) * ME_CTU + cb.y;
    k.w = w; k.h = h; k.tw = tw; k.th = th;
    return k.x + w <= P.W && k.y + h <= P.H;
}

__device__ __forceinline__ void int_winner(const MeSubParams &P, int ctu, int b, int ref, int &dx, int &dy, u64 &key)
{
    key = P.keys[((size_t)ctu * P.n_refs + ref) * ME_BLOCKS_PER_CTU + b];
    const u32 raster = (u32)(key & 0x7FFF);
    dx = P.lo_x + (int)(raster % P.ndx);
    dy = P.lo_y + (int)(raster / P.ndx);
}

__device__ __forceinline__ u64 sub_cost(const MeSubParams &P, int vx, int vy, u32 satd)
{
    return (u64)((mvbits(vx) + mvbits(vy)) * P.lambda_mv) + ((u64)satd << 16);
}

// stage-1 winner (centre first, then the half-sample pattern, strict '<')
__device__ __forceinline__ void hpel_winner(const MeSubParams &P, int item, int cx, int cy, int &mx, int &my,
                                            u64 &cbest, u32 &bsatd)
{
    const u32 *s1 = P.satd1 + (size_t)item * 9;
    mx = cx; my = cy; bsatd = s1[0];
    cbest = sub_cost(P, cx, cy, bsatd);
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const int vx = cx + kHalfPat[c][0], vy = cy + kHalfPat[c][1];
        const u32 sd = s1[c + 1];
        const u64 cost = sub_cost(P, vx, vy, sd);
        if (cost < cbest) { cbest = cost; mx = vx; my = vy; bsatd = sd; }
    }
}

template <int STAGE>
__global__ void __launch_bounds__(256, 2) k_me_sub_eval(MeSubParams P, long long n_tasks)
{
    const int ncand = STAGE == 1 ? 9 : 8;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n_tasks;
         t += (long long)gridDim.x * blockDim.x) {
        SubTask k;
        if (!decode_task(P, t, ncand, k)) continue;
        int dx, dy;
        u64 key;
        int_winner(P, k.ctu, k.b, k.ref, dx, dy, key);
        int cx = dx * 4, cy = dy * 4;
        const pel *pb;
        if (STAGE == 1) {
            if (k.cand == 0) {
                pb = P.planes[k.ref][0] + (long long)(k.y + dy) * P.i_ref + (k.x + dx);
            } else {
                pb = mc_ptr(P, k.ref, k.x, k.y, cx + kHalfPat[k.cand - 1][0], cy + kHalfPat[k.cand - 1][1]);
            }
        } else {
            int mx, my; u64 cb; u32 bs;
            hpel_winner(P, k.item, cx, cy, mx, my, cb, bs);
            pb = mc_ptr(P, k.ref, k.x, k.y, mx + kQuarPat[k.cand][0], my + kQuarPat[k.cand][1]);
        }
        const int ntx = k.w / k.tw;
        const int tx = (k.tile % ntx) * k.tw, ty = (k.tile / ntx) * k.th;
        const pel *ob = P.org + (long long)(k.y + ty) * P.i_org + k.x + tx;
        const u32 v = me_tile_satd(k.tw, k.th, ob, P.i_org, pb + (long long)ty * P.i_ref + tx, P.i_ref, P.sq128);
        atomicAdd((STAGE == 1 ? P.satd1 + (size_t)k.item * 9 : P.satd2 + (size_t)k.item * 8) + k.cand, v);
    }
}

__global__ void __launch_bounds__(256) k_me_sub_final(MeSubParams P)
{
    const long long total = (long long)P.n_ctu * ME_BLOCKS_PER_CTU * P.n_refs;
    for (long long item = blockIdx.x * (long long)blockDim.x + threadIdx.x; item < total;
         item += (long long)gridDim.x * blockDim.x) {
        const int ref = (int)(item % P.n_refs);
        const int b = (int)((item / P.n_refs) % ME_BLOCKS_PER_CTU);
        const int ctu = (int)(item / P.n_refs / ME_BLOCKS_PER_CTU);
        const CtuBlock cb = kCtuBlocks[b];
        const int x = (ctu % P.ctus_w) * ME_CTU + cb.x, y = (ctu / P.ctus_w) * ME_CTU + cb.y;
        MeResult r = {};
        if (x + cb.w > P.W || y + cb.h > P.H) {
            r.cost_int = ~0ull; r.cost_sub = ~0ull;
            P.out[item] = r;
            continue;
        }
        int dx, dy;
        u64 key;
        int_winner(P, ctu, b, ref, dx, dy, key);
        const u64 cost_int = key >> 15;
        const u32 mvc = (mvbits(4 * dx) + mvbits(4 * dy)) * P.lambda_mv;
        int mx, my; u64 cbest; u32 bsatd;
        hpel_winner(P, (int)item, dx * 4, dy * 4, mx, my, cbest, bsatd);
        const u32 *s2 = P.satd2 + (size_t)item * 8;
        const int hx = mx, hy = my;
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const int vx = hx + kQuarPat[c][0], vy = hy + kQuarPat[c][1];
            const u64 cost = sub_cost(P, vx, vy, s2[c]);
            if (cost < cbest) { cbest = cost; mx = vx; my = vy; bsatd = s2[c]; }
        }
        r.mv_int[0] = (s16)dx; r.mv_int[1] = (s16)dy;
        r.mv_sub[0] = (s16)mx; r.mv_sub[1] = (s16)my;
        r.sad_int = (u32)((cost_int - mvc) >> 16);
        r.satd_sub = bsatd;
        r.cost_int = cost_int;
        r.cost_sub = cbest;
        P.out[item] = r;
    }
}

static bool g_ctu_tab_uploaded[64];

int launch_me_frame(const MeFrameArgs &a, const MeTables &t, u64 *keys, cudaStream_t st)
{
    int dev = 0;
    UC_CHECK(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && !g_ctu_tab_uploaded[dev]) {
        CtuBlock tab[ME_BLOCKS_PER_CTU];
        ctu_block_table(tab);
        UC_CHECK(cudaMemcpyToSymbol(kCtuBlocks, tab, sizeof(tab)));
        g_ctu_tab_uploaded[dev] = true;
    }
    const int ctus_w = (a.W + 63) / 64, ctus_h = (a.H + 63) / 64;
    MeIntParams P;
    P.org = a.org; P.i_org = a.i_org;
    for (int r = 0; r < ME_MAX_REFS; r++) P.ref[r] = r < a.n_refs ? a.planes[r][0] : nullptr;
    P.i_ref = a.i_ref; P.W = a.W; P.H = a.H; P.ctus_w = ctus_w;
    P.lo_x = t.lo_x; P.hi_x = t.hi_x; P.lo_y = t.lo_y; P.hi_y = t.hi_y;
    P.ndx = t.ndx; P.nchunk = t.nchunk; P.n_items = t.n_items; P.lambda_mv = a.lambda_mv;
    P.q2tab = a.q2tab; P.rank2mv = a.rank2mv; P.keys = keys; P.n_refs = a.n_refs;
    constexpr int NDY = ME_NDY;
    if (t.ndy_per_item != NDY) return set_status(UC_ERR_ARG, "me: table built for another NDY");
    P.win_h = 64 + t.nchunk * NDY - 1 + 1;
    P.win_cols = ((15 + 64 + t.ndx + 4 + 15) / 16) * 16;
    P.win_ww = (P.win_cols >> 2) + 18 + 2;    // even, room for the largest skew
    const size_t smem = (size_t)P.win_h * P.win_ww * 4;
    static bool attr_set[64];
    if (dev >= 0 && dev < 64 && !attr_set[dev]) {
        UC_CHECK(cudaFuncSetAttribute(k_me_int<NDY, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
        UC_CHECK(cudaFuncSetAttribute(k_me_int<NDY, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
        attr_set[dev] = true;
    }
    if (smem > 100 * 1024) return set_status(UC_ERR_ARG, "me: window too large");
    // interior CTUs: every 8x8 tile satisfies pos + 8 + hi <= pic - 1 in both directions
    int nx = a.W - 57 - t.hi_x >= 0 ? (a.W - 57 - t.hi_x) / 64 + 1 : 0;
    int ny = a.H - 57 - t.hi_y >= 0 ? (a.H - 57 - t.hi_y) / 64 + 1 : 0;
    nx = std::min(nx, ctus_w); ny = std::min(ny, ctus_h);
    P.pad = a.pad; P.ctus_h = ctus_h; P.nx_int = nx; P.ny_int = ny;
    prof_begin(PROF_ME_INT, st);
    if (nx * ny > 0) {
        P.edge = 0;
        k_me_int<NDY, false><<<dim3(nx * ny, a.n_refs), 256, smem, st>>>(P);
        UC_CHECK(cudaGetLastError());
        count_launch(1);
    }
    const int n_edge = ctus_w * ctus_h - nx * ny;
    if (n_edge > 0) {
        P.edge = 1;
        k_me_int<NDY, true><<<dim3(n_edge, a.n_refs), 256, smem, st>>>(P);
        UC_CHECK(cudaGetLastError());
        count_launch(1);
    }
    prof_end(PROF_ME_INT, st);

    MeSubParams S;
    S.org = a.org; S.i_org = a.i_org;
    for (int r = 0; r < ME_MAX_REFS; r++)
        for (int q = 0; q < 16; q++) S.planes[r][q] = r < a.n_refs ? a.planes[r][q] : nullptr;
    S.i_ref = a.i_ref; S.W = a.W; S.H = a.H; S.ctus_w = ctus_w; S.n_ctu = ctus_w * ctus_h; S.n_refs = a.n_refs;
    S.lo_x = t.lo_x; S.lo_y = t.lo_y; S.ndx = t.ndx; S.lambda_mv = a.lambda_mv;
    S.sq32 = sqrt(32.0); S.sq128 = sqrt(128.0);
    S.keys = keys; S.out = a.out;
    const long long items = (long long)S.n_ctu * ME_BLOCKS_PER_CTU * a.n_refs;
    S.satd1 = a.sub_scratch;
    S.satd2 = a.sub_scratch + items * 9;
    CtuBlock tab[ME_BLOCKS_PER_CTU];
    ctu_block_table(tab);
    static const int first[11] = { 0, 64, 96, 128, 144, 152, 160, 164, 166, 168, 169 };
    long long tb1[11], tb2[11];
    tb1[0] = tb2[0] = 0;
    for (int s = 0; s < 10; s++) {
        int w = tab[first[s]].w, h = tab[first[s]].h, tw, th;
        had_tile_shape(w, h, &tw, &th);
        long long n = (long long)S.n_ctu * (first[s + 1] - first[s]) * a.n_refs * ((w * h) / (tw * th));
        tb1[s + 1] = tb1[s] + n * 9;
        tb2[s + 1] = tb2[s] + n * 8;
    }
    UC_CHECK(cudaMemsetAsync(a.sub_scratch, 0, (size_t)items * 17 * sizeof(u32), st));
    prof_begin(PROF_ME_SUB, st);
    for (int s = 0; s < 11; s++) S.task_base[s] = tb1[s];
    k_me_sub_eval<1><<<(unsigned)std::min<long long>((tb1[10] + 255) / 256, 152 * 64), 256, 0, st>>>(S, tb1[10]);
    UC_CHECK(cudaGetLastError());
    for (int s = 0; s < 11; s++) S.task_base[s] = tb2[s];
    k_me_sub_eval<2><<<(unsigned)std::min<long long>((tb2[10] + 255) / 256, 152 * 64), 256, 0, st>>>(S, tb2[10]);
    UC_CHECK(cudaGetLastError());
    k_me_sub_final<<<(unsigned)std::min<long long>((items + 255) / 256, 152 * 16), 256, 0, st>>>(S);
    UC_CHECK(cudaGetLastError());
    count_launch(3);
    prof_end(PROF_ME_SUB, st);
    return UC_OK;
}

}  // namespace uc
