// Batched motion search of every block of a frame (8x8 .. 64x64 including 2:1 shapes on the
// 64x64 CTU grid), bit-exact with the per-candidate costs of uavs3e's motion search:
//   integer stage: cost = (SAD << 16) + (mvbits(4dx) + mvbits(4dy)) * lambda_mv over the full
//     clipped window, strict '<' in raster order (cost_sad + GET_MVBITS_IPEL_*,
//     src/me.c:103-197 and src/com_cost.c:40-115; window limits as get_max_search_range,
//     src/me.c:502-527, with is_padding = 1 and mvp = 0);
//   fractional stage: me_sub_pel_search with SATD cost (src/me.c:366-500): centre, 8
//     half-sample and 8 quarter-sample neighbours, com_had on the interpolated planes.
//
// Integer stage layout: one CTA per (CTU, reference, class of dx mod 4).  Its search window
// is staged once into shared memory, pre-shifted so that the class's reference words are
// word-aligned.  A half-warp covers the CTU as a 4x4 grid of 16x16 sub-blocks (one lane each,
// org samples in registers) and sweeps NDY vertically adjacent candidates at one dx, so every
// reference word is reused by up to NDY rows of the block.  The four 8x8 tile SADs of a lane
// give the 8x8/16x8/8x16/16x16 blocks; warp shuffles give the 32x16 .. 64x64 ones.  Each
// block keeps a 32-bit running minimum of
//     ((SAD + q) << 11) | rank,   q = mvcost >> 16,
// where rank orders this lane group's candidates by (mvcost & 0xffff, raster index): the
// minimum is then exactly the (cost, raster) minimum, so a block update is one IMAD + one
// IMNMX.  Per-group winners are merged into a 64-bit (cost << 15 | raster) key, first in
// shared memory, then across the four class CTAs with global atomics.
#include "common.cuh"
#include "tma.cuh"
#include "uavs3e_cuda_internal.h"
#include <algorithm>

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

size_t me_sub_scratch_bytes(int W, int H, int n_refs)
{
    size_t nctu = (size_t)((W + 63) / 64) * ((H + 63) / 64);
    return nctu * n_refs * ME_BLOCKS_PER_CTU * 18 * sizeof(u32);
}

size_t me_key_scratch_bytes(int W, int H, int n_refs)
{
    size_t nctu = (size_t)((W + 63) / 64) * ((H + 63) / 64);
    return nctu * n_refs * ME_BLOCKS_PER_CTU * sizeof(u64) + 2 * sizeof(u32);
}

size_t me_shift_scratch_bytes(int W, int H, int n_refs)
{
    const size_t pitch = ((size_t)W + 2 * 144 + 15) & ~(size_t)15;
    return (size_t)n_refs * 4 * pitch * (size_t)(H + 2 * 144);
}

// Search items.  Candidates of one alignment class c (dx index = c mod 4) are cut into main
// items of ME_NDY vertically adjacent candidates (rows 8k .. 8k+7 of the dy range) and, for
// the ndy % 8 rows left at the bottom, tail items of one candidate.  Each list is padded to a
// multiple of ME_GROUPS items with repeats of its first items, so every lane group has work
// and needs no validity test; a repeated candidate only repeats a key.  Lane group g takes
// items g, g + 16, ...; its candidates are ranked by (mvcost & 0xffff, raster).
//
// Buffer layout (u32): per class [main q2: 8 per item][tail q2: 1 per item], then per class
// [main descriptors][tail descriptors]; a descriptor is dx_k | dy_row << 16 for the dx index
// c + 4 dx_k and the dy index dy_row (of the item's first candidate).
int me_build_tables(int W, int H, int range, u32 lambda_mv, int ndy, MeTables *t, u32 *q2tab, u16 *rank2mv,
                    size_t q2cap, MeCand *cand)
{
    if (ndy != ME_NDY) return UC_ERR_ARG;
    int M = std::max(W, H);
    t->lo_x = t->lo_y = std::max(-range, -M + 4);
    t->hi_x = t->hi_y = std::min(range, M - 4);
    t->ndx = t->hi_x - t->lo_x + 1;
    t->ndy = t->hi_y - t->lo_y + 1;
    t->ndy_per_item = ndy;
    t->nfull = t->ndy / ndy;
    t->rem = t->ndy % ndy;
    t->lambda_mv = lambda_mv;
    if (t->ndx <= 0 || t->ndx * t->ndy > (1 << 15)) return UC_ERR_ARG;
    const auto up16 = [](int n) { return (n + ME_GROUPS - 1) / ME_GROUPS * ME_GROUPS; };
    size_t pos = 0;
    int nm_real[ME_CLASSES], nt_real[ME_CLASSES];
    for (int c = 0; c < ME_CLASSES; c++) {
        t->n_dx[c] = t->ndx > c ? (t->ndx - c + ME_CLASSES - 1) / ME_CLASSES : 0;
        nm_real[c] = t->n_dx[c] * t->nfull;
        nt_real[c] = t->n_dx[c] * t->rem;
        t->n_main[c] = up16(nm_real[c]);
        t->n_tail[c] = up16(nt_real[c]);
        t->q2_main[c] = (int)pos; pos += (size_t)t->n_main[c] * ndy;
        t->q2_tail[c] = (int)pos; pos += (size_t)t->n_tail[c];
    }
    for (int c = 0; c < ME_CLASSES; c++) {
        t->d_main[c] = (int)pos; pos += (size_t)t->n_main[c];
        t->d_tail[c] = (int)pos; pos += (size_t)t->n_tail[c];
    }
    if (pos > q2cap) return UC_ERR_ARG;
    t->n_entries = (int)pos;
    // Item order: the two lane groups of a warp run items it and it + 1 (it even) side by side,
    // and their window words differ by their dx index difference k' - k.  The list therefore
    // starts with every row's pairs (k, k + 16), k < 16, so such partners sit 16 words (16 banks)
    // apart and the two half-warps' 16-bank sets do not overlap; the dx indices left unpaired
    // (k >= 32, or all of them below 17 offsets) follow, row by row.
    for (int c = 0; c < ME_CLASSES; c++) {
        const int n = t->n_dx[c];
        const int pairs = n >= 17 ? std::min(16, n - 16) : 0;
        int left[64], nl = 0;
        if (n > 64) return UC_ERR_ARG;
        for (int k = 0; k < n; k++)
            if (!(k < pairs || (k >= 16 && k < 16 + pairs))) left[nl++] = k;
        // (dx index, row) of entry ri of a list of `rows` rows
        const auto entry = [&](int ri, int rows, int *k, int *row) {
            if (ri < rows * 2 * pairs) {
                const int j = ri % (2 * pairs);
                *row = ri / (2 * pairs);
                *k = (j >> 1) + ((j & 1) ? 16 : 0);
            } else {
                const int r2 = ri - rows * 2 * pairs;
                *row = r2 / nl;
                *k = left[r2 % nl];
            }
        };
        for (int it = 0; it < t->n_main[c]; it++) {
            int k, row;
            entry(it % nm_real[c], t->nfull, &k, &row);
            q2tab[t->d_main[c] + it] = (u32)k | (u32)(ndy * row) << 16;
        }
        for (int it = 0; it < t->n_tail[c]; it++) {
            int k, row;
            entry(it % nt_real[c], t->rem, &k, &row);
            q2tab[t->d_tail[c] + it] = (u32)k | (u32)(ndy * t->nfull + row) << 16;
        }
    }
    for (int c = 0; c < ME_CLASSES; c++)
        for (int g = 0; g < ME_GROUPS; g++) {
            int n = 0;
            const auto add = [&](u32 desc, int j, u32 at) {
                const int dxi = c + ME_CLASSES * (int)(desc & 0xFFFFu), dyi = (int)(desc >> 16) + j;
                const int dx = t->lo_x + dxi, dy = t->lo_y + dyi;
                const u32 mvc = (mvbits(4 * dx) + mvbits(4 * dy)) * lambda_mv;
                cand[n++] = MeCand{ mvc & 0xFFFFu, (u32)(dyi * t->ndx + dxi), at };
            };
            for (int it = g; it < t->n_main[c]; it += ME_GROUPS)
                for (int j = 0; j < ndy; j++) {
                    if (n >= ME_MAX_GROUP) return UC_ERR_ARG;
                    add(q2tab[t->d_main[c] + it], j, (u32)(t->q2_main[c] + it * ndy + j));
                }
            for (int it = g; it < t->n_tail[c]; it += ME_GROUPS) {
                if (n >= ME_MAX_GROUP) return UC_ERR_ARG;
                add(q2tab[t->d_tail[c] + it], 0, (u32)(t->q2_tail[c] + it));
            }
            std::sort(cand, cand + n, [](const MeCand &x, const MeCand &y) {
                return x.r != y.r ? x.r < y.r : x.raster < y.raster;
            });
            for (int k = 0; k < n; k++) {
                const int dx = t->lo_x + (int)(cand[k].raster % t->ndx);
                const int dy = t->lo_y + (int)(cand[k].raster / t->ndx);
                const u32 mvc = (mvbits(4 * dx) + mvbits(4 * dy)) * lambda_mv;
                q2tab[cand[k].pos] = ((mvc >> 16) << ME_RANK_BITS) | (u32)k;
                rank2mv[(c * ME_GROUPS + g) * ME_MAX_GROUP + k] = (u16)cand[k].raster;
            }
        }
    return UC_OK;
}

// words per window row in shared memory: the TMA box is PITCH * 4 = 224 bytes wide, enough for
// range 64 (the largest byte a lane reads is 15 + 48 + 128 + 3 + 12 < 224).  A compile-time
// pitch keeps every row address of an item an immediate offset.
constexpr int ME_WIN_PITCH = 56;
constexpr int ME_WIN_BYTES_W = ME_WIN_PITCH * 4;
// byte-shifted copies of a reference plane: fixed padding and geometry (see k_shift_planes)
constexpr int ME_SHIFT_PAD = 144;
// polls of a window's mbarrier before the search gives up (about a second)
constexpr uint32_t ME_TMA_POLLS = 1u << 22;

struct MeIntParams {
    CUtensorMap maps[ME_MAX_REFS][4];   // per reference and byte shift s: the plane shifted left by s
    const pel *org; int i_org;
    int W, H, ctus_w, ctus_h;
    int lo_x, hi_x, lo_y, hi_y, ndx;
    int n_main[ME_CLASSES], n_tail[ME_CLASSES];     // items per class (multiples of ME_GROUPS)
    int q2_main[ME_CLASSES], q2_tail[ME_CLASSES];   // offsets into q2tab
    int d_main[ME_CLASSES], d_tail[ME_CLASSES];
    u32 lambda_mv;
    u32 mul, one, minus1;  // 2^11, 1, 2^32-1 as run-time values: key arithmetic stays on IMAD
    const u32 *q2tab; const u16 *rank2mv;
    u64 *keys;             // [ctu][ref][169]
    u32 *ctl;              // [1]: 0xFFFFFFFF, or 0 once a CTA gave up waiting for its window
    int n_refs;
    int win_h;             // window rows (row pitch: ME_WIN_PITCH words)
    int nx_int, ny_int;    // interior CTU rectangle (no block can reach the right/bottom MV limit)
};

// CTU of a CTA: interior launches cover the nx_int x ny_int rectangle of CTUs whose blocks can
// never reach the right/bottom MV limit; edge launches cover the rest (right strip, then bottom
// strip)
__device__ __forceinline__ void ctu_of(const MeIntParams &P, int i, bool edge, int *col, int *row)
{
    if (!edge) { *col = i % P.nx_int; *row = i / P.nx_int; return; }
    const int rw = P.ctus_w - P.nx_int;
    if (i < rw * P.ctus_h) { *col = P.nx_int + i % rw; *row = i / rw; return; }
    i -= rw * P.ctus_h;
    *col = i % P.nx_int; *row = P.ny_int + i / P.nx_int;
}

__device__ __forceinline__ void upd(u32 &b, u32 v, bool ok)
{
    if (ok) b = min(b, v);
}

// per-lane constants of the integer search
struct MeLane {
    int sx, sy;
    u32 b0, b1, b2, b3, nb0, nb1, nb2, nb3;   // bits of the lane's sub-block index and complements
    // word order of the lane: at its t-th word load the lane reads word (t ^ sy) of its four, so
    // the 16 lanes of a half-warp (rows 16 apart in a dense window) hit 16 distinct banks; the
    // lanes with sy >= 2 therefore accumulate their right 8x8 tile in the left tile's slot (A)
    // and the left one in slot B
    // largest valid dx / dy of a block whose top-left corner is the lane's 16x16 sub-block (0),
    // its right or lower 8x8 half (1), the 32-aligned pair it belongs to (p), the CTU (c)
    int X0, X1, Xp, Xc, Y0, Y1, Yp, Yc;
};

// One search item of a lane: NDY vertically adjacent candidates at one dx against the lane's
// 16x16 sub-block, folded into the running minima of the 15 blocks the lane keeps.
template <int NDY, bool EDGE>
__device__ __forceinline__ void me_item(const MeIntParams &P, const u32 *win, const u32 (&o)[16][4],
                                        u32 (&best)[15], u32 desc, const u32 *q2p, int cls, int off,
                                        const MeLane &L)
{
    const int dxi = cls + ME_CLASSES * (int)(desc & 0xFFFFu);
    const int dyi0 = (int)(desc >> 16);
    const int dx = P.lo_x + dxi, dy0 = P.lo_y + dyi0;
    const int bx = off + 16 * L.sx + dxi;             // == the window's shift (mod 4)
    const u32 *pb = win + (16 * L.sy + dyi0) * ME_WIN_PITCH + (bx >> 2);
    const u32 *w0 = pb + (0 ^ L.sy), *w1 = pb + (1 ^ L.sy), *w2 = pb + (2 ^ L.sy), *w3 = pb + (3 ^ L.sy);

    u32 acc[NDY][4];
#pragma unroll
    for (int j = 0; j < NDY; j++)
#pragma unroll
        for (int t = 0; t < 4; t++) acc[j][t] = 0;

#pragma unroll
    for (int rr = 0; rr < 16 + NDY - 1; rr++) {
        const u32 a0 = w0[rr * ME_WIN_PITCH], a1 = w1[rr * ME_WIN_PITCH];
        const u32 a2 = w2[rr * ME_WIN_PITCH], a3 = w3[rr * ME_WIN_PITCH];
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

    // keys (sad << 11) + q2 and the SAD sums of larger blocks are IMADs with run-time
    // multipliers (mul = 2^11, one = 1, m1 = -1, lane bits as selectors): they issue on the FMA
    // pipe and leave the integer ALU pipe to the vabsdiff4s and the running minima
    const u32 mul = P.mul, one = P.one, m1 = P.minus1;
    const bool xa = dx <= L.X0, xb = dx <= L.X1, xp = dx <= L.Xp, xc = dx <= L.Xc;
    const bool sw = L.sy >= 2, xA = sw ? xb : xa, xB = sw ? xa : xb;   // limits of slots A / B
    u32 s16[NDY], q2s[NDY];
#pragma unroll
    for (int j = 0; j < NDY; j++) {
        const u32 q2 = __ldg(q2p + j);
        q2s[j] = q2;
        const int dy = dy0 + j;
        const bool ya = dy <= L.Y0, yb = dy <= L.Y1;
        const u32 t00 = acc[j][0], t01 = acc[j][1], t10 = acc[j][2], t11 = acc[j][3];
        const u32 v00 = t00 * mul + q2, v01 = t01 * mul + q2;
        const u32 v10 = t10 * mul + q2, v11 = t11 * mul + q2;
        const u32 vl = t10 * mul + v00, vr = t11 * mul + v01;
        const u32 st = t00 * one + t01, sb = t10 * one + t11;
        const u32 vt = st * mul + q2, vb = sb * mul + q2;
        s16[j] = st * one + sb;
        const u32 v16 = s16[j] * mul + q2;
        upd(best[0], v00, !EDGE || (xA && ya));    // 8x8, slot A top
        upd(best[1], v01, !EDGE || (xB && ya));    // 8x8, slot B top
        upd(best[2], v10, !EDGE || (xA && yb));
        upd(best[3], v11, !EDGE || (xB && yb));
        upd(best[4], vt, !EDGE || (xa && ya));     // 16x8 top
        upd(best[5], vb, !EDGE || (xa && yb));     // 16x8 bottom
        upd(best[6], vl, !EDGE || (xA && ya));     // 8x16, slot A
        upd(best[7], vr, !EDGE || (xB && ya));     // 8x16, slot B
        upd(best[8], v16, !EDGE || (xa && ya));
    }

    if constexpr (NDY == 1) {
        // one candidate: every lane of a block's group forms the block's full sum
        const u32 q2 = q2s[0];
        const int dy = dy0;
        const bool ya = dy <= L.Y0, yp = dy <= L.Yp, yc = dy <= L.Yc;
        const u32 s32x16 = __shfl_xor_sync(0xFFFFFFFFu, s16[0], 1) * one + s16[0];
        const u32 s16x32 = __shfl_xor_sync(0xFFFFFFFFu, s16[0], 4) * one + s16[0];
        const u32 s32 = __shfl_xor_sync(0xFFFFFFFFu, s32x16, 4) * one + s32x16;
        const u32 s64x32 = __shfl_xor_sync(0xFFFFFFFFu, s32, 2) * one + s32;
        const u32 s32x64 = __shfl_xor_sync(0xFFFFFFFFu, s32, 8) * one + s32;
        const u32 s64 = __shfl_xor_sync(0xFFFFFFFFu, s64x32, 8) * one + s64x32;
        upd(best[9], s32x16 * mul + q2, !EDGE || (xp && ya));
        upd(best[10], s16x32 * mul + q2, !EDGE || (xa && yp));
        upd(best[11], s32 * mul + q2, !EDGE || (xp && yp));
        upd(best[12], s64x32 * mul + q2, !EDGE || (xc && yp));
        upd(best[13], s32x64 * mul + q2, !EDGE || (xp && yc));
        upd(best[14], s64 * mul + q2, !EDGE || (xc && yc));
    } else {
        // eight candidates: the lanes that share a larger block split the candidates between
        // them at each merge step (a lane keeps the half its bit selects and sends the other
        // half to its partner), so each lane folds only its share into the block's minimum
        static_assert(NDY == 8, "split merge of eight candidates");
        u32 h[4], v[4];   // 32x16 sums for j = 4*b0 + i, 16x32 sums for j = 4*b2 + i
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const u32 d = s16[i] * m1 + s16[i + 4];
            h[i] = __shfl_xor_sync(0xFFFFFFFFu, d * L.nb0 + s16[i], 1) * one + (d * L.b0 + s16[i]);
            v[i] = __shfl_xor_sync(0xFFFFFFFFu, d * L.nb2 + s16[i], 4) * one + (d * L.b2 + s16[i]);
        }
        const int jb = 4 * (int)L.b0 + 2 * (int)L.b2;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int jh = 4 * (int)L.b0 + i, jv = 4 * (int)L.b2 + i;
            upd(best[9], h[i] * mul + __ldg(q2p + jh), !EDGE || (xp && dy0 + jh <= L.Y0));
            upd(best[10], v[i] * mul + __ldg(q2p + jv), !EDGE || (xa && dy0 + jv <= L.Yp));
        }
        // 32x32 from the 32x16 sums of the pair below/above (same candidates), split on b2
        u32 q[2];
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const u32 d = h[i] * m1 + h[i + 2];
            q[i] = __shfl_xor_sync(0xFFFFFFFFu, d * L.nb2 + h[i], 4) * one + (d * L.b2 + h[i]);
            upd(best[11], q[i] * mul + __ldg(q2p + jb + i), !EDGE || (xp && dy0 + jb + i <= L.Yp));
        }
        // 64x32 (partner 32 samples to the side, split on b1), 32x64 (partner 32 rows away,
        // split on b3), 64x64 from the 64x32 sums (no split left)
        const u32 dq = q[0] * m1 + q[1];
        const u32 e = __shfl_xor_sync(0xFFFFFFFFu, dq * L.nb1 + q[0], 2) * one + (dq * L.b1 + q[0]);
        const u32 f = __shfl_xor_sync(0xFFFFFFFFu, dq * L.nb3 + q[0], 8) * one + (dq * L.b3 + q[0]);
        const u32 z = __shfl_xor_sync(0xFFFFFFFFu, e, 8) * one + e;
        const int je = jb + (int)L.b1, jf = jb + (int)L.b3;
        const u32 qe = __ldg(q2p + je);
        upd(best[12], e * mul + qe, !EDGE || (xc && dy0 + je <= L.Yp));
        upd(best[13], f * mul + __ldg(q2p + jf), !EDGE || (xp && dy0 + jf <= L.Yc));
        upd(best[14], z * mul + qe, !EDGE || (xc && dy0 + je <= L.Yc));
    }
}

// all items of one class against the window in shared memory
template <bool EDGE>
__device__ __forceinline__ void me_search_class(const MeIntParams &P, const u32 *win, const u32 (&o)[16][4],
                                                u32 (&best)[15], int cls, int off, int g, const MeLane &L)
{
    // item counts are multiples of ME_GROUPS: the trip counts are warp-uniform
    {
        const u32 *dsc = P.q2tab + P.d_main[cls], *q2b = P.q2tab + P.q2_main[cls];
        for (int it = g; it < P.n_main[cls]; it += ME_GROUPS)
            me_item<ME_NDY, EDGE>(P, win, o, best, __ldg(dsc + it), q2b + it * ME_NDY, cls, off, L);
    }
    {
        const u32 *dsc = P.q2tab + P.d_tail[cls], *q2b = P.q2tab + P.q2_tail[cls];
        for (int it = g; it < P.n_tail[cls]; it += ME_GROUPS)
            me_item<1, EDGE>(P, win, o, best, __ldg(dsc + it), q2b + it, cls, off, L);
    }
}

// Integer search: one CTA per (CTU, reference, class of dx mod 4).  Its window (rows cy + lo_y
// .., 224 bytes from a 16-byte boundary, of the reference plane shifted so that the class's
// candidate words are word-aligned) is staged by one TMA tensor copy, issued first so that it
// lands while the threads load their org sub-blocks; the two CTAs an SM holds overlap one's
// window load with the other's search.
template <bool EDGE>
__global__ void __launch_bounds__(256, 2) k_me_int(const __grid_constant__ MeIntParams P)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ unsigned long long skey[ME_BLOCKS_PER_CTU];
    __shared__ __align__(8) u64 bar;
    // the window starts on a 128-byte boundary (TMA destination); the launch reserves 128 bytes
    // of slack for this
    const u32 *win = reinterpret_cast<const u32 *>(smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u));
    const int tid = threadIdx.x;
    const u32 bar_a = smem_u32(&bar);

    const int ref = blockIdx.y, cls = blockIdx.z;
    int ccol, crow;
    ctu_of(P, blockIdx.x, EDGE, &ccol, &crow);
    const int ctu = crow * P.ctus_w + ccol;
    const int cx = ccol * ME_CTU, cy = crow * ME_CTU;
    const int gx = ME_SHIFT_PAD + cx + P.lo_x;            // first window column (padded coordinates)
    const int off = gx & 15;
    // the barrier is initialised and made visible to every thread before any thread polls it
    // and before the copy is issued: a poll of an uninitialised barrier could pass early and let
    // the CTA finish while its copy is still landing
    if (tid == 0) {
        mbar_init(bar_a, 1);
        mbar_fence_init();
    }
    for (int i = tid; i < ME_BLOCKS_PER_CTU; i += blockDim.x) skey[i] = ~0ull;
    __syncthreads();
    if (tid == 0) {
        mbar_arrive_expect_tx(bar_a, (u32)P.win_h * ME_WIN_BYTES_W);
        tma_load_2d(smem_u32(win), &P.maps[ref][(off + cls) & 3], gx - off, ME_SHIFT_PAD + cy + P.lo_y, bar_a);
    }

    const int lane = tid & 31, warp = tid >> 5;
    const int s = lane & 15, g = warp * 2 + (lane >> 4);
    MeLane L;
    L.sx = s & 3; L.sy = s >> 2;
    // multiplied by the run-time 1, the selectors stay opaque: d * b + x remains one IMAD
    L.b0 = (s & 1) * P.one; L.b1 = ((s >> 1) & 1) * P.one; L.b2 = ((s >> 2) & 1) * P.one; L.b3 = ((s >> 3) & 1) * P.one;
    L.nb0 = (1 - (s & 1)) * P.one; L.nb1 = (1 - ((s >> 1) & 1)) * P.one;
    L.nb2 = (1 - ((s >> 2) & 1)) * P.one; L.nb3 = (1 - ((s >> 3) & 1)) * P.one;
    // block-validity limits at the right/bottom picture edge (max_mv = pic - 1 - pos)
    L.X0 = P.W - 1 - (cx + 16 * L.sx); L.X1 = L.X0 - 8;
    L.Xp = P.W - 1 - (cx + 16 * (L.sx & 2)); L.Xc = P.W - 1 - cx;
    L.Y0 = P.H - 1 - (cy + 16 * L.sy); L.Y1 = L.Y0 - 8;
    L.Yp = P.H - 1 - (cy + 16 * (L.sy & 2)); L.Yc = P.H - 1 - cy;
    const bool swapped = L.sy >= 2;

    // org 16x16 sub-block in registers (reads clamped to the picture), words in the lane's
    // order: o[r][t] = org word t ^ sy of row r
    u32 o[16][4];
    {
        const int ox = cx + 16 * L.sx, oy = cy + 16 * L.sy;
#pragma unroll
        for (int r = 0; r < 16; r++) {
            const pel *orow = P.org + (long long)min(oy + r, P.H - 1) * P.i_org;
#pragma unroll
            for (int t = 0; t < 4; t++) {
                const int c0 = ox + 4 * (t ^ L.sy);
                u32 v = 0;
#pragma unroll
                for (int b = 0; b < 4; b++) v |= (u32)orow[min(c0 + b, P.W - 1)] << (8 * b);
                o[r][t] = v;
            }
        }
    }

    // the window (bounded wait; a CTA that gives up records it, waits for its copy once more
    // so that no copy lands in released shared memory, and leaves the keys untouched)
    const bool landed = mbar_wait_bounded(bar_a, 0, ME_TMA_POLLS);
    if (__syncthreads_or(!landed)) {
        if (tid == 0) atomicAnd(P.ctl + 1, 0u);
        mbar_wait_bounded(bar_a, 0, ME_TMA_POLLS);
        return;
    }

    u32 best[15];
#pragma unroll
    for (int i = 0; i < 15; i++) best[i] = 0xFFFFFFFFu;
    me_search_class<EDGE>(P, win, o, best, cls, off, g, L);

    // ---- decode the lane's winners and merge into the CTU's 64-bit keys.  The lanes that
    // share a block hold minima over disjoint (or repeated) candidates of the same lane group.
    {
        const int sx = L.sx, sy = L.sy;
        int ids[15];
#pragma unroll
        for (int i = 0; i < 2; i++)
#pragma unroll
            for (int j = 0; j < 2; j++) ids[j * 2 + i] = (2 * sy + j) * 8 + 2 * sx + (swapped ? 1 - i : i);
        ids[4] = 64 + (2 * sy) * 4 + sx;
        ids[5] = 64 + (2 * sy + 1) * 4 + sx;
        ids[6] = 96 + sy * 8 + 2 * sx + (swapped ? 1 : 0);
        ids[7] = 96 + sy * 8 + 2 * sx + (swapped ? 0 : 1);
        ids[8] = 128 + sy * 4 + sx;
        ids[9] = 144 + sy * 2 + (sx >> 1);
        ids[10] = 152 + (sy >> 1) * 4 + sx;
        ids[11] = 160 + (sy >> 1) * 2 + (sx >> 1);
        ids[12] = 164 + (sy >> 1);
        ids[13] = 166 + (sx >> 1);
        ids[14] = 168;
        const u16 *r2m = P.rank2mv + (cls * ME_GROUPS + g) * ME_MAX_GROUP;
#pragma unroll
        for (int i = 0; i < 15; i++) {
            const u32 b = best[i];
            if (b == 0xFFFFFFFFu) continue;
            const u32 raster = r2m[b & (ME_MAX_GROUP - 1)];
            const int dx = P.lo_x + (int)(raster % P.ndx), dy = P.lo_y + (int)(raster / P.ndx);
            const u32 mvc = (mvbits(4 * dx) + mvbits(4 * dy)) * P.lambda_mv;
            const u64 cost = ((u64)(b >> ME_RANK_BITS) << 16) + (mvc & 0xFFFFu);
            atomicMin(&skey[ids[i]], (unsigned long long)((cost << 15) | raster));
        }
    }
    __syncthreads();
    // the four alignment-class CTAs of this (CTU, reference) merge into keys preset to ~0
    u64 *dst = P.keys + ((size_t)ctu * P.n_refs + ref) * ME_BLOCKS_PER_CTU;
    for (int i = tid; i < ME_BLOCKS_PER_CTU; i += blockDim.x)
        if (skey[i] != ~0ull) atomicMin(reinterpret_cast<unsigned long long *>(dst + i), skey[i]);
}

// The four byte-shifted copies of each reference's integer plane that the integer search's TMA
// windows read: copy s of reference r holds, at padded position (x, y), the sample at
// (x - 144 + s, y - 144) of the reference's padded plane (0 beyond its right padding), with row
// pitch `pitch` (a multiple of 16) and H + 288 rows.  The source needs padding >= 144.  A thread
// writes one 16-byte chunk of every copy; sources on a 16-byte grid are read as two vectors.
__global__ void __launch_bounds__(256) k_shift_planes(MeShiftSrc S, pel *dst, int W, int H, int pitch)
{
    const int rows = H + 2 * ME_SHIFT_PAD;
    const int chunks = pitch >> 4;                   // 16-byte chunks per row
    const long long per_ref = (long long)rows * chunks;
    const long long total = per_ref * S.n_refs;
    const int xmax = W + ME_SHIFT_PAD;               // first source column past the padding
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int ref = (int)(i / per_ref);
        const long long rem = i - ref * per_ref;
        const int y = (int)(rem / chunks), c = (int)(rem - (long long)y * chunks);
        const pel *srow = S.plane[ref] + (long long)(y - ME_SHIFT_PAD) * S.stride;
        const int x0 = c * 16 - ME_SHIFT_PAD;        // source column of the chunk's first byte
        u32 b[5];                                    // source bytes x0 .. x0 + 19
        const pel *sp = srow + x0;
        if ((((uintptr_t)sp) & 15) == 0 && x0 + 32 <= xmax) {
            const uint4 v0 = *reinterpret_cast<const uint4 *>(sp);
            b[0] = v0.x; b[1] = v0.y; b[2] = v0.z; b[3] = v0.w;
            b[4] = *reinterpret_cast<const u32 *>(sp + 16);
        } else {
#pragma unroll
            for (int q = 0; q < 5; q++) {
                u32 v = 0;
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const int x = x0 + 4 * q + k;
                    v |= (x < xmax ? (u32)sp[4 * q + k] : 0u) << (8 * k);
                }
                b[q] = v;
            }
        }
        pel *d = dst + (size_t)ref * 4 * rows * pitch + (size_t)y * pitch + c * 16;
#pragma unroll
        for (int s = 0; s < 4; s++) {
            uint4 v;
            v.x = __funnelshift_r(b[0], b[1], 8 * s); v.y = __funnelshift_r(b[1], b[2], 8 * s);
            v.z = __funnelshift_r(b[2], b[3], 8 * s); v.w = __funnelshift_r(b[3], b[4], 8 * s);
            *reinterpret_cast<uint4 *>(d + (size_t)s * rows * pitch) = v;
        }
    }
}

int launch_shift_planes(const pel *const *planes, int n_refs, int i_ref, int W, int H, pel *dst, cudaStream_t st)
{
    if (n_refs < 1 || n_refs > ME_MAX_REFS || !dst) return set_status(UC_ERR_ARG, "shift_planes: bad argument");
    MeShiftSrc src;
    memset(&src, 0, sizeof(src));
    for (int r = 0; r < n_refs; r++) src.plane[r] = planes[r];
    src.stride = i_ref; src.n_refs = n_refs;
    const int pitch = (W + 2 * ME_SHIFT_PAD + 15) & ~15;
    const long long chunks = (long long)n_refs * (H + 2 * ME_SHIFT_PAD) * (pitch >> 4);
    prof_begin(PROF_SHIFT, st);
    k_shift_planes<<<(unsigned)std::min<long long>((chunks + 255) / 256, 152LL * 16), 256, 0, st>>>(src, dst, W, H,
                                                                                                   pitch);
    UC_CHECK(cudaGetLastError());
    count_launch(1);
    prof_end(PROF_SHIFT, st);
    return UC_OK;
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
    u64 k32, k128;       // had_scale_k of sq32, sq128
    const u64 *keys;
    u32 *satd1;          // [item][9]
    u32 *satd2;          // [item][8]
    u32 *hpel;           // [item]: stage-1 winner (mx, my)
    int cls_base[4], cls_nx[3];   // refinement items per tile class (per reference), tiles per row
    u32 cls_nx_inv[3];            // floor(2^32 / cls_nx) + 1 (nx > 1): r / nx = umulhi(r, inv) for r nx < 2^32
    const u32 *ctl;      // the integer search's control words ([1] != 0xFFFFFFFF: it gave up)
    MeResult *out;
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

// one row of 8 differences o - p (+ sgn * (o2 - p2) when o2), unpacked
__device__ __forceinline__ void diff_row8(const pel *o, const pel *p, const pel *o2, const pel *p2, int sgn, int (&v)[8])
{
    u32 ol, oh, pl, ph;
    load8(o, ol, oh);
    load8(p, pl, ph);
#pragma unroll
    for (int c = 0; c < 4; c++) {
        v[c] = (int)__byte_perm(ol, 0u, 0x4440 + c) - (int)__byte_perm(pl, 0u, 0x4440 + c);
        v[c + 4] = (int)__byte_perm(oh, 0u, 0x4440 + c) - (int)__byte_perm(ph, 0u, 0x4440 + c);
    }
    if (o2) {
        load8(o2, ol, oh);
        load8(p2, pl, ph);
#pragma unroll
        for (int c = 0; c < 4; c++) {
            v[c] += sgn * ((int)__byte_perm(ol, 0u, 0x4440 + c) - (int)__byte_perm(pl, 0u, 0x4440 + c));
            v[c + 4] += sgn * ((int)__byte_perm(oh, 0u, 0x4440 + c) - (int)__byte_perm(ph, 0u, 0x4440 + c));
        }
    }
}

// magnitude sum of the 2-D WHT of the 8x8 difference org - pred; with o2/p2 the second 8x8
// half of a 16x8 / 8x16 tile is folded in as first + sgn * second (the first stage of the
// 16-point transform).  Columns c and c + 2 of a row travel packed in one register as
// d[c+2] * 2^16 + d[c] (PRMT spreads the two bytes of a word into 16-bit lanes, and one 32-bit
// subtract of the packed org and prediction gives both differences exactly; every value stays
// below 2^15 in magnitude, so integer adds and subtracts keep both halves exact).  The WHT's
// stages commute, so the row stages of distance 1 and 4 and all column stages run on the packed
// pairs, and the row stage of distance 2 -- the one between the two halves -- is left to the
// end, where |lo + hi| + |lo - hi| = 2 max(|lo|, |hi|).
__device__ __noinline__ int satd8x8_raw(const pel *o, int io, const pel *p, int ip, const pel *o2, const pel *p2,
                                           int sgn)
{
    int Q[8][4];
#pragma unroll
    for (int r = 0; r < 8; r++) {
        u32 ol, oh, pl, ph;
        load8(o + r * io, ol, oh);
        load8(p + r * ip, pl, ph);
        int q0 = (int)(__byte_perm(ol, 0u, 0x4240) - __byte_perm(pl, 0u, 0x4240));   // columns 0, 2
        int q1 = (int)(__byte_perm(ol, 0u, 0x4341) - __byte_perm(pl, 0u, 0x4341));   // columns 1, 3
        int q2 = (int)(__byte_perm(oh, 0u, 0x4240) - __byte_perm(ph, 0u, 0x4240));   // columns 4, 6
        int q3 = (int)(__byte_perm(oh, 0u, 0x4341) - __byte_perm(ph, 0u, 0x4341));   // columns 5, 7
        if (o2) {
            load8(o2 + r * io, ol, oh);
            load8(p2 + r * ip, pl, ph);
            const int e0 = (int)(__byte_perm(ol, 0u, 0x4240) - __byte_perm(pl, 0u, 0x4240));
            const int e1 = (int)(__byte_perm(ol, 0u, 0x4341) - __byte_perm(pl, 0u, 0x4341));
            const int e2 = (int)(__byte_perm(oh, 0u, 0x4240) - __byte_perm(ph, 0u, 0x4240));
            const int e3 = (int)(__byte_perm(oh, 0u, 0x4341) - __byte_perm(ph, 0u, 0x4341));
            if (sgn > 0) { q0 += e0; q1 += e1; q2 += e2; q3 += e3; }
            else { q0 -= e0; q1 -= e1; q2 -= e2; q3 -= e3; }
        }
        // row stages of distance 1 (words 0/1, 2/3) and 4 (words 0/2, 1/3)
        const int a = q0 + q1, b = q0 - q1, c = q2 + q3, d = q2 - q3;
        Q[r][0] = a + c; Q[r][2] = a - c; Q[r][1] = b + d; Q[r][3] = b - d;
    }
    int s = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        int v[8];
#pragma unroll
        for (int r = 0; r < 8; r++) v[r] = Q[r][k];
        wht<8>(v);
#pragma unroll
        for (int r = 0; r < 8; r++) {
            const int lo = (int)(short)(v[r] & 0xFFFF), hi = (v[r] - lo) >> 16;
            s += max(abs(lo), abs(hi));
        }
    }
    return 2 * s;
}

// Refinement work items: one per (reference, com_had tile position, tile class).  The tile
// classes are 8x8 (tiles of the square blocks 8x8 .. 64x64), 16x8 (16x8, 32x16, 64x32) and 8x16
// (8x16, 16x32, 32x64); a tile of a class lies in exactly one block of each of the class's
// shapes (4 or 3 nested blocks).  A thread takes one (item, candidate): it forms the candidate's
// prediction pointer for every nested block, evaluates the tile SATD once per distinct
// pointer (nested blocks that share the integer or half-sample winner share the prediction)
// and adds it to each block's sum for that candidate.
__constant__ s8 kClassShapes[3][4] = { { 0, 3, 6, 9 }, { 1, 4, 7, -1 }, { 2, 5, 8, -1 } };

struct SubItem {
    int ref, cls, px, py, tw, th, nb;
    int bx[4], by[4], ctu[4], b[4], item[4];
    bool ok[4];
};

__device__ __forceinline__ void decode_sub_item(const MeSubParams &P, int it, SubItem &I)
{
    // two references (the usual case) by a shift
    I.ref = P.n_refs == 2 ? (it & 1) : it % P.n_refs;
    int rest = P.n_refs == 2 ? (it >> 1) : it / P.n_refs;
    int c = 0;
    while (c < 2 && rest >= P.cls_base[c + 1]) c++;
    rest -= P.cls_base[c];
    I.cls = c;
    I.tw = c == 1 ? 16 : 8; I.th = c == 2 ? 16 : 8;
    const int nx = P.cls_nx[c];
    const int ry = nx > 1 ? (int)__umulhi((u32)rest, P.cls_nx_inv[c]) : rest;
    I.px = (rest - ry * nx) * I.tw; I.py = ry * I.th;
    I.nb = c == 0 ? 4 : 3;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        I.ok[j] = false; I.item[j] = 0; I.bx[j] = 0; I.by[j] = 0; I.ctu[j] = 0; I.b[j] = 0;
        if (j >= I.nb) continue;
        const int sh = kClassShapes[c][j];
        // block sides are powers of two: positions within the CTU by shifts (a division by a
        // table value would compile to a full integer division)
        const int w = kShapeWH[sh][0], h = kShapeWH[sh][1];
        const int lw = 31 - __clz(w), lh = 31 - __clz(h);
        const int bx = I.px & ~(w - 1), by = I.py & ~(h - 1);
        const int ctu = (by >> 6) * P.ctus_w + (bx >> 6);
        const int b = kShapeFirst[sh] + (((by & 63) >> lh) << (6 - lw)) + ((bx & 63) >> lw);
        I.bx[j] = bx; I.by[j] = by; I.ctu[j] = ctu; I.b[j] = b;
        I.item[j] = (ctu * ME_BLOCKS_PER_CTU + b) * P.n_refs + I.ref;
        I.ok[j] = bx + w <= P.W && by + h <= P.H;
    }
}

// com_had tile SATD of the item's tile against prediction pb.  For 16x8 (8x16) the 16-point
// transform's first stage forms left+right and left-right (top+bottom, top-bottom); the
// magnitude sum is the sum of the two 8x8 transforms of those.
__device__ __forceinline__ u32 sub_tile_satd(const MeSubParams &P, const SubItem &I, const pel *pb)
{
    const pel *ob = P.org + (long long)I.py * P.i_org + I.px;
    if (I.cls == 0) return (u32)((satd8x8_raw(ob, P.i_org, pb, P.i_ref, nullptr, nullptr, 0) + 2) >> 2);
    const int bo = I.cls == 1 ? 8 : 8 * P.i_org, bp = I.cls == 1 ? 8 : 8 * P.i_ref;
    int s = satd8x8_raw(ob, P.i_org, pb, P.i_ref, ob + bo, pb + bp, 1);
    s += satd8x8_raw(ob, P.i_org, pb, P.i_ref, ob + bo, pb + bp, -1);
    return had_scale(s, P.sq128, P.k128);
}

template <int STAGE>
__global__ void __launch_bounds__(256, 3) k_me_sub_eval(MeSubParams P, int n_threads)
{
    constexpr int NC = STAGE == 1 ? 9 : 8;
    // candidate-major order: consecutive threads take consecutive tiles with the same candidate,
    // so the tiles of one block (sharing its winner, hence its plane and offset) read adjacent
    // columns of the same rows
    const int n_items = n_threads / NC;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n_threads; t += gridDim.x * blockDim.x) {
        const int c = t / n_items, it = t - c * n_items;
        SubItem I;
        decode_sub_item(P, it, I);
        const pel *ptr[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            ptr[j] = nullptr;
            if (!I.ok[j]) continue;
            const long long toff = (long long)(I.py - I.by[j]) * P.i_ref + (I.px - I.bx[j]);
            if (STAGE == 1) {
                int dx, dy;
                u64 key;
                int_winner(P, I.ctu[j], I.b[j], I.ref, dx, dy, key);
                if (c == 0) ptr[j] = P.planes[I.ref][0] + (long long)(I.by[j] + dy) * P.i_ref + (I.bx[j] + dx) + toff;
                else ptr[j] = mc_ptr(P, I.ref, I.bx[j], I.by[j], 4 * dx + kHalfPat[c - 1][0], 4 * dy + kHalfPat[c - 1][1]) + toff;
            } else {
                const u32 hp = P.hpel[I.item[j]];
                const int mx = (int)(s16)(hp & 0xFFFF), my = (int)(s16)(hp >> 16);
                ptr[j] = mc_ptr(P, I.ref, I.bx[j], I.by[j], mx + kQuarPat[c][0], my + kQuarPat[c][1]) + toff;
            }
        }
        u32 val[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            val[j] = 0;
            if (!I.ok[j]) continue;
            int same = -1;
#pragma unroll
            for (int i = 0; i < j; i++)
                if (same < 0 && I.ok[i] && ptr[i] == ptr[j]) same = i;
            u32 v = 0;
#pragma unroll
            for (int i = 0; i < j; i++)
                if (i == same) v = val[i];
            if (same < 0) v = sub_tile_satd(P, I, ptr[j]);
            val[j] = v;
            atomicAdd((STAGE == 1 ? P.satd1 + (size_t)I.item[j] * 9 : P.satd2 + (size_t)I.item[j] * 8) + c, v);
        }
    }
}

// stage-1 winner of every (block, reference): (mx, my) packed as two s16
__global__ void __launch_bounds__(256) k_me_sub_pick(MeSubParams P)
{
    const long long total = (long long)P.n_ctu * ME_BLOCKS_PER_CTU * P.n_refs;
    for (long long item = blockIdx.x * (long long)blockDim.x + threadIdx.x; item < total;
         item += (long long)gridDim.x * blockDim.x) {
        const int ref = (int)(item % P.n_refs);
        const int b = (int)((item / P.n_refs) % ME_BLOCKS_PER_CTU);
        const int ctu = (int)(item / P.n_refs / ME_BLOCKS_PER_CTU);
        int dx, dy;
        u64 key;
        int_winner(P, ctu, b, ref, dx, dy, key);
        int mx, my; u64 cb; u32 bs;
        hpel_winner(P, (int)item, dx * 4, dy * 4, mx, my, cb, bs);
        P.hpel[item] = ((u32)(u16)(s16)my << 16) | (u16)(s16)mx;
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
        // a search that gave up waiting for a window leaves no result: every record is marked
        // invalid rather than filled from incomplete keys
        if (x + cb.w > P.W || y + cb.h > P.H || P.ctl[1] != 0xFFFFFFFFu) {
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

// one-time per-device setup of the frame search (block table upload, shared-memory limits);
// synchronous, so it runs before a frame is captured into a graph
int me_frame_once()
{
    int dev = 0;
    UC_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return UC_OK;
    if (!g_ctu_tab_uploaded[dev]) {
        CtuBlock tab[ME_BLOCKS_PER_CTU];
        ctu_block_table(tab);
        UC_CHECK(cudaMemcpyToSymbol(kCtuBlocks, tab, sizeof(tab)));
        g_ctu_tab_uploaded[dev] = true;
    }
    static bool attr_set[64];
    if (!attr_set[dev]) {
        UC_CHECK(cudaFuncSetAttribute(k_me_int<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
        UC_CHECK(cudaFuncSetAttribute(k_me_int<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
        attr_set[dev] = true;
    }
    return UC_OK;
}

int launch_me_frame(const MeFrameArgs &a, const MeTables &t, u64 *keys, cudaStream_t st)
{
    int rc = me_frame_once();
    if (rc) return rc;
    const int ctus_w = (a.W + 63) / 64, ctus_h = (a.H + 63) / 64;
    MeIntParams P;
    memset(&P, 0, sizeof(P));
    P.org = a.org; P.i_org = a.i_org;
    P.W = a.W; P.H = a.H; P.ctus_w = ctus_w; P.ctus_h = ctus_h;
    P.lo_x = t.lo_x; P.hi_x = t.hi_x; P.lo_y = t.lo_y; P.hi_y = t.hi_y;
    P.ndx = t.ndx; P.lambda_mv = a.lambda_mv;
    for (int c = 0; c < ME_CLASSES; c++) {
        P.n_main[c] = t.n_main[c]; P.n_tail[c] = t.n_tail[c];
        P.q2_main[c] = t.q2_main[c]; P.q2_tail[c] = t.q2_tail[c];
        P.d_main[c] = t.d_main[c]; P.d_tail[c] = t.d_tail[c];
    }
    P.mul = 1u << ME_RANK_BITS; P.one = 1u; P.minus1 = 0xFFFFFFFFu;
    P.q2tab = a.q2tab; P.rank2mv = a.rank2mv; P.keys = keys; P.n_refs = a.n_refs;
    const size_t n_keys = (size_t)ctus_w * ctus_h * a.n_refs * ME_BLOCKS_PER_CTU;
    P.ctl = reinterpret_cast<u32 *>(keys + n_keys);
    if (t.ndy_per_item != ME_NDY) return set_status(UC_ERR_ARG, "me: table built for another NDY");
    if (a.pad < ME_SHIFT_PAD || !a.shift_scratch) return set_status(UC_ERR_ARG, "me: padding below 144 or no scratch");
    // rows read: main items up to 48 + 8 (nfull - 1) + 22, tail items up to 48 + ndy - 1 + 15
    P.win_h = t.ndy + 63;
    const int win_cols = ((15 + 64 + t.ndx + 4 + 15) / 16) * 16;
    if (win_cols > ME_WIN_BYTES_W || P.win_h > 256) return set_status(UC_ERR_ARG, "me: window too large");
    const size_t smem = (size_t)P.win_h * ME_WIN_BYTES_W + 128;
    if (smem > 100 * 1024) return set_status(UC_ERR_ARG, "me: window too large");
    // interior CTUs: every 8x8 tile satisfies pos + 8 + hi <= pic - 1 in both directions
    int nx = a.W - 57 - t.hi_x >= 0 ? (a.W - 57 - t.hi_x) / 64 + 1 : 0;
    int ny = a.H - 57 - t.hi_y >= 0 ? (a.H - 57 - t.hi_y) / 64 + 1 : 0;
    nx = std::min(nx, ctus_w); ny = std::min(ny, ctus_h);
    if (t.nfull == 0) nx = ny = 0;   // the interior path has no row limit: short ranges go to the edge path
    P.nx_int = nx; P.ny_int = ny;

    // the byte-shifted reference copies the windows are read from (made here unless the caller
    // keeps them current), and their tensor maps
    const size_t pitch = ((size_t)a.W + 2 * ME_SHIFT_PAD + 15) & ~(size_t)15;
    const size_t rows = (size_t)a.H + 2 * ME_SHIFT_PAD;
    for (int r = 0; r < a.n_refs; r++)
        for (int sft = 0; sft < 4; sft++) {
            const pel *base = a.shift_scratch + ((size_t)r * 4 + sft) * rows * pitch;
            int e = encode_tensor_map_u8(&P.maps[r][sft], base, pitch, rows, pitch, ME_WIN_BYTES_W, (u32)P.win_h);
            if (e) return e;
        }
    if (!a.shift_ready) {
        const pel *src[ME_MAX_REFS];
        for (int r = 0; r < a.n_refs; r++) src[r] = a.planes[r][0];
        int e = launch_shift_planes(src, a.n_refs, a.i_ref, a.W, a.H, a.shift_scratch, st);
        if (e) return e;
    }
    prof_begin(PROF_ME_INT, st);
    UC_CHECK(cudaMemsetAsync(keys, 0xFF, n_keys * sizeof(u64) + 2 * sizeof(u32), st));
    if (nx * ny > 0) {
        k_me_int<false><<<dim3(nx * ny, a.n_refs, ME_CLASSES), 256, smem, st>>>(P);
        UC_CHECK(cudaGetLastError());
        count_launch(1);
    }
    const int n_edge = ctus_w * ctus_h - nx * ny;
    if (n_edge > 0) {
        k_me_int<true><<<dim3(n_edge, a.n_refs, ME_CLASSES), 256, smem, st>>>(P);
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
    S.k32 = had_scale_k(S.sq32); S.k128 = had_scale_k(S.sq128);
    S.keys = keys; S.out = a.out; S.ctl = P.ctl;
    const long long items = (long long)S.n_ctu * ME_BLOCKS_PER_CTU * a.n_refs;
    S.satd1 = a.sub_scratch;
    S.satd2 = a.sub_scratch + items * 9;
    // refinement items: per reference, every tile position of the three tile classes
    const int cnx[3] = { (a.W + 7) / 8, (a.W + 15) / 16, (a.W + 7) / 8 };
    const int cny[3] = { (a.H + 7) / 8, (a.H + 7) / 8, (a.H + 15) / 16 };
    S.cls_base[0] = 0;
    for (int c = 0; c < 3; c++) {
        S.cls_nx[c] = cnx[c];
        S.cls_nx_inv[c] = cnx[c] > 1 ? (u32)((1ull << 32) / (unsigned long long)cnx[c] + 1) : 0u;   // nx = 1: ry = r
        S.cls_base[c + 1] = S.cls_base[c] + cnx[c] * cny[c];
    }
    const long long n_items = (long long)S.cls_base[3] * a.n_refs;
    if (n_items * 9 >= (1ll << 31)) return set_status(UC_ERR_ARG, "me: frame too large for the refinement grid");
    S.hpel = a.sub_scratch + items * 17;
    UC_CHECK(cudaMemsetAsync(a.sub_scratch, 0, (size_t)items * 17 * sizeof(u32), st));
    prof_begin(PROF_ME_SUB, st);
    const int n1 = (int)(n_items * 9), n2 = (int)(n_items * 8);
    k_me_sub_eval<1><<<(unsigned)std::min<long long>((n1 + 255) / 256, 152 * 32), 256, 0, st>>>(S, n1);
    UC_CHECK(cudaGetLastError());
    k_me_sub_pick<<<(unsigned)std::min<long long>((items + 255) / 256, 152 * 16), 256, 0, st>>>(S);
    UC_CHECK(cudaGetLastError());
    k_me_sub_eval<2><<<(unsigned)std::min<long long>((n2 + 255) / 256, 152 * 32), 256, 0, st>>>(S, n2);
    UC_CHECK(cudaGetLastError());
    k_me_sub_final<<<(unsigned)std::min<long long>((items + 255) / 256, 152 * 16), 256, 0, st>>>(S);
    UC_CHECK(cudaGetLastError());
    count_launch(4);
    prof_end(PROF_ME_SUB, st);
    return UC_OK;
}

}  // namespace uc
