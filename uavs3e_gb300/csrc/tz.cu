// Per-call motion search of the encoder, batched: me_search_tz (src/me.c:529-568) for a list of
// independent calls (block, reference, predictor, MV resolution, bi-prediction state), each
// bit-exact with the reference's call on the same state.
//
// One warp per call.  The org block (or, for a bi call, 2 org - the other list's prediction,
// create_bi_org src/inter.c:55) sits in shared memory.  The search's stages run one after the
// other -- first diamond, raster grids, refinement diamond (search_diamond :199, search_raster
// :103, get_raster_range :65) -- and each stage's candidates, in the reference's visit order,
// are costed 32 at a time (a 16..64-sample-wide SAD per lane); the stage keeps the minimum of
// (cost << 20 | visit position) and moves the running best only when that minimum is strictly
// smaller, as the reference's sequence of strict updates does.  The fractional refinement
// (me_sub_pel_search :366-500) costs its centre and 8 half-sample points in one batch, then 8
// quarter-sample points, with the rows of the com_had tiles spread over the lanes (columns
// transformed through shuffles; per-lane SADs for subpel_cost_type 1), and compares them in the
// reference's order.
#include "common.cuh"
#include "uavs3e_cuda_internal.h"
#include "../../include/uavs3e_cuda.h"

#include <algorithm>
#include <math.h>
#include <string.h>

namespace uc {

constexpr int TZ_WARPS = 1;
constexpr int TZ_KEY_BITS = 20;

struct TzReq {
    s16 x, y; u8 w, h; u8 ref_slot; s8 refi; u8 num_refp; u8 mvr; u8 bi; u8 flags;
    s16 mvp[2]; s16 mv[2]; s16 mv_ipel[2]; s16 other_mv[2]; u8 other_slot; u8 pad0[3];
    s32 mot_bits_other; u32 lambda_mv; s32 dist; s32 pad1;
};
struct TzOut { s16 mv[2]; s16 mv_ipel[2]; u64 cost; };
static_assert(sizeof(TzReq) == sizeof(uavs3e_cuda_tz_req_t), "request layout");
static_assert(sizeof(TzOut) == sizeof(uavs3e_cuda_tz_out_t), "result layout");

struct TzParams {
    const pel *planes[UAVS3E_CUDA_TZ_MAX_SLOTS * 16];   // sample (0,0) of each slot's 16 planes
    const pel *org;
    int i_org, i_ref, n_slots;
    int W, H, is_padding, max_search_range, gop_size, mto;
    const TzReq *reqs;
    int n;
    TzOut *out;
    double sq32, sq128;
    u64 k32, k128;       // had_scale_k of sq32, sq128
};

// search_diamond's ring points (src/me.c:307-331) at MV resolution <= integer: step 4, 8, 16
__device__ __constant__ static const s8 kTzRing[28][3] = {
    { -4, 0, 4 }, { 0, 4, 4 }, { 4, 0, 4 }, { 0, -4, 4 },
    { -8, 0, 8 }, { -4, 4, 8 }, { 0, 8, 8 }, { 4, 4, 8 }, { 8, 0, 8 }, { 4, -4, 8 }, { 0, -8, 8 }, { -4, -4, 8 },
    { -16, 0, 16 }, { -12, 4, 16 }, { -8, 8, 16 }, { -4, 12, 16 }, { 0, 16, 16 }, { 4, 12, 16 }, { 8, 8, 16 },
    { 12, 4, 16 }, { 16, 0, 16 }, { 12, -4, 16 }, { 8, -8, 16 }, { 4, -12, 16 }, { 0, -16, 16 }, { -4, -12, 16 },
    { -8, -8, 16 }, { -12, -4, 16 },
};
// me_sub_pel_search's patterns (src/me.c:413-415, :451-453)
__device__ __constant__ static const s8 kTzHalf[8][2] = { { -2, 0 }, { -2, 2 }, { 0, 2 }, { 2, 2 },
                                                         { 2, 0 }, { 2, -2 }, { 0, -2 }, { -2, -2 } };
__device__ __constant__ static const s8 kTzQuar[8][2] = { { -1, 0 }, { 0, 1 }, { 1, 0 }, { 0, -1 },
                                                         { -1, 1 }, { 1, 1 }, { -1, -1 }, { 1, -1 } };

// MV bits at table index v (inter_search_create, src/inter.c:2029-2057)
__device__ __forceinline__ u32 tz_bits(int v)
{
    return v == 0 ? 1u : 2u * (32u - (u32)__clz(abs(v) + 1));
}

struct TzS {
    const u32 *so;          // org block (smem), wq words per row
    int wq, w, h;
    const pel *ref;         // integer plane at the block origin
    int stride;
    int minx, maxx, miny, maxy;
    int mvr, shift;         // shift = 16 - bi
    int bpx, bpy;           // predictor at the MV-bits table's resolution (mvp >> mvr)
    u32 lambda;
    u64 best;
    int mvx, mvy;
};

// w x h SAD of the org block against p (stride a multiple of 4)
__device__ __forceinline__ u32 tz_sad(const TzS &S, const pel *p)
{
    const uintptr_t a = (uintptr_t)p;
    const u32 *wp = (const u32 *)(a & ~(uintptr_t)3);
    const u32 sh = (u32)(a & 3) * 8;
    const int ws = S.stride >> 2;
    u32 s = 0;
    for (int r = 0; r < S.h; r++) {
        const u32 *q = wp + r * ws;
        const u32 *o = S.so + r * S.wq;
        u32 prev = __ldg(q);
        for (int k = 0; k < S.wq; k++) {
            const u32 next = __ldg(q + k + 1);
            s = sad4(o[k], __funnelshift_r(prev, next, sh), s);
            prev = next;
        }
    }
    return s;
}

// integer-MV cost of search_diamond / search_raster: (SAD << shift) + bits * lambda (u32 product)
__device__ __forceinline__ u64 tz_cost(const TzS &S, int mx, int my)
{
    const u32 sad = tz_sad(S, S.ref + my * S.stride + mx);
    const u32 bits = tz_bits(((mx * 4) >> S.mvr) - S.bpx) + tz_bits(((my * 4) >> S.mvr) - S.bpy);
    return ((u64)sad << S.shift) + (u64)(bits * S.lambda);
}

__device__ __forceinline__ u64 tz_key(u64 cost, int k) { return (cost << TZ_KEY_BITS) | (u64)k; }

// search_diamond (src/me.c:199-334): centre, core square, and (not bi) rings below max_step.
// Returns best_step.
__device__ int tz_diamond(TzS &S, int max_step, int bi, int mvpx, int mvpy, int lane)
{
    const int cx = S.mvx, cy = S.mvy;
    int core = bi ? 5 : 2, cstep = 1;
    if (bi) {
        if (S.mvr > 2) core++;
        const int ix = (mvpx + 2) >> 2, iy = (mvpy + 2) >> 2;
        const int diff = max(abs(ix - cx), abs(iy - cy)) >> max(0, S.mvr - 2);
        core = min(max(diff, 2), core);
    }
    if (S.mvr > 2) { core <<= S.mvr - 2; cstep <<= S.mvr - 2; }
    int x0 = cx - core, y0 = cy - core, x1 = cx + core, y1 = cy + core;
    while (x0 <= S.minx) x0 += cstep;
    while (y0 <= S.miny) y0 += cstep;
    while (x1 >= S.maxx) x1 -= cstep;
    while (y1 >= S.maxy) y1 -= cstep;
    const int ncx = x1 >= x0 ? (x1 - x0) / cstep + 1 : 0, ncy = y1 >= y0 ? (y1 - y0) / cstep + 1 : 0;
    const int ncore = ncx * ncy;
    const int n_ring = bi ? 0 : (max_step > 16 ? 28 : max_step > 8 ? 12 : max_step > 4 ? 4 : 0);
    const int msh = max(S.mvr - 2, 0);
    const int n = 1 + ncore + n_ring;
    u64 kmin = ~0ull;
    for (int base = 0; base < n; base += 32) {
        const int k = base + lane;
        if (k >= n) continue;
        int mx, my;
        if (k == 0) { mx = cx; my = cy; }
        else if (k <= ncore) { mx = x0 + ((k - 1) % ncx) * cstep; my = y0 + ((k - 1) / ncx) * cstep; }
        else {
            const int j = k - 1 - ncore;
            mx = cx + (kTzRing[j][0] << msh); my = cy + (kTzRing[j][1] << msh);
            if (mx < S.minx || mx > S.maxx || my < S.miny || my > S.maxy) continue;
        }
        const u64 key = tz_key(tz_cost(S, mx, my), k);
        kmin = key < kmin ? key : kmin;
    }
    kmin = warp_min_u64(kmin);
    int step = -1;
    if (kmin != ~0ull && (kmin >> TZ_KEY_BITS) < S.best) {
        const int k = (int)(kmin & ((1u << TZ_KEY_BITS) - 1));
        S.best = kmin >> TZ_KEY_BITS;
        if (k == 0) { S.mvx = cx; S.mvy = cy; }
        else if (k <= ncore) { S.mvx = x0 + ((k - 1) % ncx) * cstep; S.mvy = y0 + ((k - 1) / ncx) * cstep; }
        else {
            const int j = k - 1 - ncore;
            S.mvx = cx + (kTzRing[j][0] << msh); S.mvy = cy + (kTzRing[j][1] << msh);
            step = kTzRing[j][2];
        }
    }
    if (step < 0) step = (S.mvx != cx || S.mvy != cy) ? 2 : 0;
    return step;
}

// one grid of search_raster: [x0, x1] x [y0, y1] in steps of s, rows outer
__device__ void tz_grid(TzS &S, int x0, int x1, int y0, int y1, int s, int lane)
{
    const int nx = (x1 - x0) / s + 1, ny = (y1 - y0) / s + 1, n = nx * ny;
    u64 kmin = ~0ull;
    for (int base = 0; base < n; base += 32) {
        const int k = base + lane;
        if (k >= n) continue;
        const u64 key = tz_key(tz_cost(S, x0 + (k % nx) * s, y0 + (k / nx) * s), k);
        kmin = key < kmin ? key : kmin;
    }
    kmin = warp_min_u64(kmin);
    if ((kmin >> TZ_KEY_BITS) < S.best) {
        const int k = (int)(kmin & ((1u << TZ_KEY_BITS) - 1));
        S.best = kmin >> TZ_KEY_BITS;
        S.mvx = x0 + (k % nx) * s;
        S.mvy = y0 + (k / nx) * s;
    }
}

// search_raster with get_raster_range (src/me.c:65-197)
__device__ void tz_raster(TzS &S, const TzReq &q, const TzParams &P, int lane)
{
    const int base[5] = { 5, 5, 5, 6, 8 }, smin[5] = { 1, 1, 1, 2, 4 };
    const int mvr = S.mvr;
    int step = max(base[mvr], min(S.w >> 1, S.h >> 1)) * (q.refi + 1);
    const int max_sr = P.max_search_range >> max(3 - mvr, 0);
    const int rxy = min(max((max_sr * q.dist + (P.gop_size >> 1)) / P.gop_size, max_sr >> 2), max_sr);
    int rx = rxy, ry = rxy;
    if (mvr && (q.flags & 2)) {
        rx = min(max(max(abs(q.mv_ipel[0] - S.mvx) * 4, max_sr >> 2), step * 8), rxy);
        ry = min(max(max(abs(q.mv_ipel[1] - S.mvy) * 2, max_sr >> 2), step * 4), rxy);
    }
    if (mvr > 2) { rx = (rx >> (mvr - 2)) << (mvr - 2); ry = (ry >> (mvr - 2)) << (mvr - 2); }
    int x0 = min(max(S.mvx - rx, S.minx), S.maxx), x1 = min(max(S.mvx + rx, S.minx), S.maxx);
    int y0 = min(max(S.mvy - ry, S.miny), S.maxy), y1 = min(max(S.mvy + ry, S.miny), S.maxy);
    for (int round = 0; step >= smin[mvr]; round++) {
        if (round) {
            x0 = max(S.mvx - step, S.minx); x1 = min(S.mvx + step, S.maxx);
            y0 = max(S.mvy - step, S.miny); y1 = min(S.mvy + step, S.maxy);
        }
        tz_grid(S, x0, x1, y0, y1, step, lane);
        step >>= 1;
        if (mvr > 2) step = (step >> (mvr - 2)) << (mvr - 2);
    }
}

// com_mc_blk_luma_pointer (src/com_mc.c:89-101) into a slot's planes
__device__ __forceinline__ const pel *tz_mc_ptr(const TzParams &P, int slot, int qx, int qy)
{
    const int px = min(max(qx >> 2, -128 - 4), P.W + 4), py = min(max(qy >> 2, -128 - 4), P.H + 4);
    return P.planes[slot * 16 + (qy & 3) * 4 + (qx & 3)] + (long long)py * P.i_ref + px;
}

// candidate k of a refinement batch: pattern 0 = centre + the 8 half-sample points, 1 = the 8
// quarter-sample points, 2 = the centre alone
__device__ __forceinline__ void tz_sub_mv(int pattern, int k, int cx, int cy, int &vx, int &vy)
{
    if (pattern == 1) { vx = cx + kTzQuar[k][0]; vy = cy + kTzQuar[k][1]; }
    else if (pattern == 0 && k > 0) { vx = cx + kTzHalf[k - 1][0]; vy = cy + kTzHalf[k - 1][1]; }
    else { vx = cx; vy = cy; }
}

// com_had of nc refinement candidates, tiles spread over the warp as (candidate, tile, row) tasks
template <int TW, int TH>
__device__ void tz_had_batch(const TzS &S, const TzParams &P, int slot, int bx, int by, int pattern, int cx, int cy,
                             int nc, u32 *sum, int lane)
{
    const int ntx = S.w / TW, nt = ntx * (S.h / TH), total = nc * nt * TH;
    const pel *ob = (const pel *)S.so;
    for (int base = 0; base < total; base += 32) {
        const int t = base + lane;
        const bool active = t < total;
        const int tt = active ? t : 0;
        const int k = tt / (nt * TH), rem = tt - k * nt * TH, tile = rem / TH, row = rem - tile * TH;
        const int ox = (tile % ntx) * TW, oy = (tile / ntx) * TH + row;
        int vx, vy;
        tz_sub_mv(pattern, k, cx, cy, vx, vy);
        const pel *p = tz_mc_ptr(P, slot, bx + vx, by + vy) + oy * P.i_ref + ox;
        const u32 v = had_tile_rows<TW, TH>(ob + oy * S.w + ox, S.w, p, P.i_ref, active, lane, P.sq32, P.sq128,
                                             P.k32, P.k128);
        if (active && row == 0) atomicAdd(&sum[k], v);
    }
}

// costs (com_had, or SAD when sad) of the nc candidates of a refinement batch into sum[k]; every
// lane returns with sum[] complete
__device__ void tz_sub_costs(const TzS &S, const TzParams &P, int slot, int bx, int by, int pattern, int cx, int cy,
                             int nc, bool sad, u32 *sum, int lane)
{
    if (lane < 9) sum[lane] = 0;
    __syncwarp();
    if (sad) {
        if (lane < nc) {
            int vx, vy;
            tz_sub_mv(pattern, lane, cx, cy, vx, vy);
            sum[lane] = tz_sad(S, tz_mc_ptr(P, slot, bx + vx, by + vy));
        }
    } else {
        int tw, th;
        had_tile_shape(S.w, S.h, &tw, &th);
        if (tw == 8 && th == 8) tz_had_batch<8, 8>(S, P, slot, bx, by, pattern, cx, cy, nc, sum, lane);
        else if (tw == 4 && th == 4) tz_had_batch<4, 4>(S, P, slot, bx, by, pattern, cx, cy, nc, sum, lane);
        else if (tw == 16) tz_had_batch<16, 8>(S, P, slot, bx, by, pattern, cx, cy, nc, sum, lane);
        else if (th == 16) tz_had_batch<8, 16>(S, P, slot, bx, by, pattern, cx, cy, nc, sum, lane);
        else if (tw == 8) tz_had_batch<8, 4>(S, P, slot, bx, by, pattern, cx, cy, nc, sum, lane);
        else tz_had_batch<4, 8>(S, P, slot, bx, by, pattern, cx, cy, nc, sum, lane);
    }
    __syncwarp();
}

__global__ void __launch_bounds__(32 * TZ_WARPS) k_me_tz(const TzParams P)
{
    __shared__ __align__(16) u32 s_org[TZ_WARPS][64 * 64 / 4];
    __shared__ u32 s_sum[TZ_WARPS][9];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.x * TZ_WARPS + warp;
    if (r >= P.n) return;
    const TzReq q = P.reqs[r];
    TzOut o;
    o.mv[0] = q.mv[0]; o.mv[1] = q.mv[1];
    o.mv_ipel[0] = q.mv_ipel[0]; o.mv_ipel[1] = q.mv_ipel[1];
    const int x = q.x, y = q.y, w = q.w, h = q.h, mvr = q.mvr, bi = q.bi;
    // calls outside the supported domain (block inside the picture, sides 4..64 powers of two,
    // known slots, resolution 0..4) come back with cost UINT64_MAX and their MVs unchanged
    const bool pow2 = (w & (w - 1)) == 0 && (h & (h - 1)) == 0;
    if (!pow2 || w < 4 || w > 64 || h < 4 || h > 64 || x < 0 || y < 0 || x + w > P.W || y + h > P.H || mvr > 4 ||
        q.ref_slot >= P.n_slots || (bi && q.other_slot >= P.n_slots) || q.refi < 0 || q.refi > 15 ||
        q.num_refp > 16) {
        o.cost = ~0ull;
        if (lane == 0) P.out[r] = o;
        return;
    }
    TzS S;
    // get_max_search_range (src/me.c:502-527), com_ipel_range_rounding above integer resolution
    const int mt = (P.mto << mvr) >> 2, px = q.mvp[0] >> 2, py = q.mvp[1] >> 2;
    if (P.is_padding) {
        S.minx = max(-127 - x, px - mt + 4); S.miny = max(-127 - y, py - mt + 4);
        S.maxx = min(P.W - 1 - x, px + mt - 4); S.maxy = min(P.H - 1 - y, py + mt - 4);
    } else {
        S.minx = max(-x, px - mt + 4); S.miny = max(-y, py - mt + 4);
        S.maxx = min(P.W - 1 - x - w, px + mt - 4); S.maxy = min(P.H - 1 - y - h, py + mt - 4);
    }
    if (mvr > 2) {
        const int s = mvr - 2;
        S.minx = S.minx >= 0 ? (S.minx >> s) << s : -(((-S.minx) >> s) << s);
        S.miny = S.miny >= 0 ? (S.miny >> s) << s : -(((-S.miny) >> s) << s);
        S.maxx = S.maxx >= 0 ? (S.maxx >> s) << s : -(((-S.maxx) >> s) << s);
        S.maxy = S.maxy >= 0 ? (S.maxy >> s) << s : -(((-S.maxy) >> s) << s);
    }
    if (S.minx > S.maxx || S.miny > S.maxy) {
        o.cost = ~0ull;
        if (lane == 0) P.out[r] = o;
        return;
    }
    // the block searched against: org, or 2 org - the other list's prediction (clipped)
    u32 *so = s_org[warp];
    const int wq = w >> 2;
    {
        const pel *og = P.org + (long long)y * P.i_org + x;
        const pel *pr = bi ? tz_mc_ptr(P, q.other_slot, (x << 2) + q.other_mv[0], (y << 2) + q.other_mv[1]) : og;
        for (int i = lane; i < wq * h; i += 32) {
            const int rr = i / wq, c = (i - rr * wq) * 4;
            u32 v = 0;
#pragma unroll
            for (int b = 0; b < 4; b++) {
                int s = og[rr * P.i_org + c + b];
                if (bi) s = min(max(2 * s - (int)pr[rr * P.i_ref + c + b], 0), 255);
                v |= (u32)s << (8 * b);
            }
            so[i] = v;
        }
    }
    __syncwarp();
    S.so = so; S.wq = wq; S.w = w; S.h = h;
    S.ref = P.planes[q.ref_slot * 16] + (long long)y * P.i_ref + x;
    S.stride = P.i_ref;
    S.mvr = mvr; S.shift = 16 - bi;
    S.bpx = q.mvp[0] >> mvr; S.bpy = q.mvp[1] >> mvr;
    S.lambda = q.lambda_mv;
    const int mx0 = bi ? q.mv[0] : q.mvp[0], my0 = bi ? q.mv[1] : q.mvp[1];
    S.mvx = min(max((mx0 + 2) >> 2, S.minx), S.maxx);
    S.mvy = min(max((my0 + 2) >> 2, S.miny), S.maxy);
    S.best = ~0ull;
    const int bs = tz_diamond(S, 32, bi, q.mvp[0], q.mvp[1], lane);
    if (!bi && (abs(q.mvp[0] - (S.mvx << 2)) > 2 || abs(q.mvp[1] - (S.mvy << 2)) > 2)) {
        if (bs > 5) tz_raster(S, q, P, lane);
        tz_diamond(S, 8, bi, q.mvp[0], q.mvp[1], lane);
    }
    if (!bi) { o.mv_ipel[0] = (s16)S.mvx; o.mv_ipel[1] = (s16)S.mvy; }
    int qx = S.mvx << 2, qy = S.mvy << 2;
    u64 cost = S.best;
    if (mvr < 2) {
        // me_sub_pel_search: centre + 8 half-sample points, then 8 quarter-sample points
        const bool sad = q.flags & 1;
        const int bx = x << 2, by = y << 2;
        u32 *sum = s_sum[warp];
        const int cx0 = qx, cy0 = qy;
        tz_sub_costs(S, P, q.ref_slot, bx, by, 0, cx0, cy0, 9, sad, sum, lane);
        u64 best = (u64)(S.lambda * (tz_bits((qx >> mvr) - S.bpx) + tz_bits((qy >> mvr) - S.bpy))) +
                   ((u64)sum[0] << S.shift);
        for (int i = 1; i < 9; i++) {
            int vx, vy;
            tz_sub_mv(0, i, cx0, cy0, vx, vy);
            const u64 c = (u64)(S.lambda * (tz_bits((vx >> mvr) - S.bpx) + tz_bits((vy >> mvr) - S.bpy))) +
                          ((u64)sum[i] << S.shift);
            if (c < best) { best = c; qx = vx; qy = vy; }
        }
        if (mvr == 0) {
            const int cx1 = qx, cy1 = qy;
            __syncwarp();
            tz_sub_costs(S, P, q.ref_slot, bx, by, 1, cx1, cy1, 8, sad, sum, lane);
            for (int i = 0; i < 8; i++) {
                int vx, vy;
                tz_sub_mv(1, i, cx1, cy1, vx, vy);
                const u64 c = (u64)(S.lambda * (tz_bits((vx >> mvr) - S.bpx) + tz_bits((vy >> mvr) - S.bpy))) +
                              ((u64)sum[i] << S.shift);
                if (c < best) { best = c; qx = vx; qy = vy; }
            }
        }
        if (sad) {   // SAD search, SATD at the winner
            __syncwarp();
            tz_sub_costs(S, P, q.ref_slot, bx, by, 2, qx, qy, 1, false, sum, lane);
            best = (u64)(S.lambda * (tz_bits((qx >> mvr) - S.bpx) + tz_bits((qy >> mvr) - S.bpy))) +
                   ((u64)sum[0] << (16 - bi));
        }
        cost = best;
    }
    const int rb = q.num_refp <= 1 ? 0 : min(q.refi + 1, q.num_refp - 1);   // tbl_refi_bits, src/tables.c:52
    const int extra = rb + mvr + (mvr < 4) + (bi ? q.mot_bits_other + 1 : 2);
    cost += (u64)(q.lambda_mv * (u32)extra);
    o.mv[0] = (s16)qx; o.mv[1] = (s16)qy;
    o.cost = (u32)((cost + (1u << 15)) >> 16);
    if (lane == 0) P.out[r] = o;
}

int launch_me_tz(const uavs3e_cuda_tz_pic_t *pic, const pel *org, int i_org, const pel *const *planes, int n_slots,
                 int i_ref, int pad, const void *reqs, int n, void *out, cudaStream_t st)
{
    if (!pic || !org || !planes || !reqs || !out || n < 0) return set_status(UC_ERR_ARG, "me_tz: null argument");
    if (n_slots < 1 || n_slots > UAVS3E_CUDA_TZ_MAX_SLOTS) return set_status(UC_ERR_ARG, "me_tz: slot count");
    if (pic->width < 8 || pic->height < 8 || pic->gop_size < 1 || pic->max_search_range < 4 ||
        pic->max_search_range > 1024)
        return set_status(UC_ERR_ARG, "me_tz: picture parameters");
    if ((i_ref & 3) || i_ref < pic->width + 2 * pad || pad < 144 || i_org < pic->width)
        return set_status(UC_ERR_ARG, "me_tz: strides / padding (planes padded by >= 144, stride a multiple of 4)");
    if (n == 0) return UC_OK;
    TzParams P;
    memset(&P, 0, sizeof(P));
    for (int i = 0; i < n_slots * 16; i++) {
        if (!planes[i]) return set_status(UC_ERR_ARG, "me_tz: null plane");
        P.planes[i] = planes[i];
    }
    P.org = org; P.i_org = i_org; P.i_ref = i_ref; P.n_slots = n_slots;
    P.W = pic->width; P.H = pic->height; P.is_padding = pic->is_padding ? 1 : 0;
    P.max_search_range = pic->max_search_range; P.gop_size = pic->gop_size;
    P.mto = (std::max(pic->width, pic->height) << 2) + 3;
    P.reqs = (const TzReq *)reqs; P.n = n; P.out = (TzOut *)out;
    P.sq32 = sqrt(32.0); P.sq128 = sqrt(128.0);
    P.k32 = had_scale_k(P.sq32); P.k128 = had_scale_k(P.sq128);
    prof_begin(PROF_TZ, st);
    k_me_tz<<<(unsigned)((n + TZ_WARPS - 1) / TZ_WARPS), 32 * TZ_WARPS, 0, st>>>(P);
    UC_CHECK(cudaGetLastError());
    count_launch(1);
    prof_end(PROF_TZ, st);
    return UC_OK;
}

}  // namespace uc

using namespace uc;

extern "C" UAVS3E_CUDA_API int uavs3e_cuda_me_tz_device(const uavs3e_cuda_tz_pic_t *pic, const uint8_t *d_org, int i_org,
                                                        const uint8_t *const *d_planes, int n_slots, int i_ref, int pad,
                                                        const uavs3e_cuda_tz_req_t *d_reqs, int n,
                                                        uavs3e_cuda_tz_out_t *d_out, void *stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    return launch_me_tz(pic, d_org, i_org, d_planes, n_slots, i_ref, pad, d_reqs, n, d_out, (cudaStream_t)stream);
}
