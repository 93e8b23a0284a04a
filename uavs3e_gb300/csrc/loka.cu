// Lookahead cost estimation on the GPU: loka_estimate_coding_cost (src/lookahead.c:82-293) for
// every 16x16 unit of a picture at once.
//
// k_loka_search: one warp per (unit, reference) runs the integer search of me_search_tz
//   (src/me.c:529-568) with the lookahead's settings (curr_mvr 2, predictor (0,0), no
//   bi-prediction).  Its stages depend on one another (diamond -> raster rounds -> refinement
//   diamond) but the candidates inside one stage do not: each stage is a list of candidates in
//   the reference's evaluation order, the warp costs 32 of them at a time (one 16x16 SAD per
//   lane) and keeps the minimum of (cost << 20 | position in the list).  The first minimum in
//   list order is what the reference's strictly-smaller updates keep, and a stage replaces the
//   running best only when its minimum is strictly smaller, as each of its updates would.
//   The SATD (com_had) of the winner closes the search.
// k_loka_unit: one warp per unit picks each list's winner, builds the two bi-prediction
//   averages, predicts the 11 intra modes from the original picture's neighbours, the chroma
//   blocks with the best mode, the unit's energy, and sums the picture totals.  Every 16x16
//   prediction is spread over the warp (8 samples a lane, one mode at a time) and its SATD is a
//   warp Hadamard (rows in registers, columns through shuffles).
#include "common.cuh"
#include "intra.cuh"
#include "uavs3e_cuda_internal.h"
#include "../../include/uavs3e_cuda.h"

#include <algorithm>
#include <math.h>
#include <mutex>
#include <string.h>
#include <vector>

namespace uc {

constexpr int LK_REFS = UAVS3E_CUDA_LOKA_MAX_REFS;
constexpr int LK_WARPS = 4;         // units per CTA
constexpr int LK_LIST_BITS = 20;    // candidate position bits of a stage key (cost < 2^33 above them)

struct LokaUnit {
    s16 mv[2][LK_REFS][2];
    u32 satd[2][LK_REFS];
    u32 bi_satd, zero_satd, min_cost, min_icost, icost_u, icost_v;
    u64 energy;
    u8 best_mode, pad[7];
};
static_assert(sizeof(LokaUnit) == sizeof(uavs3e_cuda_loka_unit_t), "unit record layout");

struct LokaParams {
    const pel *org, *org_u, *org_v;
    int i_org, i_org_c;
    const pel *ref[2][LK_REFS];
    int i_ref;
    int W, H, nux, n_units, is_padding;
    int n_ref[2];
    int range[2][LK_REFS];    // raster half-range of each reference (get_raster_range, src/me.c:65-100)
    u32 lambda;
    LokaUnit *units;
    u64 *energy;              // per unit, compact copy of LokaUnit::energy
    u64 *totals;              // sums of min_cost, min_icost, icost_u, icost_v; SAD evaluations
};

// diamond ring points of search_diamond (src/me.c:307-331) for max_step 32: step 4 (4 points),
// step 8 (8 points), step 16 (16 points), in evaluation order; {dx, dy, step}
__device__ __constant__ static const s8 kRing[28][3] = {
    { -4, 0, 4 }, { 0, 4, 4 }, { 4, 0, 4 }, { 0, -4, 4 },
    { -8, 0, 8 }, { -4, 4, 8 }, { 0, 8, 8 }, { 4, 4, 8 }, { 8, 0, 8 }, { 4, -4, 8 }, { 0, -8, 8 }, { -4, -4, 8 },
    { -16, 0, 16 }, { -12, 4, 16 }, { -8, 8, 16 }, { -4, 12, 16 }, { 0, 16, 16 }, { 4, 12, 16 }, { 8, 8, 16 },
    { 12, 4, 16 }, { 16, 0, 16 }, { 12, -4, 16 }, { 8, -8, 16 }, { 4, -12, 16 }, { 0, -16, 16 }, { -4, -12, 16 },
    { -8, -8, 16 }, { -12, -4, 16 },
};

// the 11 intra modes of the estimate (src/lookahead.c:213)
__device__ __constant__ static const u8 kLokaModes[11] = { 0, 1, 2, 4, 8, 12, 16, 20, 24, 28, 32 };

// MV bits of an integer MV component with predictor 0 at integer resolution: the table of
// inter_search_create (src/inter.c:2029-2057) is 1 at 0 and 2e for |v| in [2^(e-1) - 1, 2^e - 2]
__device__ __forceinline__ u32 lk_bits(int v)
{
    return v == 0 ? 1u : 2u * (32u - (u32)__clz(abs(v) + 1));
}

// 16x16 SAD of the org block (smem words, row-major 4 per row) against p (stride a multiple of 4)
__device__ __forceinline__ u32 lk_sad16(const u32 *so, const pel *p, int stride)
{
    const uintptr_t a = (uintptr_t)p;
    const u32 *w = (const u32 *)(a & ~(uintptr_t)3);
    const u32 sh = (u32)(a & 3) * 8;
    const int ws = stride >> 2;
    u32 s = 0;
#pragma unroll 4
    for (int r = 0; r < 16; r++) {
        const u32 *q = w + r * ws;
        u32 w0 = __ldg(q), w1 = __ldg(q + 1), w2 = __ldg(q + 2), w3 = __ldg(q + 3), w4 = __ldg(q + 4);
        uint4 o = *(const uint4 *)(so + r * 4);
        s = sad4(o.x, __funnelshift_r(w0, w1, sh), s);
        s = sad4(o.y, __funnelshift_r(w1, w2, sh), s);
        s = sad4(o.z, __funnelshift_r(w2, w3, sh), s);
        s = sad4(o.w, __funnelshift_r(w3, w4, sh), s);
    }
    return s;
}

struct LkSearch {
    const u32 *so;            // org block (smem)
    const pel *ref;           // reference sample co-located with the unit origin
    int stride;
    int minx, maxx, miny, maxy;
    u32 lambda;
    u64 best;
    int mvx, mvy;
    int evals;                // SADs this lane computed
};

__device__ __forceinline__ u64 lk_cost(LkSearch &S, int mx, int my)
{
    S.evals++;
    u32 sad = lk_sad16(S.so, S.ref + my * S.stride + mx, S.stride);
    return ((u64)sad << 16) + (u64)((lk_bits(mx) + lk_bits(my)) * S.lambda);
}

// The reference rows every candidate of one diamond reads, staged in shared memory: rows
// [wy0, wy1 + 15] and, per row, the words from the aligned start of column wx0 to the 5th word of
// the last candidate (the span the global loads of lk_sad16 cover, nothing beyond it)
struct LkWin {
    const u32 *w;
    int nw, wx0, wy0, sh0;
};

constexpr int LK_WIN_WORDS = 48 * 13;    // radius 16: 48 rows of (32 + 3) / 4 + 5 words

__device__ __forceinline__ LkWin lk_stage(const LkSearch &S, int cx, int cy, int radius, u32 *buf, int lane)
{
    LkWin W;
    W.wx0 = max(cx - radius, S.minx);
    W.wy0 = max(cy - radius, S.miny);
    const int wx1 = min(cx + radius, S.maxx), wy1 = min(cy + radius, S.maxy);
    const uintptr_t base = (uintptr_t)(S.ref + W.wy0 * S.stride + W.wx0);
    W.sh0 = (int)(base & 3);
    W.nw = (wx1 - W.wx0 + W.sh0) / 4 + 5;
    const int rows = wy1 - W.wy0 + 16;
    const u32 *a0 = (const u32 *)(base & ~(uintptr_t)3);
    const int ws = S.stride >> 2;
    for (int i = lane; i < rows * W.nw; i += 32) {
        const int r = i / W.nw, k = i - r * W.nw;
        buf[i] = __ldg(a0 + r * ws + k);
    }
    __syncwarp();
    W.w = buf;
    return W;
}

// lk_cost with the SAD read from a staged window
__device__ __forceinline__ u64 lk_cost_win(LkSearch &S, const LkWin &W, int mx, int my)
{
    S.evals++;
    const int b = mx - W.wx0 + W.sh0;
    const u32 *q = W.w + (my - W.wy0) * W.nw + (b >> 2);
    const u32 sh = (u32)(b & 3) * 8;
    u32 sad = 0;
#pragma unroll 4
    for (int r = 0; r < 16; r++, q += W.nw) {
        const u32 w0 = q[0], w1 = q[1], w2 = q[2], w3 = q[3], w4 = q[4];
        const uint4 o = *(const uint4 *)(S.so + r * 4);
        sad = sad4(o.x, __funnelshift_r(w0, w1, sh), sad);
        sad = sad4(o.y, __funnelshift_r(w1, w2, sh), sad);
        sad = sad4(o.z, __funnelshift_r(w2, w3, sh), sad);
        sad = sad4(o.w, __funnelshift_r(w3, w4, sh), sad);
    }
    return ((u64)sad << 16) + (u64)((lk_bits(mx) + lk_bits(my)) * S.lambda);
}

// search_diamond with bi = 0 (src/me.c:199-334) around the current MV; n_ring 28 for max_step 32
// (candidates within 16 of the centre), 4 for max_step 8 (within 4).  Returns the reference's
// best_step.
__device__ int lk_diamond(LkSearch &S, int n_ring, u32 *buf, int lane)
{
    const int cx = S.mvx, cy = S.mvy;
    __syncwarp();                            // the previous stage's reads of buf are done
    const LkWin W = lk_stage(S, cx, cy, n_ring > 4 ? 16 : 4, buf, lane);
    // core square with its edges strictly inside the MV range (src/me.c:240-243)
    const int x0 = max(cx - 2, S.minx + 1), x1 = min(cx + 2, S.maxx - 1);
    const int y0 = max(cy - 2, S.miny + 1), y1 = min(cy + 2, S.maxy - 1);
    const int ncx = max(0, x1 - x0 + 1), ncy = max(0, y1 - y0 + 1);
    const int ncore = ncx * ncy, n = 1 + ncore + n_ring;
    u64 kmin = ~0ull;
    for (int base = 0; base < n; base += 32) {
        const int k = base + lane;
        if (k >= n) continue;
        int mx, my;
        if (k == 0) { mx = cx; my = cy; }
        else if (k <= ncore) { mx = x0 + (k - 1) % ncx; my = y0 + (k - 1) / ncx; }
        else {
            const int j = k - 1 - ncore;
            mx = cx + kRing[j][0]; my = cy + kRing[j][1];
            if (mx < S.minx || mx > S.maxx || my < S.miny || my > S.maxy) continue;
        }
        const u64 key = (lk_cost_win(S, W, mx, my) << LK_LIST_BITS) | (u64)k;
        kmin = key < kmin ? key : kmin;
    }
    kmin = warp_min_u64(kmin);
    int step = -1;
    if (kmin != ~0ull && (kmin >> LK_LIST_BITS) < S.best) {
        const int k = (int)(kmin & ((1u << LK_LIST_BITS) - 1));
        S.best = kmin >> LK_LIST_BITS;
        if (k == 0) { S.mvx = cx; S.mvy = cy; }
        else if (k <= ncore) { S.mvx = x0 + (k - 1) % ncx; S.mvy = y0 + (k - 1) / ncx; }
        else { const int j = k - 1 - ncore; S.mvx = cx + kRing[j][0]; S.mvy = cy + kRing[j][1]; step = kRing[j][2]; }
    }
    if (step < 0) step = (S.mvx != cx || S.mvy != cy) ? 2 : 0;
    return step;
}

// one grid of search_raster (src/me.c:126-190): [x0, x1] x [y0, y1] in steps of s, rows outer
__device__ void lk_grid(LkSearch &S, int x0, int x1, int y0, int y1, int s, int lane)
{
    const int nx = (x1 - x0) / s + 1, ny = (y1 - y0) / s + 1, n = nx * ny;
    u64 kmin = ~0ull;
    for (int base = 0; base < n; base += 32) {
        const int k = base + lane;
        if (k >= n) continue;
        const int mx = x0 + (k % nx) * s, my = y0 + (k / nx) * s;
        const u64 key = (lk_cost(S, mx, my) << LK_LIST_BITS) | (u64)k;
        kmin = key < kmin ? key : kmin;
    }
    kmin = warp_min_u64(kmin);
    if ((kmin >> LK_LIST_BITS) < S.best) {
        const int k = (int)(kmin & ((1u << LK_LIST_BITS) - 1));
        S.best = kmin >> LK_LIST_BITS;
        S.mvx = x0 + (k % nx) * s;
        S.mvy = y0 + (k / nx) * s;
    }
}

// A grid of step 8 with the lanes along one grid row: the 16 samples of lane l's candidate are
// the words w[2l .. 2l+4] of the row (from the common aligned base), so each lane loads its own
// two words and takes the next three from lanes l+1 and l+2.  30 candidates per pass; the two
// lanes after the last candidate only load, and only the words of the last candidate's span.
// Vertically the candidates of consecutive grid rows are 8 rows apart and share 8 of their 16
// reference rows, so a pass walks the reference rows once, top to bottom: each row feeds the
// candidate it is row r of (r = 0..15) and, for r >= 8, also the next grid row's candidate (its
// row r - 8); a candidate's SAD is complete at its row 15.
__device__ void lk_grid8(LkSearch &S, int x0, int x1, int y0, int y1, int lane)
{
    const int nx = (x1 - x0) / 8 + 1, ny = (y1 - y0) / 8 + 1;
    const u32 sh = (u32)(((uintptr_t)(S.ref + x0)) & 3) * 8;       // the same for every row and lane
    const int ws = S.stride >> 2;
    u64 kmin = ~0ull;
    for (int c0 = 0; c0 < nx; c0 += 30) {
        const int nc = min(30, nx - c0);
        const bool ld = lane < nc + 2, ld1 = lane < nc + 1;
        const int mx = x0 + 8 * (c0 + lane);
        const u32 *q = (const u32 *)(((uintptr_t)(S.ref + y0 * S.stride + mx)) & ~(uintptr_t)3);
        u32 sa = 0, sb = 0;   // SADs of grid rows g and g + 1
        int g = 0, ra = 0;    // ra: the current reference row's index within grid row g's candidate
        const int rows = 8 * ny + 8;
        for (int R = 0; R < rows; R++, q += ws) {
            const u32 w0 = ld ? __ldg(q) : 0u, w1 = ld1 ? __ldg(q + 1) : 0u;
            const u32 w2 = __shfl_down_sync(0xffffffffu, w0, 1), w3 = __shfl_down_sync(0xffffffffu, w1, 1);
            const u32 w4 = __shfl_down_sync(0xffffffffu, w0, 2);
            const u32 d0 = __funnelshift_r(w0, w1, sh), d1 = __funnelshift_r(w1, w2, sh);
            const u32 d2 = __funnelshift_r(w2, w3, sh), d3 = __funnelshift_r(w3, w4, sh);
            const uint4 o = *(const uint4 *)(S.so + ra * 4);
            sa = sad4(o.x, d0, sa);
            sa = sad4(o.y, d1, sa);
            sa = sad4(o.z, d2, sa);
            sa = sad4(o.w, d3, sa);
            if (ra >= 8 && g + 1 < ny) {
                const uint4 ob = *(const uint4 *)(S.so + (ra - 8) * 4);
                sb = sad4(ob.x, d0, sb);
                sb = sad4(ob.y, d1, sb);
                sb = sad4(ob.z, d2, sb);
                sb = sad4(ob.w, d3, sb);
            }
            if (ra == 15) {
                if (lane < nc) {
                    S.evals++;
                    const int my = y0 + 8 * g;
                    const u64 cost = ((u64)sa << 16) + (u64)((lk_bits(mx) + lk_bits(my)) * S.lambda);
                    const u64 key = (cost << LK_LIST_BITS) | (u64)(g * nx + c0 + lane);
                    kmin = key < kmin ? key : kmin;
                }
                sa = sb;
                sb = 0;
                g++;
                ra = 8;
                if (g >= ny) break;
            } else {
                ra++;
            }
        }
    }
    kmin = warp_min_u64(kmin);
    if ((kmin >> LK_LIST_BITS) < S.best) {
        const int k = (int)(kmin & ((1u << LK_LIST_BITS) - 1));
        S.best = kmin >> LK_LIST_BITS;
        S.mvx = x0 + (k % nx) * 8;
        S.mvy = y0 + (k / nx) * 8;
    }
}

// search_raster with adaptive_raster_range 0: the full-range grid of step 8 (refi + 1), then
// grids of the halved step around the running best until the step is 1
__device__ void lk_raster(LkSearch &S, int refi, int range, int lane)
{
    int s = 8 * (refi + 1);
    const int gx0 = min(max(S.mvx - range, S.minx), S.maxx), gx1 = min(max(S.mvx + range, S.minx), S.maxx);
    const int gy0 = min(max(S.mvy - range, S.miny), S.maxy), gy1 = min(max(S.mvy + range, S.miny), S.maxy);
    if (s == 8) lk_grid8(S, gx0, gx1, gy0, gy1, lane);
    else lk_grid(S, gx0, gx1, gy0, gy1, s, lane);
    for (s >>= 1; s >= 1; s >>= 1)
        lk_grid(S, max(S.mvx - s, S.minx), min(S.mvx + s, S.maxx), max(S.mvy - s, S.miny), min(S.mvy + s, S.maxy), s,
                lane);
}

// org block of a unit into shared memory as 64 little-endian words (byte loads: any alignment)
__device__ __forceinline__ void lk_load_org(u32 *so, const pel *org, int i_org, int lane)
{
    const int r = lane >> 1, c = (lane & 1) * 8;
    const pel *p = org + r * i_org + c;
    so[r * 4 + (c >> 2)] = (u32)p[0] | (u32)p[1] << 8 | (u32)p[2] << 16 | (u32)p[3] << 24;
    so[r * 4 + (c >> 2) + 1] = (u32)p[4] | (u32)p[5] << 8 | (u32)p[6] << 16 | (u32)p[7] << 24;
}

// com_had of a 16x16 difference block held by the warp: lane l has row l >> 1, columns
// (l & 1) * 8 .. +7.  Rows of each 8x8 tile are transformed in registers, columns across the
// lanes whose bits 1..3 differ (butterflies on lane ^ 2, ^ 4, ^ 8); each tile's sum of magnitudes
// is rounded as com_had_8x8 does ((s + 2) >> 2) and the four tiles are added.  Every lane
// returns the total.
__device__ __forceinline__ u32 warp_had16(int *d, int lane)
{
    wht<8>(d);
#pragma unroll
    for (int b = 2; b <= 8; b <<= 1) {
        const bool hi = lane & b;
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int p = __shfl_xor_sync(0xffffffffu, d[i], b);
            d[i] = hi ? p - d[i] : d[i] + p;
        }
    }
    int s = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) s += abs(d[i]);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    s += __shfl_xor_sync(0xffffffffu, s, 4);
    s += __shfl_xor_sync(0xffffffffu, s, 8);
    u32 t = (u32)((s + 2) >> 2);
    t += __shfl_xor_sync(0xffffffffu, t, 1);
    t += __shfl_xor_sync(0xffffffffu, t, 16);
    return t;
}

// com_had of two 8x8 difference blocks: lane l has row l & 7 of block (l >> 3) & 1 (lanes 16..31
// repeat 0..15); columns are transformed across lane ^ 1, ^ 2, ^ 4.  Returns the block's SATD.
__device__ __forceinline__ u32 warp_had8x2(int *d, int lane)
{
    wht<8>(d);
#pragma unroll
    for (int b = 1; b <= 4; b <<= 1) {
        const bool hi = lane & b;
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int p = __shfl_xor_sync(0xffffffffu, d[i], b);
            d[i] = hi ? p - d[i] : d[i] + p;
        }
    }
    int s = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) s += abs(d[i]);
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    s += __shfl_xor_sync(0xffffffffu, s, 4);
    return (u32)((s + 2) >> 2);
}

// the 16x16 SATD of the org block (smem bytes, stride 16) against p
__device__ __forceinline__ u32 lk_had16(const pel *o, const pel *p, int ip, int lane)
{
    const int j = lane >> 1, i0 = (lane & 1) * 8;
    int d[8];
#pragma unroll
    for (int k = 0; k < 8; k++) d[k] = (int)o[j * 16 + i0 + k] - (int)p[j * ip + i0 + k];
    return warp_had16(d, lane);
}

__global__ void __launch_bounds__(32 * LK_WARPS) k_loka_search(const LokaParams P)
{
    __shared__ __align__(16) u32 s_org[LK_WARPS][64];
    __shared__ u32 s_win[LK_WARPS][LK_WIN_WORDS];
    __shared__ unsigned long long s_evals;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int u = blockIdx.x * LK_WARPS + warp;
    const int l = (int)blockIdx.y < P.n_ref[0] ? 0 : 1;
    const int r = (int)blockIdx.y - (l ? P.n_ref[0] : 0);
    if (threadIdx.x == 0) s_evals = 0;
    __syncthreads();
    if (u < P.n_units) {
        const int x = (u % P.nux) * 16, y = (u / P.nux) * 16;
        lk_load_org(s_org[warp], P.org + y * P.i_org + x, P.i_org, lane);
        __syncwarp();
        LkSearch S;
        S.so = s_org[warp];
        S.ref = P.ref[l][r] + y * P.i_ref + x;
        S.stride = P.i_ref;
        S.lambda = P.lambda;
        S.evals = 0;
        // get_max_search_range (src/me.c:502-527), predictor 0, integer resolution
        const int mto = (max(P.W, P.H) << 2) + 3;
        if (P.is_padding) {
            S.minx = max(-127 - x, -mto + 4); S.miny = max(-127 - y, -mto + 4);
            S.maxx = min(P.W - 1 - x, mto - 4); S.maxy = min(P.H - 1 - y, mto - 4);
        } else {
            S.minx = max(-x, -mto + 4); S.miny = max(-y, -mto + 4);
            S.maxx = min(P.W - 17 - x, mto - 4); S.maxy = min(P.H - 17 - y, mto - 4);
        }
        S.mvx = min(max(0, S.minx), S.maxx);
        S.mvy = min(max(0, S.miny), S.maxy);
        S.best = ~0ull;
        const int best_step = lk_diamond(S, 28, s_win[warp], lane);
        if (S.mvx != 0 || S.mvy != 0) {
            if (best_step > 5) lk_raster(S, r, P.range[l][r], lane);
            lk_diamond(S, 4, s_win[warp], lane);
        }
        const pel *blk = S.ref + S.mvy * P.i_ref + S.mvx;
        const u32 satd = lk_had16((const pel *)s_org[warp], blk, P.i_ref, lane);
        if (lane == 0) {
            LokaUnit &U = P.units[u];
            U.mv[l][r][0] = (s16)S.mvx;
            U.mv[l][r][1] = (s16)S.mvy;
            U.satd[l][r] = satd;
        }
        int ev = S.evals;
#pragma unroll
        for (int o = 16; o; o >>= 1) ev += __shfl_xor_sync(0xffffffffu, ev, o);
        if (lane == 0) atomicAdd(&s_evals, (unsigned long long)ev);
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_evals) atomicAdd((unsigned long long *)&P.totals[4], s_evals);
}

// get_ipred_neighbor (src/lookahead.c:40-80) into c[-range .. range] (c = array centre)
__device__ __forceinline__ void lk_nbr(pel *c, int x, int y, int w, int h, int W, int H, const pel *src, int s,
                                       int lane)
{
    const int range = max(w, h) * 4 + 4;
    const int nu = min(2 * w, W - x), nl = min(2 * h, H - y);
    for (int i = lane; i < range; i += 32) {
        c[1 + i] = y ? src[-s + min(i, nu - 1)] : (pel)128;
        c[-1 - i] = x ? src[min(i, nl - 1) * s - 1] : (pel)128;
    }
    if (lane == 0) c[0] = (x && y) ? src[-s - 1] : y ? src[-s] : x ? src[-1] : (pel)128;
}

__device__ __forceinline__ u64 lk_var_sums(const pel *p, int s, int n, int lane, u64 *sq_out)
{
    // n x n block, lanes stride over the samples
    u32 sum = 0, sq = 0;
    for (int i = lane; i < n * n; i += 32) {
        const u32 v = p[(i / n) * s + (i % n)];
        sum += v; sq += v * v;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        sq += __shfl_xor_sync(0xffffffffu, sq, o);
    }
    *sq_out = sq;
    return sum;
}

// cost_var (src/com_cost.c:139-151)
__device__ __forceinline__ u64 lk_var(const pel *p, int s, int n, int log2n, int lane)
{
    u64 sq;
    const u64 sum = lk_var_sums(p, s, n, lane, &sq);
    return sq - ((sum * sum) >> (2 * log2n));
}

__global__ void __launch_bounds__(32 * LK_WARPS) k_loka_unit(const LokaParams P)
{
    __shared__ __align__(16) pel s_org[LK_WARPS][256];
    __shared__ pel s_nb[LK_WARPS][3][144];
    __shared__ unsigned long long s_tot[4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int u = blockIdx.x * LK_WARPS + warp;
    if (threadIdx.x < 4) s_tot[threadIdx.x] = 0;
    __syncthreads();
    if (u < P.n_units) {
        const int x = (u % P.nux) * 16, y = (u / P.nux) * 16;
        const pel *org = P.org + y * P.i_org + x;
        pel *so = s_org[warp];
        // lane l covers row j, columns i0 .. i0 + 7 of the unit in every 16x16 pass below
        const int j = lane >> 1, i0 = (lane & 1) * 8;
#pragma unroll
        for (int k = 0; k < 8; k++) so[j * 16 + i0 + k] = org[j * P.i_org + i0 + k];
        LokaUnit &U = P.units[u];
        // per list: the first reference with the smallest SATD (src/lookahead.c:131-175)
        u64 min_cost = ~0ull;
        int best_ref[2] = { -1, -1 };
        for (int l = 0; l < 2; l++) {
            u64 min_dir = ~0ull;
            for (int r = 0; r < P.n_ref[l]; r++) {
                const u32 c = U.satd[l][r];
                if (c < min_dir) { min_dir = c; best_ref[l] = r; if (c < min_cost) min_cost = c; }
            }
        }
        u32 bi_satd = 0, zero_satd = 0;
        if (P.n_ref[0] && P.n_ref[1]) {
            // pel_avrg of the two list winners, then of the (0,0) blocks of the first references
            const int r0 = best_ref[0], r1 = best_ref[1];
            const pel *a = P.ref[0][r0] + (y + U.mv[0][r0][1] + j) * P.i_ref + x + U.mv[0][r0][0] + i0;
            const pel *b = P.ref[1][r1] + (y + U.mv[1][r1][1] + j) * P.i_ref + x + U.mv[1][r1][0] + i0;
            const pel *za = P.ref[0][0] + (y + j) * P.i_ref + x + i0, *zb = P.ref[1][0] + (y + j) * P.i_ref + x + i0;
            int d[8];
#pragma unroll
            for (int k = 0; k < 8; k++) d[k] = (int)so[j * 16 + i0 + k] - ((a[k] + b[k] + 1) >> 1);
            bi_satd = warp_had16(d, lane);
#pragma unroll
            for (int k = 0; k < 8; k++) d[k] = (int)so[j * 16 + i0 + k] - ((za[k] + zb[k] + 1) >> 1);
            zero_satd = warp_had16(d, lane);
            if (bi_satd < min_cost) min_cost = bi_satd;
            if (zero_satd < min_cost) min_cost = zero_satd;
        }
        // intra: the 11 modes one after another over the whole warp, neighbours from the original
        // picture (src/lookahead.c:204-230)
        pel *c = s_nb[warp][0] + 70;
        lk_nbr(c, x, y, 16, 16, P.W, P.H, org, P.i_org, lane);
        __syncwarp();
        const int avail = (x ? 2 : 0) | (y ? 1 : 0) | ((x && y) ? 4 : 0);
        u32 min_icost = 0xFFFFFFFFu;
        int best_mode = 0;
        {
            IpredBlock B;
            ipred_block_setup(c, 16, 16, avail, 8, B);
            for (int m = 0; m < 11; m++) {
                const int mode = kLokaModes[m];
                int d[8];
#pragma unroll
                for (int k = 0; k < 8; k++) d[k] = (int)so[j * 16 + i0 + k] - ipred_sample(c, B, mode, 0, i0 + k, j);
                const u32 cost = warp_had16(d, lane);
                if (cost < min_cost) min_cost = cost;
                if (cost < min_icost) { min_icost = cost; best_mode = mode; }
            }
        }
        // chroma 8x8 blocks with the luma winner (src/lookahead.c:231-243): lanes 0..7 U, 8..15 V
        const int xc = x >> 1, yc = y >> 1;
        const pel *ou = P.org_u + yc * P.i_org_c + xc, *ov = P.org_v + yc * P.i_org_c + xc;
        pel *cu = s_nb[warp][1] + 40, *cv = s_nb[warp][2] + 40;
        lk_nbr(cu, xc, yc, 8, 8, P.W >> 1, P.H >> 1, ou, P.i_org_c, lane);
        lk_nbr(cv, xc, yc, 8, 8, P.W >> 1, P.H >> 1, ov, P.i_org_c, lane);
        __syncwarp();
        u32 icost_u, icost_v;
        {
            const int plane = (lane >> 3) & 1, row = lane & 7;
            const pel *cc = plane ? cv : cu, *oc = (plane ? ov : ou) + row * P.i_org_c;
            IpredBlock B;
            ipred_block_setup(cc, 8, 8, avail, 8, B);
            int d[8];
#pragma unroll
            for (int k = 0; k < 8; k++) d[k] = (int)oc[k] - ipred_sample(cc, B, best_mode, 0, k, row);
            const u32 t = warp_had8x2(d, lane);
            icost_u = __shfl_sync(0xffffffffu, t, 0);
            icost_v = __shfl_sync(0xffffffffu, t, 8);
        }
        // energy of the dQP map (src/lookahead.c:248-262)
        const u64 energy = lk_var(org, P.i_org, 16, 4, lane) + lk_var(ou, P.i_org_c, 8, 3, lane) +
                           lk_var(ov, P.i_org_c, 8, 3, lane);
        if (lane == 0) {
            U.bi_satd = bi_satd;
            U.zero_satd = zero_satd;
            U.min_cost = (u32)min_cost;
            U.min_icost = min_icost;
            U.icost_u = icost_u;
            U.icost_v = icost_v;
            U.energy = energy;
            U.best_mode = (u8)best_mode;
#pragma unroll
            for (int i = 0; i < 7; i++) U.pad[i] = 0;
            for (int l = 0; l < 2; l++)           // slots of absent references read as zero
                for (int r = P.n_ref[l]; r < LK_REFS; r++) {
                    U.mv[l][r][0] = 0; U.mv[l][r][1] = 0; U.satd[l][r] = 0;
                }
            P.energy[u] = energy;
            atomicAdd(&s_tot[0], (unsigned long long)(u32)min_cost);
            atomicAdd(&s_tot[1], (unsigned long long)min_icost);
            atomicAdd(&s_tot[2], (unsigned long long)icost_u);
            atomicAdd(&s_tot[3], (unsigned long long)icost_v);
        }
    }
    __syncthreads();
    if (threadIdx.x < 4 && s_tot[threadIdx.x]) atomicAdd((unsigned long long *)&P.totals[threadIdx.x], s_tot[threadIdx.x]);
}

// lambda_mv of the estimate: base QP 32 (src/lookahead.c:85-106)
static u32 loka_lambda()
{
    const double base_lambda = 1.43631 * pow(2.0, (32 - 16.0) / 4.0);
    return (u32)floor(65536.0 * sqrt(base_lambda));
}

int loka_check_cfg(const uavs3e_cuda_loka_cfg_t *cfg)
{
    if (!cfg) return set_status(UC_ERR_ARG, "loka: no configuration");
    const int W = cfg->width, H = cfg->height;
    if (W < 17 || H < 17 || (W & 1) || (H & 1) || W > 8192 || H > 8192)
        return set_status(UC_ERR_ARG, "loka: picture size (17..8192, even)");
    // raster grids of up to (max_search_range / 8 + 1)^2 points keep their positions below 2^20
    if (cfg->gop_size < 1 || cfg->max_search_range < 4 || cfg->max_search_range > 4096)
        return set_status(UC_ERR_ARG, "loka: gop size / search range");
    for (int l = 0; l < 2; l++)
        if (cfg->num_ref[l] < 0 || cfg->num_ref[l] > LK_REFS) return set_status(UC_ERR_ARG, "loka: reference count");
    return UC_OK;
}

int launch_loka(const uavs3e_cuda_loka_cfg_t *cfg, const pel *org, int i_org, const pel *org_u, const pel *org_v,
                int i_org_c, const pel *const *ref_l0, const pel *const *ref_l1, int i_ref, int ref_pad,
                LokaUnit *units, u64 *energy, u64 *totals, cudaStream_t st)
{
    int rc = loka_check_cfg(cfg);
    if (rc) return rc;
    if (!org || !org_u || !org_v || !units || !energy || !totals) return set_status(UC_ERR_ARG, "loka: null buffer");
    if (i_org < cfg->width || i_org_c < cfg->width / 2) return set_status(UC_ERR_ARG, "loka: org stride");
    const int n_search = cfg->num_ref[0] + cfg->num_ref[1];
    if (n_search) {
        if ((i_ref & 3) || i_ref < cfg->width + 2 * ref_pad) return set_status(UC_ERR_ARG, "loka: reference stride");
        if (ref_pad < (cfg->is_padding ? 144 : 4)) return set_status(UC_ERR_ARG, "loka: reference padding");
    }
    LokaParams P;
    memset(&P, 0, sizeof(P));
    P.org = org; P.org_u = org_u; P.org_v = org_v; P.i_org = i_org; P.i_org_c = i_org_c;
    P.i_ref = i_ref;
    P.W = cfg->width; P.H = cfg->height; P.nux = cfg->width / 16;
    P.n_units = (cfg->width / 16) * (cfg->height / 16);
    P.is_padding = cfg->is_padding ? 1 : 0;
    const int max_sr = cfg->max_search_range >> 1;
    for (int l = 0; l < 2; l++) {
        P.n_ref[l] = cfg->num_ref[l];
        for (int r = 0; r < cfg->num_ref[l]; r++) {
            const pel *p = (l ? ref_l1 : ref_l0) ? (l ? ref_l1 : ref_l0)[r] : nullptr;
            if (!p) return set_status(UC_ERR_ARG, "loka: null reference");
            P.ref[l][r] = p;
            long long d = cfg->ptr - cfg->ref_ptr[l][r];
            const int dist = (int)(d < 0 ? -d : d);
            const long long v = ((long long)max_sr * dist + (cfg->gop_size >> 1)) / cfg->gop_size;
            P.range[l][r] = (int)std::min<long long>(max_sr, std::max<long long>(max_sr >> 2, v));
        }
    }
    P.lambda = loka_lambda();
    P.units = units; P.energy = energy; P.totals = totals;
    if (P.n_units == 0) return UC_OK;
    prof_begin(PROF_LOKA, st);
    UC_CHECK(cudaMemsetAsync(totals, 0, 5 * sizeof(u64), st));
    const unsigned nb = (unsigned)((P.n_units + LK_WARPS - 1) / LK_WARPS);
    int launches = 1;
    if (n_search) {
        k_loka_search<<<dim3(nb, (unsigned)n_search), 32 * LK_WARPS, 0, st>>>(P);
        UC_CHECK(cudaGetLastError());
        launches++;
    }
    k_loka_unit<<<nb, 32 * LK_WARPS, 0, st>>>(P);
    UC_CHECK(cudaGetLastError());
    count_launch(launches);
    prof_end(PROF_LOKA, st);
    return UC_OK;
}

// the picture-level results from the totals and energies (src/lookahead.c:255-292): integer
// totals converted to double equal the reference's unit-by-unit double sums (every partial sum
// is an integer below 2^53); the dQP map is formed in raster order as the reference does
double loka_finish(int W, int H, const u64 *totals, const u64 *energy, double *icost, double *icost_uv, float *map_dqp)
{
    const int n = (W / 16) * (H / 16);
    if (icost) *icost = (double)totals[1] / n / 16 / 16;
    if (icost_uv) {
        icost_uv[0] = (double)totals[2] / n / 8 / 8;
        icost_uv[1] = (double)totals[3] / n / 8 / 8;
    }
    if (map_dqp) {
        double tvar = 0;
        for (int i = 0; i < n; i++) {
            const u64 e = energy[i];
            map_dqp[i] = (float)(0.8 * log2((double)(e > 1 ? e : 1)));
            tvar += map_dqp[i];
        }
        const float avg = (float)(tvar / n);
        for (int i = 0; i < n; i++) map_dqp[i] -= avg;
    }
    return (double)totals[0] / n / 16 / 16;
}

// per device: buffers of the host-memory entry point
struct LokaScratch {
    std::mutex mu;
    cudaStream_t st = nullptr;
    pel *org = nullptr, *ref = nullptr;
    size_t org_cap = 0, ref_cap = 0;
    LokaUnit *units = nullptr;
    u64 *energy = nullptr, *totals = nullptr, *h_totals = nullptr;
    size_t unit_cap = 0, energy_cap = 0;
};
static LokaScratch g_loka[64];

template <class T>
static int grow(T **p, size_t *cap, size_t n)
{
    if (*cap >= n) return UC_OK;
    if (*p) UC_CHECK(cudaFree(*p));
    *p = nullptr;
    *cap = 0;
    UC_CHECK(cudaMalloc(p, n * sizeof(T)));
    *cap = n;
    return UC_OK;
}

}  // namespace uc

using namespace uc;

extern "C" {

UAVS3E_CUDA_API int uavs3e_cuda_loka_units_device(const uavs3e_cuda_loka_cfg_t *cfg, const uint8_t *d_org_y,
                                                  int i_org, const uint8_t *d_org_u, const uint8_t *d_org_v,
                                                  int i_org_c, const uint8_t *const *d_ref_l0,
                                                  const uint8_t *const *d_ref_l1, int i_ref, int ref_pad,
                                                  uavs3e_cuda_loka_unit_t *d_units, uint64_t *d_energy,
                                                  uint64_t *d_totals, void *stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    return launch_loka(cfg, d_org_y, i_org, d_org_u, d_org_v, i_org_c, d_ref_l0, d_ref_l1, i_ref, ref_pad,
                       (LokaUnit *)d_units, (u64 *)d_energy, (u64 *)d_totals, (cudaStream_t)stream);
}

UAVS3E_CUDA_API double uavs3e_cuda_loka_finish(const uavs3e_cuda_loka_cfg_t *cfg, const uint64_t totals[4],
                                               const uint64_t *energy, double *icost, double icost_uv[2],
                                               float *map_dqp)
{
    if (loka_check_cfg(cfg) || !totals || (map_dqp && !energy)) {
        set_status(UC_ERR_ARG, "loka_finish: bad arguments");
        return -1.0;
    }
    return loka_finish(cfg->width, cfg->height, (const u64 *)totals, (const u64 *)energy, icost, icost_uv, map_dqp);
}

UAVS3E_CUDA_API int uavs3e_cuda_loka_estimate(const uavs3e_cuda_loka_cfg_t *cfg, const uint8_t *org_y, int i_org,
                                              const uint8_t *org_u, const uint8_t *org_v, int i_org_c,
                                              const uint8_t *const *ref_l0, const uint8_t *const *ref_l1, int i_ref,
                                              int ref_pad, double *cost, double *icost, double icost_uv[2],
                                              float *map_dqp, uavs3e_cuda_loka_unit_t *units)
{
    int rc = ensure_init();
    if (rc) return rc;
    rc = loka_check_cfg(cfg);
    if (rc) return rc;
    if (!org_y || !org_u || !org_v) return set_status(UC_ERR_ARG, "loka_estimate: null org plane");
    int dev = 0;
    UC_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_status(UC_ERR_UNSUPPORTED, "loka_estimate: device index");
    LokaScratch &S = g_loka[dev];
    std::lock_guard<std::mutex> lk(S.mu);
    if (!S.st) UC_CHECK(cudaStreamCreateWithFlags(&S.st, cudaStreamNonBlocking));
    if (!S.totals) {
        UC_CHECK(cudaMalloc(&S.totals, 8 * sizeof(u64)));
        UC_CHECK(cudaMallocHost(&S.h_totals, 8 * sizeof(u64)));
    }
    const int W = cfg->width, H = cfg->height, Wc = W / 2, Hc = H / 2;
    const int n_units = (W / 16) * (H / 16);
    const int n_search = cfg->num_ref[0] + cfg->num_ref[1];
    // device copies: org planes at stride W (16-aligned), references with `pad` samples around
    const int so = (W + 15) & ~15, soc = (Wc + 15) & ~15;
    // the device copies carry `pad` samples around the picture; the caller's planes need
    // padding only when the search may leave the picture (only then is the padding copied)
    const int pad = cfg->is_padding ? 144 : 4;
    if (n_search && cfg->is_padding && ref_pad < 144)
        return set_status(UC_ERR_ARG, "loka_estimate: reference padding");
    const int sr = (W + 2 * pad + 15) & ~15;
    const size_t plane = (size_t)sr * (H + 2 * pad);
    rc = grow(&S.org, &S.org_cap, (size_t)so * H + 2 * (size_t)soc * Hc);
    if (!rc) rc = grow(&S.ref, &S.ref_cap, plane * (size_t)std::max(n_search, 1));
    if (!rc) rc = grow(&S.units, &S.unit_cap, (size_t)std::max(n_units, 1));
    if (!rc) rc = grow(&S.energy, &S.energy_cap, (size_t)std::max(n_units, 1));
    if (rc) return rc;
    pel *d_y = S.org, *d_u = S.org + (size_t)so * H, *d_v = d_u + (size_t)soc * Hc;
    UC_CHECK(cudaMemcpy2DAsync(d_y, so, org_y, i_org, W, H, cudaMemcpyHostToDevice, S.st));
    UC_CHECK(cudaMemcpy2DAsync(d_u, soc, org_u, i_org_c, Wc, Hc, cudaMemcpyHostToDevice, S.st));
    UC_CHECK(cudaMemcpy2DAsync(d_v, soc, org_v, i_org_c, Wc, Hc, cudaMemcpyHostToDevice, S.st));
    const pel *d_refs[2][LK_REFS] = {};
    int k = 0;
    for (int l = 0; l < 2; l++)
        for (int r = 0; r < cfg->num_ref[l]; r++, k++) {
            const uint8_t *src = (l ? ref_l1 : ref_l0) ? (l ? ref_l1 : ref_l0)[r] : nullptr;
            if (!src) return set_status(UC_ERR_ARG, "loka_estimate: null reference");
            pel *dst = S.ref + plane * k;
            if (cfg->is_padding) {
                // the padded region the search can reach, as the encoder holds it
                UC_CHECK(cudaMemcpy2DAsync(dst, sr, src - (size_t)pad * i_ref - pad, i_ref, W + 2 * pad, H + 2 * pad,
                                           cudaMemcpyHostToDevice, S.st));
            } else {
                UC_CHECK(cudaMemcpy2DAsync(dst + (size_t)pad * sr + pad, sr, src, i_ref, W, H, cudaMemcpyHostToDevice,
                                           S.st));
            }
            d_refs[l][r] = dst + (size_t)pad * sr + pad;
        }
    rc = launch_loka(cfg, d_y, so, d_u, d_v, soc, d_refs[0], d_refs[1], sr, pad, S.units, S.energy, S.totals, S.st);
    if (rc) return rc;
    UC_CHECK(cudaMemcpyAsync(S.h_totals, S.totals, 5 * sizeof(u64), cudaMemcpyDeviceToHost, S.st));
    u64 *h_energy = nullptr;
    std::vector<u64> e_host;
    if (map_dqp) {
        e_host.resize((size_t)n_units);
        h_energy = e_host.data();
        UC_CHECK(cudaMemcpyAsync(h_energy, S.energy, (size_t)n_units * sizeof(u64), cudaMemcpyDeviceToHost, S.st));
    }
    if (units)
        UC_CHECK(cudaMemcpyAsync(units, S.units, (size_t)n_units * sizeof(LokaUnit), cudaMemcpyDeviceToHost, S.st));
    UC_CHECK(cudaStreamSynchronize(S.st));
    const double c = loka_finish(W, H, S.h_totals, h_energy, icost, icost_uv, map_dqp);
    if (cost) *cost = c;
    return UC_OK;
}

UAVS3E_CUDA_API int uavs3e_cuda_loka_sc_ratio(int width, int height, int is_padding, int max_search_range,
                                              int gop_size, int64_t ptr, const uint8_t *org_y, int i_org,
                                              const uint8_t *org_u, const uint8_t *org_v, int i_org_c,
                                              const uint8_t *last_y, int64_t last_ptr, int i_last, int last_pad,
                                              double *ratio)
{
    uavs3e_cuda_loka_cfg_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.width = width; cfg.height = height; cfg.is_padding = is_padding;
    cfg.max_search_range = max_search_range; cfg.gop_size = gop_size;
    cfg.num_ref[0] = 1; cfg.num_ref[1] = 0;
    cfg.ptr = ptr; cfg.ref_ptr[0][0] = last_ptr;
    const uint8_t *refs[1] = { last_y };
    double pcost = 0, icost = 0;
    int rc = uavs3e_cuda_loka_estimate(&cfg, org_y, i_org, org_u, org_v, i_org_c, refs, nullptr, i_last, last_pad,
                                       &pcost, &icost, nullptr, nullptr, nullptr);
    if (rc) return rc;
    if (ratio) *ratio = pcost / icost;
    return UC_OK;
}

}  // extern "C"
