// Affine motion search for lists of calls: affine_me_gradient (src/inter.c:1339-1470) -- up to 7
// (uni) / 5 (bi) Gauss-Newton steps of the 4-parameter affine model, each from the normal
// equations of the residual and the Sobel gradients of the current prediction, its CPMV change
// rounded to the AMVR step and kept when the SATD + MV cost drops -- with the start CPMVs of
// analyze_affine_uni (:1607-1647) or the bi org of analyze_affine_bi (:1730-1790) on request.
// Bit-exact with the reference, including its double-precision solve.
//
// One warp per call.  The CU's org (or bi org) and the current prediction sit in shared memory;
// the prediction (com_mc_blk_affine_luma, src/com_mc.c:202-250) is rebuilt there after every
// step, the lanes walk its samples for the SATD tiles and the equation sums, which reduce across
// the warp in 64-bit integers.  The 4x4 solve runs over the warp's lanes in IEEE double with every
// operation rounded on its own (no fused multiply-add), in the reference's order.
#include "common.cuh"
#include "affine.cuh"
#include "uavs3e_cuda_internal.h"
#include "../../include/uavs3e_cuda.h"

#include <math.h>
#include <string.h>

namespace uc {

constexpr int AME_WARPS = 2;
constexpr s32 CPMV_MIN = -131072, CPMV_MAX = 131071;

struct AffMeReq {
    s16 x, y; u8 w, h; u8 ref_slot; s8 refi; u8 num_refp; u8 mvr; u8 flags; u8 other_slot;
    u32 lambda_mv; s32 mot_bits_other; s32 pad;
    s32 mvp[2][2]; s32 mv[2][2]; s32 other_mv[2][2];
};
struct AffMeOut { s32 mv[2][2]; u32 satd; s32 bits; u64 cost; };
static_assert(sizeof(AffMeReq) == sizeof(uavs3e_cuda_affme_req_t), "affine search request layout");
static_assert(sizeof(AffMeOut) == sizeof(uavs3e_cuda_affme_out_t), "affine search result layout");

struct AffMeParams {
    const pel *planes[UAVS3E_CUDA_TZ_MAX_SLOTS];   // integer plane of each slot
    const pel *org;
    int i_org, i_ref, n_slots, W, H, n;
    double sq32, sq128;
    u64 k32, k128;       // had_scale_k of sq32, sq128
    const AffMeReq *reqs;
    AffMeOut *out;
};

// Tab_Affine_AMVR (inc/com_define.h:203)
__device__ __forceinline__ int ame_shift(int mvr) { return mvr == 0 ? 2 : (mvr == 1 ? 4 : 0); }

// MV_COST (src/inter.c:41): unsigned 32-bit product, rounded
__device__ __forceinline__ u32 ame_mv_cost(u32 lambda, int bits) { return (lambda * (u32)bits + 32768u) >> 16; }

__device__ __forceinline__ int ame_log2(int v) { return 31 - __clz(v); }

// affine_mv_bits (src/inter.c:1317-1337), tbl_refi_bits (src/tables.c:52) in closed form
__device__ __forceinline__ int ame_bits(const s32 *mv, const s32 *mvp, int num_refp, int refi, int sh)
{
    int bits = num_refp <= 1 ? 0 : min(refi + 1, num_refp - 1);
#pragma unroll
    for (int v = 0; v < 2; v++) {
        const int dx = abs((mv[2 * v] - mvp[2 * v]) >> sh), dy = abs((mv[2 * v + 1] - mvp[2 * v + 1]) >> sh);
        bits += ((ame_log2(dx + 1) + ame_log2(dy + 1)) << 1) + 2 + (dx != 0) + (dy != 0);
    }
    return bits;
}

// com_mc_blk_affine_luma (src/com_mc.c:202-250) into dst (w x h, stride w): each sample takes the
// MV of its SUB x SUB block (centre, or the control point for the two top corner blocks), rounded
// to 1/16 and clipped to 18 bits, and is filtered from the integer plane (com_mc_blk_luma, hp).
// A lane takes one column of one band of sub-blocks (aff_luma_column).
template <int SUB>
__device__ void ame_pred_t(const AffMeParams &P, const pel *plane, int x, int y, int w, int h, int lw, const s32 *mv,
                           pel *dst, int lane)
{
    const s32 dhx = ((mv[2] - mv[0]) * 128) >> lw, dhy = ((mv[3] - mv[1]) * 128) >> lw;
    const s32 dvx = -dhy, dvy = dhx;
    const int tasks = w * (h / SUB);
    for (int t = lane; t < tasks; t += 32) {
        const int c = t & (w - 1), by = (t >> lw) * SUB, bx = c & ~(SUB - 1);
        int px = bx + SUB / 2, py = by + SUB / 2;
        if (bx == 0 && by == 0) { px = 0; py = 0; }
        else if (bx + SUB == w && by == 0) { px = w; py = 0; }
        const s32 mx = min(max(aff_round7(mv[0] * 128 + dhx * px + dvx * py), CPMV_MIN), CPMV_MAX);
        const s32 my = min(max(aff_round7(mv[1] * 128 + dhy * px + dvy * py), CPMV_MIN), CPMV_MAX);
        const int qx = ((x + bx) << 4) + mx, qy = ((y + by) << 4) + my;
        int v[SUB];
        aff_luma_column<SUB>(plane, P.i_ref, P.W, P.H, qx, qy, c - bx, v);
#pragma unroll
        for (int o = 0; o < SUB; o++) dst[(by + o) * w + c] = (pel)v[o];
    }
}

__device__ __noinline__ void ame_pred(const AffMeParams &P, const pel *plane, int x, int y, int w, int h, int lw,
                                      const s32 *mv, int sub, pel *dst, int lane)
{
    if (sub == 8) ame_pred_t<8>(P, plane, x, y, w, h, lw, mv, dst, lane);
    else ame_pred_t<4>(P, plane, x, y, w, h, lw, mv, dst, lane);
}

// com_had (src/com_cost.c:712-812) of the w x h block o - p (both stride w) with TW x TH tiles.
// 2:1 tiles: each pass's group sums move to one lane per tile, and the double normalisation runs
// once for all (at most 16) tiles of the block instead of once per pass.
template <int TW, int TH>
__device__ u32 ame_had_tiles(const pel *o, const pel *p, int w, int h, int lane, double sq32, double sq128, u64 k32,
                             u64 k128)
{
    constexpr int G = 32 / TH;                      // tiles per pass
    const int ntx = w / TW, ntiles = ntx * (h / TH), total = ntiles * TH;
    u32 acc = 0;
    int held = 0;
    for (int base = 0, pass = 0; base < total; base += 32, pass++) {
        const int t = base + lane;
        const bool active = t < total;
        const int tt = active ? t : 0, tile = tt / TH, row = tt - tile * TH;
        const int off = ((tile / ntx) * TH + row) * w + (tile % ntx) * TW;
        const int s = had_tile_sum<TW, TH>(o + off, p + off, active, lane);
        if (TW == TH) {
            if (active && row == 0) acc += had_tile_norm<TW, TH>(s, sq32, sq128, k32, k128);
        } else {
            const int got = __shfl_sync(0xffffffffu, s, ((lane - pass * G) * TH) & 31);
            if (lane >= pass * G && lane < pass * G + G) held = got;
        }
    }
    if (TW != TH && lane < ntiles) acc = had_tile_norm<TW, TH>(held, sq32, sq128, k32, k128);
#pragma unroll
    for (int m = 16; m; m >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, m);
    return acc;
}

__device__ __noinline__ u32 ame_had(const pel *o, const pel *p, int w, int h, int lane, const AffMeParams &P)
{
    if (w == h) return ame_had_tiles<8, 8>(o, p, w, h, lane, P.sq32, P.sq128, P.k32, P.k128);
    if (w > h) return ame_had_tiles<16, 8>(o, p, w, h, lane, P.sq32, P.sq128, P.k32, P.k128);
    return ame_had_tiles<8, 16>(o, p, w, h, lane, P.sq32, P.sq128, P.k32, P.k128);
}

// the sums of one gradient step (affine_sobel_flt_hor / _ver and affine_coef_computer,
// src/com_util.c:2966-3045): per sample the Sobel gradients of the prediction at the nearest
// interior position, the four model columns c0..c3 and the residual; e[0..9] = the products
// c_i c_j (i <= j), e[10..13] = c_i * residual, summed over the block and the warp
__device__ void ame_equations(const pel *o, const pel *p, int w, int h, int lw, int lane, s64 *e)
{
#pragma unroll
    for (int i = 0; i < 14; i++) e[i] = 0;
    for (int i = lane; i < w * h; i += 32) {
        const int j = i >> lw, k = i & (w - 1);
        const int jj = min(max(j, 1), h - 2), kk = min(max(k, 1), w - 2);
        const pel *q = p + jj * w + kk;
        const int gx = q[1 - w] - q[-1 - w] + 2 * (q[1] - q[-1]) + q[1 + w] - q[-1 + w];
        const int gy = q[w - 1] - q[-w - 1] + 2 * (q[w] - q[-w]) + q[w + 1] - q[-w + 1];
        const int r = (int)o[i] - (int)p[i];
        const int c0 = gx, c1 = k * gx + j * gy, c2 = gy, c3 = j * gx - k * gy;
        e[0] += (s64)c0 * c0; e[1] += (s64)c0 * c1; e[2] += (s64)c0 * c2; e[3] += (s64)c0 * c3;
        e[4] += (s64)c1 * c1; e[5] += (s64)c1 * c2; e[6] += (s64)c1 * c3;
        e[7] += (s64)c2 * c2; e[8] += (s64)c2 * c3; e[9] += (s64)c3 * c3;
        e[10] += (s64)c0 * r; e[11] += (s64)c1 * r; e[12] += (s64)c2 * r; e[13] += (s64)c3 * r;
    }
#pragma unroll
    for (int i = 0; i < 14; i++)
#pragma unroll
        for (int m = 16; m; m >>= 1) e[i] += __shfl_xor_sync(0xffffffffu, e[i], m);
}

// (s16) of a double as x86-64 code converts it (the reference's platform): truncation to 32 bits
// by cvttsd2si -- NaN and values outside the 32-bit range give INT_MIN -- then the low 16 bits
// (the range test on the exponent bits: |v| >= 2^31, infinities and NaN all give INT_MIN, and
// the values in (-2^31 - 1, -2^31] that truncate to INT_MIN give it too)
__device__ __forceinline__ s16 ame_to_s16(double v)
{
    const int e = (int)((unsigned long long)__double_as_longlong(v) >> 52) & 0x7ff;
    const int i = e < 1023 + 31 ? __double2int_rz(v) : (int)0x80000000u;
    return (s16)(u16)(u32)i;
}

// the bits of |v| as an unsigned integer: for non-NaN values |a| > |b| exactly when
// ame_mag(a) > ame_mag(b); NaN maps above every finite value
__device__ __forceinline__ unsigned long long ame_mag(double v)
{
    return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}

// solve_equal (src/inter.c:1280-1315) over the warp and the conversion of its solution to the four
// CPMV changes (x0, y0, x1, y1) at AMVR shift sh.  Lane 5 r + k (< 25) holds element (r, k) of the
// augmented matrix (rows 1..4, row 0 being the reference's swap buffer); in step i every element
// (j > i, k >= i) of the elimination is one lane's a[j][k] - a[i][k] * a[j][i-1] / a[i][i-1], each
// operation rounded on its own, so the values are the reference's; the back substitution runs on
// lane 0 in the reference's order.  e[] = the equation sums (identical in every lane).
__device__ __noinline__ void ame_solve(const s64 *e, int w, int sh, int lane, s16 *mvd)
{
    const bool mine = lane < 25;
    const int r = mine ? lane / 5 : 0, col = mine ? lane - 5 * (lane / 5) : 0;
    // coef[c + 1][k] = e[ix(c, k)] for k < 4 (the symmetric products), coef[c + 1][4] = 8 e[10 + c]
    const int c = r - 1;
    const int lo = min(c, col), hi = max(c, col);
    const int idx = col == 4 ? 10 + c : (lo == 0 ? hi : (lo == 1 ? 3 + hi : (lo == 2 ? 5 + hi : 9)));
    s64 val = 0;
#pragma unroll
    for (int i = 0; i < 14; i++) val = (i == idx) ? e[i] : val;
    if (col == 4) val *= 8;
    double v = (mine && r >= 1) ? __ll2double_rn(val) : 0.0;
    for (int i = 1; i < 4; i++) {
        // fabs(cand) > best in integers: false when cand is NaN, and nothing exceeds a NaN best
        unsigned long long best = ame_mag(__shfl_sync(0xffffffffu, v, i * 5 + i - 1));
        int bi = i;
        for (int j = i + 1; j < 5; j++) {
            const unsigned long long cand = ame_mag(__shfl_sync(0xffffffffu, v, j * 5 + i - 1));
            if (cand <= 0x7ff0000000000000ull && cand > best) { best = cand; bi = j; }
        }
        if (bi != i) {
            const int src = (mine && r == i) ? bi * 5 + col : ((mine && r == bi) ? i * 5 + col : lane);
            v = __shfl_sync(0xffffffffu, v, src);
        }
        const double aik = __shfl_sync(0xffffffffu, v, i * 5 + col);
        const double aji = __shfl_sync(0xffffffffu, v, r * 5 + i - 1);
        const double aii = __shfl_sync(0xffffffffu, v, i * 5 + i - 1);
        if (mine && r > i && col >= i) v = __dsub_rn(v, __ddiv_rn(__dmul_rn(aik, aji), aii));
    }
    double m[25];
#pragma unroll
    for (int k = 5; k < 25; k++) m[k] = __shfl_sync(0xffffffffu, v, k);
    double x[4] = { 0, 0, 0, 0 };
    if (lane == 0) {
#define A(i, j) m[(i) * 5 + (j)]
        x[3] = __ddiv_rn(A(4, 4), A(4, 3));
#pragma unroll
        for (int i = 2; i >= 0; i--) {
            double t = 0;
#pragma unroll
            for (int j = i + 1; j < 4; j++) t = __dadd_rn(t, __dmul_rn(A(i + 1, j), x[j]));
            x[i] = __ddiv_rn(__dsub_rn(A(i + 1, 4), t), A(i + 1, i));
        }
#undef A
    }
    // lanes 0..3 convert x0 -> mvd x0, x2 -> y0, x1 w + x0 -> x1, -x3 w + x2 -> y1
    const double x0 = __shfl_sync(0xffffffffu, x[0], 0), x1 = __shfl_sync(0xffffffffu, x[1], 0);
    const double x2 = __shfl_sync(0xffffffffu, x[2], 0), x3 = __shfl_sync(0xffffffffu, x[3], 0);
    u32 o = 0;
    if (lane < 4) {
        const double wd = (double)w;
        const double d = lane == 0 ? x0 : (lane == 1 ? x2 : (lane == 2 ? __dadd_rn(__dmul_rn(x1, wd), x0)
                                                                        : __dadd_rn(__dmul_rn(-x3, wd), x2)));
        // d >= 0: +0, -0 and positive values, not NaN
        const long long db = __double_as_longlong(d);
        const bool ge0 = db == (long long)0x8000000000000000ull ||
                         (db >= 0 && (unsigned long long)db <= 0x7ff0000000000000ull);
        const double half = ge0 ? 0.5 : -0.5;
        s16 q;
        if (sh == 0) q = ame_to_s16(__dadd_rn(__dmul_rn(d, 16.0), half));
        else {
            q = ame_to_s16(__dadd_rn(__dmul_rn(d, 4.0), half));
            q = (s16)(q << 2);
            q = (s16)(((q + (1 << (sh - 1))) >> sh) << sh);   // com_mv_rounding_s16
        }
        o = (u32)(u16)q;
    }
    u32 packed[2];
    packed[0] = __shfl_sync(0xffffffffu, o, 0) | (__shfl_sync(0xffffffffu, o, 1) << 16);
    packed[1] = __shfl_sync(0xffffffffu, o, 2) | (__shfl_sync(0xffffffffu, o, 3) << 16);
    mvd[0] = (s16)(u16)packed[0];
    mvd[1] = (s16)(u16)(packed[0] >> 16);
    mvd[2] = (s16)(u16)packed[1];
    mvd[3] = (s16)(u16)(packed[1] >> 16);
}

__device__ __forceinline__ bool ame_cpmv_ok(const s32 (*m)[2])
{
    return m[0][0] >= CPMV_MIN && m[0][0] <= CPMV_MAX && m[0][1] >= CPMV_MIN && m[0][1] <= CPMV_MAX &&
           m[1][0] >= CPMV_MIN && m[1][0] <= CPMV_MAX && m[1][1] >= CPMV_MIN && m[1][1] <= CPMV_MAX;
}

__global__ void __launch_bounds__(32 * AME_WARPS, 20 / AME_WARPS) k_me_affine(const AffMeParams P)
{
    __shared__ __align__(16) pel s_org[AME_WARPS][64 * 64];
    __shared__ __align__(16) pel s_pred[AME_WARPS][64 * 64];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.x * AME_WARPS + warp;
    if (r >= P.n) return;
    const AffMeReq q = P.reqs[r];
    AffMeOut *out = P.out + r;
    const int w = q.w, h = q.h, bi = q.flags & UAVS3E_CUDA_AFFME_BI;
    // calls outside the supported domain (CU inside the picture, sides 16..64, slots, AMVR index,
    // reference index, CPMVs within 18 bits) return cost ~0 with the start CPMVs
    if ((w != 16 && w != 32 && w != 64) || (h != 16 && h != 32 && h != 64) || q.x < 0 || q.y < 0 ||
        q.x + w > P.W || q.y + h > P.H || q.ref_slot >= P.n_slots || (bi && q.other_slot >= P.n_slots) ||
        q.mvr > 2 || q.refi < 0 || q.refi >= q.num_refp || !ame_cpmv_ok(q.mvp) ||
        (!(q.flags & UAVS3E_CUDA_AFFME_UNI_START) && !ame_cpmv_ok(q.mv)) || (bi && !ame_cpmv_ok(q.other_mv))) {
        if (lane == 0) {
            for (int v = 0; v < 2; v++) { out->mv[v][0] = q.mv[v][0]; out->mv[v][1] = q.mv[v][1]; }
            out->satd = 0;
            out->bits = 0;
            out->cost = ~0ull;
        }
        return;
    }
    pel *so = s_org[warp], *sp = s_pred[warp];
    const int lw = 31 - __clz(w), n = w * h;
    const pel *plane = P.planes[q.ref_slot];
    const pel *org = P.org + (long long)q.y * P.i_org + q.x;
    for (int i = lane; i < n; i += 32) so[i] = org[(i >> lw) * P.i_org + (i & (w - 1))];
    if (bi) {                                      // create_bi_org (src/inter.c:55), 8x8 prediction
        const s32 om[4] = { q.other_mv[0][0], q.other_mv[0][1], q.other_mv[1][0], q.other_mv[1][1] };
        ame_pred(P, P.planes[q.other_slot], q.x, q.y, w, h, lw, om, 8, sp, lane);
        __syncwarp();
        for (int i = lane; i < n; i += 32) so[i] = (pel)min(255, max(0, 2 * (int)so[i] - (int)sp[i]));
    }
    __syncwarp();
    const int sh = ame_shift(q.mvr), sub = (bi || (q.flags & UAVS3E_CUDA_AFFME_SUB8)) ? 8 : 4;
    const int other = bi ? q.mot_bits_other : 0;
    const s32 mvp[4] = { q.mvp[0][0], q.mvp[0][1], q.mvp[1][0], q.mvp[1][1] };
    s32 mv[4] = { q.mv[0][0], q.mv[0][1], q.mv[1][0], q.mv[1][1] };
    bool have_pred = false;
    u32 had = 0;
    if (!bi && (q.flags & UAVS3E_CUDA_AFFME_UNI_START)) {
        // analyze_affine_uni's start: the MVP, or the uni MV clipped (mv_clip, src/inter.c:1472) and
        // scaled to 1/16 sample (rounded to whole samples at AMVR index 1), whichever costs less
        ame_pred(P, plane, q.x, q.y, w, h, lw, mvp, sub, sp, lane);
        __syncwarp();
        const u64 c_mvp = (u64)ame_had(so, sp, w, h, lane, P) +
                          ame_mv_cost(q.lambda_mv, ame_bits(mvp, mvp, q.num_refp, q.refi, sh));
        const int x4 = q.x << 2, y4 = q.y << 2, w4 = w << 2, h4 = h << 2;
        const int min_c = (-128 - 4) << 2, max_x = (P.W - 1 + 128 + 4) << 2, max_y = (P.H - 1 + 128 + 4) << 2;
        s16 mx = (s16)q.mv[0][0], my = (s16)q.mv[0][1];
        if (x4 + mx < min_c) mx = (s16)(min_c - x4);
        if (y4 + my < min_c) my = (s16)(min_c - y4);
        if (x4 + mx + w4 - 4 > max_x) mx = (s16)(max_x - x4 - w4 + 4);
        if (y4 + my + h4 - 4 > max_y) my = (s16)(max_y - y4 - h4 + 4);
        s32 tx = (s32)mx * 4, ty = (s32)my * 4;
        if (q.mvr == 1) {
            tx = tx >= 0 ? ((tx + 8) >> 4) << 4 : -(((-tx + 8) >> 4) << 4);
            ty = ty >= 0 ? ((ty + 8) >> 4) << 4 : -(((-ty + 8) >> 4) << 4);
        }
        tx = min(max(tx, CPMV_MIN), CPMV_MAX);
        ty = min(max(ty, CPMV_MIN), CPMV_MAX);
        const s32 tmp[4] = { tx, ty, tx, ty };
        __syncwarp();
        ame_pred(P, plane, q.x, q.y, w, h, lw, tmp, sub, sp, lane);
        __syncwarp();
        const u32 had_tmp = ame_had(so, sp, w, h, lane, P);
        const u64 c_tmp = (u64)had_tmp + ame_mv_cost(q.lambda_mv, ame_bits(tmp, mvp, q.num_refp, q.refi, sh));
        if (c_tmp < c_mvp) {
#pragma unroll
            for (int v = 0; v < 4; v++) mv[v] = tmp[v];
            have_pred = true;
            had = had_tmp;
        } else {
#pragma unroll
            for (int v = 0; v < 4; v++) mv[v] = mvp[v];
        }
    }
    if (!have_pred) {
        __syncwarp();
        ame_pred(P, plane, q.x, q.y, w, h, lw, mv, sub, sp, lane);
        __syncwarp();
        had = ame_had(so, sp, w, h, lane, P);
    }
    // affine_me_gradient
    int best_bits = ame_bits(mv, mvp, q.num_refp, q.refi, sh) + other;
    u64 best = (u64)ame_mv_cost(q.lambda_mv, best_bits) + (had >> bi);
    s32 mvt[4] = { mv[0], mv[1], mv[2], mv[3] };
    for (int iter = 0; iter < (bi ? 5 : 7); iter++) {
        s64 e[14];
        ame_equations(so, sp, w, h, lw, lane, e);
        s16 mvd[4];
        ame_solve(e, w, sh, lane, mvd);
        if (!mvd[0] && !mvd[1] && !mvd[2] && !mvd[3]) break;
#pragma unroll
        for (int v = 0; v < 4; v++) {
            s32 m = min(max(mvt[v] + (s32)mvd[v], CPMV_MIN), CPMV_MAX);
            if (m == CPMV_MAX) m = m >> sh << sh;
            mvt[v] = m;
        }
        __syncwarp();
        ame_pred(P, plane, q.x, q.y, w, h, lw, mvt, sub, sp, lane);
        __syncwarp();
        const int bits = ame_bits(mvt, mvp, q.num_refp, q.refi, sh) + other;
        const u64 cost = (u64)ame_mv_cost(q.lambda_mv, bits) + (ame_had(so, sp, w, h, lane, P) >> bi);
        if (cost < best) {
            best = cost;
            best_bits = bits;
#pragma unroll
            for (int v = 0; v < 4; v++) mv[v] = mvt[v];
        }
    }
    if (lane == 0) {
        const u64 satd = best - ame_mv_cost(q.lambda_mv, best_bits);
        for (int v = 0; v < 2; v++) { out->mv[v][0] = mv[2 * v]; out->mv[v][1] = mv[2 * v + 1]; }
        out->satd = (u32)satd;
        out->bits = best_bits;
        out->cost = satd + ame_mv_cost(q.lambda_mv, best_bits);
    }
}

int launch_me_affine(int W, int H, const pel *org, int i_org, const pel *const *planes, int n_slots, int i_ref,
                     int pad, const void *reqs, int n, void *out, cudaStream_t st)
{
    if (!org || !planes || (n > 0 && (!reqs || !out)) || n < 0) return set_status(UC_ERR_ARG, "me_affine: null argument");
    if (n_slots < 1 || n_slots > UAVS3E_CUDA_TZ_MAX_SLOTS || W < 16 || H < 16 || i_org < W)
        return set_status(UC_ERR_ARG, "me_affine: slots / picture size / org stride");
    // 8-tap windows reach 132 + 3 samples before the picture and W + 4 + 7 + 4 after it
    if (pad < 144 || i_ref < W + 2 * pad) return set_status(UC_ERR_ARG, "me_affine: padding (>= 144) / stride");
    if (n == 0) return UC_OK;
    AffMeParams P;
    memset(&P, 0, sizeof(P));
    for (int s = 0; s < n_slots; s++) {
        if (!planes[s * 16]) return set_status(UC_ERR_ARG, "me_affine: null plane");
        P.planes[s] = planes[s * 16];
    }
    P.org = org; P.i_org = i_org; P.i_ref = i_ref; P.n_slots = n_slots; P.W = W; P.H = H; P.n = n;
    P.sq32 = sqrt(32.0);
    P.sq128 = sqrt(128.0);
    P.k32 = had_scale_k(P.sq32);
    P.k128 = had_scale_k(P.sq128);
    P.reqs = (const AffMeReq *)reqs;
    P.out = (AffMeOut *)out;
    prof_begin(PROF_AFFME, st);
    k_me_affine<<<(unsigned)((n + AME_WARPS - 1) / AME_WARPS), 32 * AME_WARPS, 0, st>>>(P);
    UC_CHECK(cudaGetLastError());
    count_launch(1);
    prof_end(PROF_AFFME, st);
    return UC_OK;
}

}  // namespace uc

using namespace uc;

UAVS3E_CUDA_API int uavs3e_cuda_me_affine_device(int width, int height, const uint8_t *d_org, int i_org,
                                                 const uint8_t *const *d_planes, int n_slots, int i_ref, int pad,
                                                 const uavs3e_cuda_affme_req_t *d_reqs, int n,
                                                 uavs3e_cuda_affme_out_t *d_out, void *stream)
{
    if (ensure_init()) return uavs3e_cuda_status();
    return launch_me_affine(width, height, d_org, i_org, d_planes, n_slots, i_ref, pad, d_reqs, n, d_out,
                            (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------------------------
// Affine control-point MVP: one thread per CU.  The neighbour walk, the POC-distance scaling
// (ratio = (2^14 / t_neb) * t_cur, C's truncating division first; symmetric rounding shift by
// 14; s16 clip) and the AMVR rounding of the 1/16-sample value (magnitude rounded, sign kept;
// 18-bit clip) are integer and follow com_get_affine_mvp_scaling step for step.
// ---------------------------------------------------------------------------------------------
static_assert(sizeof(uavs3e_cuda_affmvp_req_t) == 12, "affine MVP request layout");
static_assert(sizeof(uavs3e_cuda_affmvp_out_t) == 16, "affine MVP result layout");

__device__ __forceinline__ int amvp_scale(int mv, int ratio)
{
    const long long t = (long long)mv * ratio;
    const long long r = t == 0 ? 0 : t > 0 ? (t + 8192) >> 14 : -((-t + 8192) >> 14);
    return (int)max(-32768ll, min(32767ll, r));
}

__device__ __forceinline__ int amvp_round(int v, int shift)
{
    const int x = v * 4, add = shift > 0 ? 1 << (shift - 1) : 0;
    const int r = x >= 0 ? ((x + add) >> shift) << shift : -(((-x + add) >> shift) << shift);
    return max(-131072, min(131071, r));
}

__global__ void __launch_bounds__(256) k_affine_mvp(long long ptr, const long long *ref_ptr, int n_ref,
                                                    const short *map_mv, const signed char *map_refi, int i_scu,
                                                    long long n_field, const uavs3e_cuda_affmvp_req_t *reqs, int n,
                                                    uavs3e_cuda_affmvp_out_t *out, int *err)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uavs3e_cuda_affmvp_req_t q = reqs[i];
    uavs3e_cuda_affmvp_out_t o = {};
    bool bad = q.lidx < 0 || q.lidx > 1 || q.cur_refi < 0 || q.cur_refi >= n_ref || q.mvr < 0 || q.mvr > 2 ||
               q.cu_width < 4;
    int t_cur = 0;
    if (!bad) {
        t_cur = (int)(ptr * 2 - ref_ptr[q.cur_refi * 2 + q.lidx] * 2);
        bad = t_cur == 0;
    }
    int mv[2][2] = { { 0, 0 }, { 0, 0 } };
    if (!bad) {
        const long long base = (long long)i_scu + 1 + q.scup - i_scu;   // the row above the CU
        const int wsc = q.cu_width >> 2;
        // A (left, same row), B (above), D (above-left); G (above the last column), C (above-right)
        const long long nb[5] = { base + i_scu - 1, base, base - 1, base + wsc - 1, base + wsc };
#pragma unroll
        for (int g = 0; g < 2; g++) {
            bool found = false;
#pragma unroll
            for (int k = g == 0 ? 0 : 3; k < (g == 0 ? 3 : 5); k++) {
                if (found || bad) continue;
                const long long a = nb[k];
                if (a < 0 || a >= n_field) { bad = true; continue; }
                const int refi = map_refi[a * 2 + q.lidx];
                if (refi < 0) continue;
                if (refi >= n_ref) { bad = true; continue; }
                const int t_neb = (int)(ptr * 2 - ref_ptr[refi * 2 + q.lidx] * 2);
                if (t_neb == 0) { bad = true; continue; }
                const int ratio = (1 << 14) / t_neb * t_cur;
                const short2 v = *(const short2 *)(map_mv + (a * 2 + q.lidx) * 2);
                mv[g][0] = amvp_scale(v.x, ratio);
                mv[g][1] = amvp_scale(v.y, ratio);
                found = true;
            }
        }
    }
    if (!bad) {
        const int shift = q.mvr == 0 ? 2 : q.mvr == 1 ? 4 : 0;
#pragma unroll
        for (int g = 0; g < 2; g++) {
            o.mvp[g][0] = amvp_round(mv[g][0], shift);
            o.mvp[g][1] = amvp_round(mv[g][1], shift);
        }
    } else if (err) {
        atomicAdd(err, 1);
    }
    out[i] = o;
}

int launch_affine_mvp(long long ptr, const long long *d_ref_ptr, int n_ref, const short *d_map_mv,
                      const signed char *d_map_refi, int i_scu, int rows, const void *d_reqs, int n, void *d_out,
                      int *d_err, cudaStream_t st)
{
    if (n < 0 || n_ref < 1 || i_scu < 3 || rows < 2 || (n > 0 && (!d_ref_ptr || !d_map_mv || !d_map_refi || !d_reqs || !d_out)))
        return set_status(UC_ERR_ARG, "affine_mvp: bad argument");
    if (((uintptr_t)d_map_mv & 3) != 0) return set_status(UC_ERR_ARG, "affine_mvp: map_mv not 4-byte aligned");
    if (n == 0) return UC_OK;
    k_affine_mvp<<<(n + 255) / 256, 256, 0, st>>>(ptr, d_ref_ptr, n_ref, d_map_mv, d_map_refi, i_scu,
                                                  (long long)rows * i_scu, (const uavs3e_cuda_affmvp_req_t *)d_reqs, n,
                                                  (uavs3e_cuda_affmvp_out_t *)d_out, d_err);
    UC_CHECK(cudaGetLastError());
    count_launch(1);
    return UC_OK;
}

UAVS3E_CUDA_API int uavs3e_cuda_affine_mvp_device(int64_t ptr, const int64_t *d_ref_ptr, int n_ref,
                                                  const int16_t *d_map_mv, const int8_t *d_map_refi, int i_scu,
                                                  int rows, const uavs3e_cuda_affmvp_req_t *d_reqs, int n,
                                                  uavs3e_cuda_affmvp_out_t *d_out, int32_t *d_err, void *stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    return launch_affine_mvp(ptr, (const long long *)d_ref_ptr, n_ref, d_map_mv, (const signed char *)d_map_refi,
                             i_scu, rows, d_reqs, n, d_out, (int *)d_err, (cudaStream_t)stream);
}

UAVS3E_CUDA_API int uavs3e_cuda_affine_mvp(int64_t ptr, const int64_t *ref_ptr, int n_ref, const int16_t *map_mv,
                                           const int8_t *map_refi, int i_scu, int rows,
                                           const uavs3e_cuda_affmvp_req_t *reqs, int n,
                                           uavs3e_cuda_affmvp_out_t *out)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (n < 0 || n_ref < 1 || i_scu < 3 || rows < 2 || (n > 0 && (!ref_ptr || !map_mv || !map_refi || !reqs || !out)))
        return set_status(UC_ERR_ARG, "affine_mvp: bad argument");
    if (n == 0) return UC_OK;
    cudaStream_t st = nullptr;
    UC_CHECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    const size_t field = (size_t)rows * i_scu;
    const size_t b_ref = (size_t)n_ref * 16, b_mv = field * 8, b_refi = (field * 2 + 255) & ~(size_t)255;
    const size_t b_req = (size_t)n * sizeof(uavs3e_cuda_affmvp_req_t), b_out = (size_t)n * sizeof(uavs3e_cuda_affmvp_out_t);
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    char *buf = nullptr;
    cudaError_t ce = cudaMallocAsync((void **)&buf, up(b_ref) + up(b_mv) + b_refi + up(b_req) + up(b_out) + 256, st);
    if (ce != cudaSuccess) { cudaStreamDestroy(st); return check_cuda(ce, "affine_mvp: allocate"); }
    char *d_ref = buf, *d_mv = d_ref + up(b_ref), *d_refi = d_mv + up(b_mv), *d_req = d_refi + b_refi;
    char *d_out = d_req + up(b_req), *d_err = d_out + up(b_out);
    int bad = 0;
    rc = UC_OK;
    if ((ce = cudaMemcpyAsync(d_ref, ref_ptr, b_ref, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(d_mv, map_mv, b_mv, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(d_refi, map_refi, field * 2, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(d_req, reqs, b_req, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (ce = cudaMemsetAsync(d_err, 0, 4, st)) != cudaSuccess)
        rc = check_cuda(ce, "affine_mvp: upload");
    if (!rc) rc = launch_affine_mvp(ptr, (const long long *)d_ref, n_ref, (const short *)d_mv,
                                    (const signed char *)d_refi, i_scu, rows, d_req, n, d_out, (int *)d_err, st);
    if (!rc && ((ce = cudaMemcpyAsync(out, d_out, b_out, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
                (ce = cudaMemcpyAsync(&bad, d_err, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess))
        rc = check_cuda(ce, "affine_mvp: download");
    cudaFreeAsync(buf, st);
    ce = cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (rc) return rc;
    if (ce != cudaSuccess) return check_cuda(ce, "affine_mvp: synchronise");
    if (bad) return set_status(UC_ERR_ARG, "affine_mvp: requests outside the domain");
    return UC_OK;
}

// ---------------------------------------------------------------------------------------------
// Affine merge candidates: one thread per CU, the reference's derivation order.  Model-based
// candidates: the first two affine neighbours among F, G, C, A, D (same-CU duplicates dropped),
// each neighbour CU's corner MVs (found through its map_pos entry) extrapolated to the CU's
// corners in 1/128 units with the magnitude-rounding shift, a 4-parameter model when the
// neighbour's bottom edge is the CTU row boundary above the CU.  Constructed candidates: LT, RT,
// LB from the first inter neighbour of each corner, RB from the colocated picture (scaled by POC
// distances), combined in the 6 model orders while the list has room.  Every read of the maps is
// bounds-checked; a request with an out-of-field read gets a zeroed result and is counted.
// Records are assembled in shared memory and written out by the CTA as contiguous words.
// ---------------------------------------------------------------------------------------------
static_assert(sizeof(uavs3e_cuda_affmrg_req_t) == 8, "affine merge request layout");
static_assert(sizeof(uavs3e_cuda_affmrg_out_t) == 260, "affine merge result layout");
static_assert(sizeof(uavs3e_cuda_affmrg_pic_t) == 184, "affine merge picture layout");

struct AmrgMaps {
    const short *mv; const signed char *refi; const unsigned char *scu; const unsigned *pos;
    const short *col_mv; const signed char *col_refi;
    long long origin, nf;
};

struct AmrgReader {
    const AmrgMaps &M;
    bool bad;
    __device__ bool in(long long a)
    {
        const long long k = a + M.origin;
        if (k < 0 || k >= M.nf) { bad = true; return false; }
        return true;
    }
    __device__ int scu(long long a) { return in(a) ? M.scu[a + M.origin] : 0; }
    __device__ unsigned pos(long long a) { return in(a) ? M.pos[a + M.origin] : 0u; }
    __device__ int refi(long long a, int l) { return in(a) ? M.refi[(a + M.origin) * 2 + l] : -1; }
    __device__ int mv(long long a, int l, int d) { return in(a) ? M.mv[((a + M.origin) * 2 + l) * 2 + d] : 0; }
};

__device__ __forceinline__ int amrg_round7(int v)
{
    return v >= 0 ? (int)(((unsigned)v + 64u) >> 7) : -(int)(((unsigned)(-(long long)v) + 64u) >> 7);
}

__device__ __forceinline__ int amrg_clip18(int v) { return max(-131072, min(131071, v)); }

__device__ __forceinline__ int amrg_shl(int v, int s) { return (int)((unsigned)v << s); }

// scaling_mv1 of an MV (x, y): false on a zero POC distance
__device__ __forceinline__ bool amrg_scale(long long cur, long long cur_ref, long long neb, long long neb_ref, int mx,
                                           int my, int &ox, int &oy)
{
    const int t0 = (int)(neb * 2 - neb_ref * 2), t1 = (int)(cur * 2 - cur_ref * 2);
    if (t0 == 0 || t1 == 0) return false;
    const int ratio = (1 << 14) / t0 * t1;
    ox = amvp_scale(mx, ratio);
    oy = amvp_scale(my, ratio);
    return true;
}

// com_derive_affine_model_mv: control points of the CU at scup from the affine CU covering scun
__device__ void amrg_model(AmrgReader &R, const uavs3e_cuda_affmrg_pic_t &P, int scup, int scun, int l, int cw, int ch,
                           int (*mvp)[2], int &vn)
{
    const int i_scu = P.i_scu;
    const unsigned pos = R.pos(scun);
    const int lw = (int)(pos & 7), lh = (int)((pos >> 3) & 7), nw = 1 << lw, nh = 1 << lh;
    const int a0 = (int)(pos >> 6), a1 = a0 + ((nw >> 2) - 1), a2 = a0 + ((nh >> 2) - 1) * i_scu, a3 = a2 + ((nw >> 2) - 1);
    const int neb_x = (a0 % i_scu) << 2;
    int neb_y = (a0 / i_scu) << 2;
    const int cur_x = (scup % i_scu) << 2, cur_y = (scup / i_scu) << 2;
    int m0x = R.mv(a0, l, 0), m0y = R.mv(a0, l, 1), m1x = R.mv(a1, l, 0), m1y = R.mv(a1, l, 1);
    const int m2x = R.mv(a2, l, 0), m2y = R.mv(a2, l, 1), m3x = R.mv(a3, l, 0), m3y = R.mv(a3, l, 1);
    bool top = false;
    if ((neb_y + nh) % (1 << P.log2_max_cuwh) == 0 && neb_y + nh == cur_y) {
        top = true;
        neb_y += nh;
        m0x = m2x; m0y = m2y; m1x = m3x; m1y = m3y;
    }
    const int dhx = amrg_shl(m1x - m0x, 7 - lw), dhy = amrg_shl(m1y - m0y, 7 - lw);
    int dvx, dvy;
    if (vn == 3 && !top) {
        dvx = amrg_shl(m2x - m0x, 7 - lh);
        dvy = amrg_shl(m2y - m0y, 7 - lh);
    } else {
        dvx = -dhy;
        dvy = dhx;
        vn = 2;
    }
    const int hb = amrg_shl(m0x, 7), vb = amrg_shl(m0y, 7);
    for (int k = 0; k < vn; k++) {
        const int ox = cur_x - neb_x + (k == 1 ? cw : 0), oy = cur_y - neb_y + (k == 2 ? ch : 0);
        const int th = (int)((unsigned)dhx * (unsigned)ox + (unsigned)dvx * (unsigned)oy + (unsigned)hb);
        const int tv = (int)((unsigned)dhy * (unsigned)ox + (unsigned)dvy * (unsigned)oy + (unsigned)vb);
        mvp[k][0] = amrg_clip18(amrg_shl(amrg_round7(th), 2));
        mvp[k][1] = amrg_clip18(amrg_shl(amrg_round7(tv), 2));
    }
}

// com_derive_affine_constructed_candidate for the control points c0, c1[, c2] of model m
__device__ void amrg_construct(uavs3e_cuda_affmrg_out_t &o, int &cnt, int cw, int ch, const bool *valid,
                               const int (*cmv)[4][2], const int (*crefi)[4], int c0, int c1, int c2, int m, int ver)
{
    if (cnt >= 5) return;
    const int idx[3] = { c0, c1, c2 };
    for (int i = 0; i < ver; i++)
        if (!valid[idx[i]]) return;
    bool vm[2];
    for (int l = 0; l < 2; l++) {
        bool ok = true;
        for (int i = 0; i < ver; i++) ok = ok && crefi[l][idx[i]] >= 0 && crefi[l][idx[i]] == crefi[l][c0];
        vm[l] = ok;
    }
    if (!vm[0] && !vm[1]) return;
    o.cp_num[cnt] = (signed char)ver;
    const int sh = 7 + (31 - __clz(cw)) - (31 - __clz(ch));
    for (int l = 0; l < 2; l++) {
        if (!vm[l]) {
            o.refi[cnt][l] = -1;
            for (int i = 0; i < ver; i++) o.cpmv[cnt][l][i][0] = o.cpmv[cnt][l][i][1] = 0;
            continue;
        }
        int t[4][2] = { { 0, 0 }, { 0, 0 }, { 0, 0 }, { 0, 0 } };
        for (int i = 0; i < ver; i++) { t[idx[i]][0] = cmv[l][idx[i]][0]; t[idx[i]][1] = cmv[l][idx[i]][1]; }
        for (int d = 0; d < 2; d++) {
            if (m == 1) t[2][d] = t[3][d] + t[0][d] - t[1][d];
            if (m == 2) t[1][d] = t[3][d] + t[0][d] - t[2][d];
            if (m == 3) t[0][d] = t[1][d] + t[2][d] - t[3][d];
        }
        if (m == 5) {
            const int th = (int)((unsigned)amrg_shl(t[2][1] - t[0][1], sh) + (unsigned)amrg_shl(t[0][0], 7));
            const int tv = (int)((unsigned)(-amrg_shl(t[2][0] - t[0][0], sh)) + (unsigned)amrg_shl(t[0][1], 7));
            t[1][0] = amrg_round7(th);
            t[1][1] = amrg_round7(tv);
        }
        o.refi[cnt][l] = (signed char)crefi[l][c0];
        for (int i = 0; i < ver; i++)
            for (int d = 0; d < 2; d++) o.cpmv[cnt][l][i][d] = amrg_clip18(amrg_shl(t[i][d], 2));
    }
    cnt++;
}

__device__ bool amrg_one(const uavs3e_cuda_affmrg_pic_t &P, const AmrgMaps &M, const uavs3e_cuda_affmrg_req_t q,
                         uavs3e_cuda_affmrg_out_t &o)
{
    const int cw = q.cu_width, ch = q.cu_height;
    if ((cw != 16 && cw != 32 && cw != 64 && cw != 128) || (ch != 16 && ch != 32 && ch != 64 && ch != 128)) return false;
    AmrgReader R{ M, false };
    const int i_scu = P.i_scu, scup = q.scup, wsc = cw >> 2, hsc = ch >> 2;
    int cnt = 0;
    {
        const int nb[5] = { scup + i_scu * (hsc - 1) - 1, scup - i_scu + wsc - 1, scup - i_scu + wsc, scup - 1,
                            scup - i_scu - 1 };
        int aff[5], tl[5];
        bool valid[5];
        for (int k = 0; k < 5; k++) {
            aff[k] = (R.scu(nb[k]) >> 4) & 3;
            valid[k] = aff[k] != 0;
            tl[k] = valid[k] ? (int)(R.pos(nb[k]) >> 6) : 0;
        }
        if (valid[2] && valid[1] && tl[1] == tl[2]) valid[2] = false;
        const bool v3 = valid[3];
        if (valid[3] && valid[0] && tl[0] == tl[3]) valid[3] = false;
        if ((valid[4] && v3 && tl[4] == tl[3]) || (valid[4] && valid[1] && tl[4] == tl[1])) valid[4] = false;
        for (int k = 0; k < 5 && cnt < 2; k++) {
            if (!valid[k]) continue;
            int vn = aff[k] == 1 ? 2 : 3;
            for (int l = 0; l < 2; l++) {
                const int r = R.refi(nb[k], l);
                if (r >= 0) {
                    o.refi[cnt][l] = (signed char)r;
                    amrg_model(R, P, scup, nb[k], l, cw, ch, o.cpmv[cnt][l], vn);
                } else {
                    o.refi[cnt][l] = -1;
                    for (int i = 0; i < 3; i++) o.cpmv[cnt][l][i][0] = o.cpmv[cnt][l][i][1] = 0;
                }
            }
            o.cp_num[cnt] = (signed char)vn;
            cnt++;
        }
    }
    {
        int cmv[2][4][2], crefi[2][4];
        bool valid[4] = { false, false, false, false };
        for (int l = 0; l < 2; l++)
            for (int i = 0; i < 4; i++) { cmv[l][i][0] = cmv[l][i][1] = 0; crefi[l][i] = -1; }
        const int corner[6] = { scup - 1, scup - i_scu, scup - i_scu - 1, scup - i_scu + wsc - 1, scup - i_scu + wsc,
                                scup + i_scu * (hsc - 1) - 1 };
        const int first[4] = { 0, 3, 5, 6 };
        for (int g = 0; g < 3; g++) {
            for (int k = first[g]; k < first[g + 1]; k++) {
                const int a = corner[k];
                if ((R.scu(a) & 3) != 1) continue;
                for (int l = 0; l < 2; l++) {
                    crefi[l][g] = R.refi(a, l);
                    cmv[l][g][0] = R.mv(a, l, 0);
                    cmv[l][g][1] = R.mv(a, l, 1);
                }
                valid[g] = true;
                break;
            }
        }
        const int rb = scup + i_scu * (hsc - 1) + (wsc - 1);
        const int bx = rb % i_scu, by = rb / i_scu;
        int xpos = (bx & ~3) + 2, ypos = (by & ~3) + 2;
        if (ypos >= P.pic_height_in_scu) ypos = ((by & ~3) + P.pic_height_in_scu) >> 1;
        if (xpos >= P.pic_width_in_scu) xpos = ((bx & ~3) + P.pic_width_in_scu) >> 1;
        const long long co = (long long)ypos * i_scu + xpos + M.origin;
        if (co < 0 || co >= M.nf) return false;
        const int cr = M.col_refi[co * 2];
        const int cx = M.col_mv[co * 4 + 0], cy = M.col_mv[co * 4 + 1];
        if (cr >= 17) return false;
        if (cr >= 0) {
            if (P.slice_type == 3) {
                for (int l = 0; l < 2; l++) {
                    if (!amrg_scale(P.ptr, P.ref0_ptr[l], P.ref0_ptr[1], P.col_list_ptr[cr], cx, cy, cmv[l][3][0], cmv[l][3][1]))
                        return false;
                    crefi[l][3] = 0;
                }
            } else {
                if (!amrg_scale(P.ptr, P.ref0_ptr[0], P.ref0_ptr[0], P.col_list_ptr[cr], cx, cy, cmv[0][3][0], cmv[0][3][1]))
                    return false;
                crefi[0][3] = 0;
                crefi[1][3] = -1;
            }
            valid[3] = true;
        }
        amrg_construct(o, cnt, cw, ch, valid, cmv, crefi, 0, 1, 2, 0, 3);
        amrg_construct(o, cnt, cw, ch, valid, cmv, crefi, 0, 1, 3, 1, 3);
        amrg_construct(o, cnt, cw, ch, valid, cmv, crefi, 0, 2, 3, 2, 3);
        amrg_construct(o, cnt, cw, ch, valid, cmv, crefi, 1, 2, 3, 3, 3);
        amrg_construct(o, cnt, cw, ch, valid, cmv, crefi, 0, 1, 0, 4, 2);
        amrg_construct(o, cnt, cw, ch, valid, cmv, crefi, 0, 2, 0, 5, 2);
    }
    o.num = cnt;
    for (int k = cnt; k < 5; k++) {
        o.cp_num[k] = 2;
        o.refi[k][0] = 0;
        o.refi[k][1] = -1;
    }
    for (int k = 0; k < 5; k++)
        for (int l = 0; l < 2; l++)
            for (int i = (k < cnt ? o.cp_num[k] : 0); i < 3; i++) o.cpmv[k][l][i][0] = o.cpmv[k][l][i][1] = 0;
    return !R.bad;
}

constexpr int AMRG_THREADS = 128;

__global__ void __launch_bounds__(AMRG_THREADS) k_affine_merge(const uavs3e_cuda_affmrg_pic_t P, AmrgMaps M,
                                                              const uavs3e_cuda_affmrg_req_t *reqs, int n,
                                                              uavs3e_cuda_affmrg_out_t *out, int *err)
{
    __shared__ uavs3e_cuda_affmrg_out_t s_out[AMRG_THREADS];
    const int base = blockIdx.x * AMRG_THREADS, i = base + threadIdx.x;
    if (i < n) {
        uavs3e_cuda_affmrg_out_t o;
        memset(&o, 0, sizeof(o));
        if (!amrg_one(P, M, reqs[i], o)) {
            memset(&o, 0, sizeof(o));
            if (err) atomicAdd(err, 1);
        }
        s_out[threadIdx.x] = o;
    }
    __syncthreads();
    // the CTA's records are contiguous: copy them out as words
    const int nrec = min(AMRG_THREADS, n - base);
    const unsigned *src = reinterpret_cast<const unsigned *>(s_out);
    unsigned *dst = reinterpret_cast<unsigned *>(out + base);
    const int words = nrec * (int)(sizeof(uavs3e_cuda_affmrg_out_t) / 4);
    for (int w = threadIdx.x; w < words; w += AMRG_THREADS) dst[w] = src[w];
}

int launch_affine_merge(const uavs3e_cuda_affmrg_pic_t &pic, const short *d_mv, const signed char *d_refi,
                        const unsigned char *d_scu, const unsigned *d_pos, const short *d_col_mv,
                        const signed char *d_col_refi, const uavs3e_cuda_affmrg_req_t *d_reqs, int n,
                        uavs3e_cuda_affmrg_out_t *d_out, int *d_err, cudaStream_t st)
{
    if (n < 0 || pic.i_scu < 3 || pic.rows < 2 || pic.pic_width_in_scu < 1 || pic.pic_height_in_scu < 1 ||
        pic.log2_max_cuwh < 2 || pic.log2_max_cuwh > 7 ||
        (n > 0 && (!d_mv || !d_refi || !d_scu || !d_pos || !d_col_mv || !d_col_refi || !d_reqs || !d_out)))
        return set_status(UC_ERR_ARG, "affine_merge: bad argument");
    if (((uintptr_t)d_mv & 3) || ((uintptr_t)d_col_mv & 3) || ((uintptr_t)d_pos & 3) || ((uintptr_t)d_out & 3))
        return set_status(UC_ERR_ARG, "affine_merge: map_mv, col_mv, map_pos or out not 4-byte aligned");
    if (n == 0) return UC_OK;
    AmrgMaps M{ d_mv, d_refi, d_scu, d_pos, d_col_mv, d_col_refi, (long long)pic.i_scu + 1,
                (long long)pic.rows * pic.i_scu };
    k_affine_merge<<<(n + AMRG_THREADS - 1) / AMRG_THREADS, AMRG_THREADS, 0, st>>>(pic, M, d_reqs, n, d_out, d_err);
    UC_CHECK(cudaGetLastError());
    count_launch(1);
    return UC_OK;
}

UAVS3E_CUDA_API int uavs3e_cuda_affine_merge_device(const uavs3e_cuda_affmrg_pic_t *pic, const int16_t *d_map_mv,
                                                    const int8_t *d_map_refi, const uint8_t *d_map_scu,
                                                    const uint32_t *d_map_pos, const int16_t *d_col_mv,
                                                    const int8_t *d_col_refi, const uavs3e_cuda_affmrg_req_t *d_reqs,
                                                    int n, uavs3e_cuda_affmrg_out_t *d_out, int32_t *d_err,
                                                    void *stream)
{
    if (ensure_init()) return uavs3e_cuda_status();
    if (!pic) return set_status(UC_ERR_ARG, "affine_merge: bad argument");
    return launch_affine_merge(*pic, d_map_mv, (const signed char *)d_map_refi, d_map_scu, d_map_pos, d_col_mv,
                               (const signed char *)d_col_refi, d_reqs, n, d_out, (int *)d_err, (cudaStream_t)stream);
}

UAVS3E_CUDA_API int uavs3e_cuda_affine_merge(const uavs3e_cuda_affmrg_pic_t *pic, const int16_t *map_mv,
                                             const int8_t *map_refi, const uint8_t *map_scu,
                                             const uint32_t *map_pos, const int16_t *col_mv, const int8_t *col_refi,
                                             const uavs3e_cuda_affmrg_req_t *reqs, int n,
                                             uavs3e_cuda_affmrg_out_t *out)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (!pic || n < 0 || pic->i_scu < 3 || pic->rows < 2 ||
        (n > 0 && (!map_mv || !map_refi || !map_scu || !map_pos || !col_mv || !col_refi || !reqs || !out)))
        return set_status(UC_ERR_ARG, "affine_merge: bad argument");
    if (n == 0) return UC_OK;
    const size_t field = (size_t)pic->rows * pic->i_scu;
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t b_mv = up(field * 8), b_refi = up(field * 2), b_scu = up(field), b_pos = up(field * 4);
    const size_t b_req = up((size_t)n * sizeof(uavs3e_cuda_affmrg_req_t)), b_out = up((size_t)n * sizeof(uavs3e_cuda_affmrg_out_t));
    cudaStream_t st = nullptr;
    UC_CHECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    char *buf = nullptr;
    cudaError_t ce = cudaMallocAsync((void **)&buf, 2 * b_mv + 2 * b_refi + b_scu + b_pos + b_req + b_out + 256, st);
    if (ce != cudaSuccess) { cudaStreamDestroy(st); return check_cuda(ce, "affine_merge: allocate"); }
    char *d_mv = buf, *d_refi = d_mv + b_mv, *d_scu = d_refi + b_refi, *d_pos = d_scu + b_scu;
    char *d_cmv = d_pos + b_pos, *d_crefi = d_cmv + b_mv, *d_req = d_crefi + b_refi, *d_out = d_req + b_req;
    char *d_err = d_out + b_out;
    int bad = 0;
    rc = UC_OK;
    if ((ce = cudaMemcpyAsync(d_mv, map_mv, field * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(d_refi, map_refi, field * 2, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(d_scu, map_scu, field, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(d_pos, map_pos, field * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(d_cmv, col_mv, field * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(d_crefi, col_refi, field * 2, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(d_req, reqs, (size_t)n * sizeof(uavs3e_cuda_affmrg_req_t), cudaMemcpyHostToDevice, st)) !=
            cudaSuccess ||
        (ce = cudaMemsetAsync(d_err, 0, 4, st)) != cudaSuccess)
        rc = check_cuda(ce, "affine_merge: upload");
    if (!rc)
        rc = launch_affine_merge(*pic, (const short *)d_mv, (const signed char *)d_refi, (const unsigned char *)d_scu,
                                 (const unsigned *)d_pos, (const short *)d_cmv, (const signed char *)d_crefi,
                                 (const uavs3e_cuda_affmrg_req_t *)d_req, n, (uavs3e_cuda_affmrg_out_t *)d_out,
                                 (int *)d_err, st);
    if (!rc && ((ce = cudaMemcpyAsync(out, d_out, (size_t)n * sizeof(uavs3e_cuda_affmrg_out_t), cudaMemcpyDeviceToHost,
                                      st)) != cudaSuccess ||
                (ce = cudaMemcpyAsync(&bad, d_err, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess))
        rc = check_cuda(ce, "affine_merge: download");
    cudaFreeAsync(buf, st);
    ce = cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (rc) return rc;
    if (ce != cudaSuccess) return check_cuda(ce, "affine_merge: synchronise");
    if (bad) return set_status(UC_ERR_ARG, "affine_merge: requests outside the domain");
    return UC_OK;
}
