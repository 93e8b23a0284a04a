// CU motion compensation for lists of CUs: com_mc_cu (src/com_mc.c:140-200) with hp_flag 0 --
// luma copied from the reference's quarter-sample plane (com_mc_blk_luma :41-87), chroma by the
// 4-tap filters at 1/8-sample positions (com_mc_blk_chroma :103-138: copy, ipflt H_4 / V_4,
// ipflt_ext EXT_4), the two lists averaged (pel_avrg) -- bit-exact with the reference.
//
// Affine CUs: com_mc_cu_affine (:361-422) -- sub-block MVs from the control points, luma by the
// 16-phase 8-tap filters, chroma by the 32-phase 4-tap filters, 1/16-sample positions.
//
// One warp per CU; lanes walk the CU's samples in raster order, so every store of the warp is
// one contiguous run of the output buffer.
#include "common.cuh"
#include "affine.cuh"
#include "uavs3e_cuda_internal.h"
#include "../../include/uavs3e_cuda.h"

#include <string.h>

namespace uc {

constexpr int MC_WARPS = 8;

struct McReq {
    s16 x, y; u8 w, h; s8 slot[2]; s16 mv[2][2]; u8 channel; u8 pad[3]; u32 out_offset;
};
static_assert(sizeof(McReq) == sizeof(uavs3e_cuda_mc_req_t), "request layout");

struct McParams {
    const pel *planes[UAVS3E_CUDA_TZ_MAX_SLOTS * 16];
    const pel *chroma[UAVS3E_CUDA_TZ_MAX_SLOTS * 2];
    int i_ref, i_c, n_slots, W, H;
    const McReq *reqs;
    int n;
    pel *out;
    unsigned long long out_bytes;
};

// 4-tap chroma filters at the 8 eighth-sample phases (com_tbl_mc_c_coeff, src/com_tables.c)
__device__ __constant__ static const s8 kMcChroma[8][4] = {
    { 0, 64, 0, 0 }, { -4, 62, 6, 0 }, { -6, 56, 15, -1 }, { -5, 47, 25, -3 },
    { -4, 36, 36, -4 }, { -3, 25, 47, -5 }, { -1, 15, 56, -6 }, { 0, 6, 62, -4 },
};

// one chroma prediction sample: src at the block's integer position (i, j) of the sample
__device__ __forceinline__ int mc_chroma_sample(const pel *s, int ic, int dx, int dy)
{
    if (!dx && !dy) return s[0];
    if (!dy) {
        const int v = s[-1] * kMcChroma[dx][0] + s[0] * kMcChroma[dx][1] + s[1] * kMcChroma[dx][2] +
                      s[2] * kMcChroma[dx][3];
        return min(255, max(0, (v + 32) >> 6));
    }
    if (!dx) {
        const int v = s[-ic] * kMcChroma[dy][0] + s[0] * kMcChroma[dy][1] + s[ic] * kMcChroma[dy][2] +
                      s[2 * ic] * kMcChroma[dy][3];
        return min(255, max(0, (v + 32) >> 6));
    }
    // two passes: horizontal into 16 bits (8-bit: no rounding), vertical (sum + 2048) >> 12
    int v = 0;
#pragma unroll
    for (int t = 0; t < 4; t++) {
        const pel *r = s + (t - 1) * ic;
        const int hs = r[-1] * kMcChroma[dx][0] + r[0] * kMcChroma[dx][1] + r[1] * kMcChroma[dx][2] +
                       r[2] * kMcChroma[dx][3];
        v += (int)(s16)hs * kMcChroma[dy][t];
    }
    return min(255, max(0, (v + 2048) >> 12));
}

__global__ void __launch_bounds__(32 * MC_WARPS) k_mc_cu(const McParams P)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.x * MC_WARPS + warp;
    if (r >= P.n) return;
    const McReq q = P.reqs[r];
    const int w = q.w, h = q.h, wc = w >> 1, hc = h >> 1;
    const bool luma = q.channel != 2, chroma = q.channel != 1;
    const int nl = (q.slot[0] >= 0) + (q.slot[1] >= 0);
    const unsigned long long size = (luma ? w * h : 0) + (chroma ? w * h / 2 : 0);
    // CUs outside the supported domain are skipped (nothing written)
    if ((w != 8 && w != 16 && w != 32 && w != 64) || (h != 8 && h != 16 && h != 32 && h != 64) || q.x < 0 ||
        q.y < 0 || q.x + w > P.W || q.y + h > P.H || q.channel > 2 || nl == 0 || q.slot[0] >= P.n_slots ||
        q.slot[1] >= P.n_slots || (unsigned long long)q.out_offset + size > P.out_bytes)
        return;
    pel *o = P.out + q.out_offset;
    if (luma) {
        const pel *src[2];
        int k = 0;
        for (int l = 0; l < 2; l++) {
            if (q.slot[l] < 0) continue;
            const int qx = (q.x << 2) + q.mv[l][0], qy = (q.y << 2) + q.mv[l][1];
            const int px = min(max(qx >> 2, -128 - 4), P.W + 4), py = min(max(qy >> 2, -128 - 4), P.H + 4);
            src[k++] = P.planes[q.slot[l] * 16 + (qy & 3) * 4 + (qx & 3)] + (long long)py * P.i_ref + px;
        }
        // 4 samples a lane: word loads from the (any-alignment) source rows, byte-wise rounded
        // average of the two lists (pel_avrg), word stores where the output is 4-byte aligned
        const int lq = 31 - __clz(w >> 2);           // log2 of the words per row
        const bool aligned = ((uintptr_t)o & 3) == 0;
        for (int i = lane; i < (w * h) >> 2; i += 32) {
            const int j = i >> lq, c = (i - (j << lq)) << 2;
            u32 v = 0;
            for (int t = 0; t < k; t++) {
                const uintptr_t a = (uintptr_t)(src[t] + j * P.i_ref + c);
                const u32 *wp = (const u32 *)(a & ~(uintptr_t)3);
                const u32 sv = __funnelshift_r(__ldg(wp), __ldg(wp + 1), (u32)(a & 3) * 8);
                v = t ? __vavgu4(v, sv) : sv;
            }
            pel *d = o + (i << 2);
            if (aligned) *(u32 *)d = v;
            else { d[0] = (pel)v; d[1] = (pel)(v >> 8); d[2] = (pel)(v >> 16); d[3] = (pel)(v >> 24); }
        }
        o += w * h;
    }
    if (chroma) {
        for (int pl = 0; pl < 2; pl++, o += wc * hc) {
            const pel *src[2];
            int dx[2], dy[2], k = 0;
            for (int l = 0; l < 2; l++) {
                if (q.slot[l] < 0) continue;
                const int qx = (q.x << 2) + q.mv[l][0], qy = (q.y << 2) + q.mv[l][1];
                const int cx = min(max(qx >> 3, -64 - 2), (P.W + 4) >> 1), cy = min(max(qy >> 3, -64 - 2), (P.H + 4) >> 1);
                dx[k] = qx & 7; dy[k] = qy & 7;
                src[k++] = P.chroma[q.slot[l] * 2 + pl] + (long long)cy * P.i_c + cx;
            }
            const int lwc = 31 - __clz(wc);
            for (int i = lane; i < wc * hc; i += 32) {
                const int j = i >> lwc, c = i - (j << lwc);
                int v = mc_chroma_sample(src[0] + j * P.i_c + c, P.i_c, dx[0], dy[0]);
                if (k == 2) v = (v + mc_chroma_sample(src[1] + j * P.i_c + c, P.i_c, dx[1], dy[1]) + 1) >> 1;
                o[i] = (pel)v;
            }
        }
    }
}

// ------------------------------------------------------------------ affine CUs
struct AffReq {
    s16 x, y; u8 w, h; s8 slot[2]; u8 cp_num; u8 sub8; u8 pad[2]; s32 cpmv[2][3][2]; u32 out_offset;
};
static_assert(sizeof(AffReq) == sizeof(uavs3e_cuda_affine_req_t), "affine request layout");

// 1/32-sample chroma filters (com_tbl_mc_c_coeff_hp, src/com_tables.c:156-189)
__device__ __constant__ static const s8 kMcChromaHp[32][4] = {
    { 0, 64, 0, 0 },    { -1, 63, 2, 0 },   { -2, 62, 4, 0 },   { -2, 60, 7, -1 },  { -2, 58, 10, -2 },
    { -3, 57, 12, -2 }, { -4, 56, 14, -2 }, { -4, 55, 15, -2 }, { -4, 54, 16, -2 }, { -5, 53, 18, -2 },
    { -6, 52, 20, -2 }, { -6, 49, 24, -3 }, { -6, 46, 28, -4 }, { -5, 44, 29, -4 }, { -4, 42, 30, -4 },
    { -4, 39, 33, -4 }, { -4, 36, 36, -4 }, { -4, 33, 39, -4 }, { -4, 30, 42, -4 }, { -4, 29, 44, -5 },
    { -4, 28, 46, -6 }, { -3, 24, 49, -6 }, { -2, 20, 52, -6 }, { -2, 18, 53, -5 }, { -2, 16, 54, -4 },
    { -2, 15, 55, -4 }, { -2, 14, 56, -4 }, { -2, 12, 57, -3 }, { -2, 10, 58, -2 }, { -1, 7, 60, -2 },
    { 0, 4, 62, -2 },   { 0, 2, 63, -1 },
};

__device__ __forceinline__ int aff_chroma_sample(const pel *s, int ic, int dx, int dy)
{
    if (!dx && !dy) return s[0];
    if (!dy) {
        const int v = s[-1] * kMcChromaHp[dx][0] + s[0] * kMcChromaHp[dx][1] + s[1] * kMcChromaHp[dx][2] +
                      s[2] * kMcChromaHp[dx][3];
        return min(255, max(0, (v + 32) >> 6));
    }
    if (!dx) {
        const int v = s[-ic] * kMcChromaHp[dy][0] + s[0] * kMcChromaHp[dy][1] + s[ic] * kMcChromaHp[dy][2] +
                      s[2 * ic] * kMcChromaHp[dy][3];
        return min(255, max(0, (v + 32) >> 6));
    }
    int v = 0;
#pragma unroll
    for (int t = 0; t < 4; t++) {
        const pel *r = s + (t - 1) * ic;
        const int hs = r[-1] * kMcChromaHp[dx][0] + r[0] * kMcChromaHp[dx][1] + r[1] * kMcChromaHp[dx][2] +
                       r[2] * kMcChromaHp[dx][3];
        v += (int)(s16)hs * kMcChromaHp[dy][t];
    }
    return min(255, max(0, (v + 2048) >> 12));
}


// the sub-block MVs of one list (com_mc_blk_affine, src/com_mc.c:256-330) into mv[16][16] per
// 4x4 unit (8x8 sub-blocks fill their four units)
__device__ void aff_subblock_mvs(const AffReq &q, int l, int sub, s32 (*mv)[16][2], int lane)
{
    const int cw = q.w, ch = q.h, lw = 31 - __clz(cw), lh = 31 - __clz(ch), half = sub >> 1;
    const s32 *a0 = q.cpmv[l][0], *a1 = q.cpmv[l][1], *a2 = q.cpmv[l][2];
    const s32 dhx = ((a1[0] - a0[0]) * 128) >> lw, dhy = ((a1[1] - a0[1]) * 128) >> lw;
    s32 dvx = -dhy, dvy = dhx;
    if (q.cp_num == 3) { dvx = ((a2[0] - a0[0]) * 128) >> lh; dvy = ((a2[1] - a0[1]) * 128) >> lh; }
    const int nx = cw / sub, n = nx * (ch / sub);
    for (int b = lane; b < n; b += 32) {
        const int w = (b % nx) * sub, h = (b / nx) * sub;
        int px = w + half, py = h + half;
        if (w == 0 && h == 0) { px = 0; py = 0; }
        else if (w + sub == cw && h == 0) { px = cw; py = 0; }
        else if (w == 0 && h + sub == ch && q.cp_num == 3) { px = 0; py = ch; }
        const s32 mx = min(max(aff_round7(a0[0] * 128 + dhx * px + dvx * py), -131072), 131071);
        const s32 my = min(max(aff_round7(a0[1] * 128 + dhy * px + dvy * py), -131072), 131071);
        for (int j = 0; j < sub / 4; j++)
            for (int i = 0; i < sub / 4; i++) { mv[(w >> 2) + i][(h >> 2) + j][0] = mx; mv[(w >> 2) + i][(h >> 2) + j][1] = my; }
    }
}

constexpr int AFF_WARPS = 4;

__global__ void __launch_bounds__(32 * AFF_WARPS) k_mc_affine(const McParams P, const AffReq *reqs)
{
    __shared__ s32 s_mv[AFF_WARPS][2][16][16][2];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.x * AFF_WARPS + warp;
    if (r >= P.n) return;
    const AffReq q = reqs[r];
    const int w = q.w, h = q.h, nl = (q.slot[0] >= 0) + (q.slot[1] >= 0);
    if ((w != 16 && w != 32 && w != 64) || (h != 16 && h != 32 && h != 64) || q.x < 0 || q.y < 0 ||
        q.x + w > P.W || q.y + h > P.H || (q.cp_num != 2 && q.cp_num != 3) || nl == 0 || q.slot[0] >= P.n_slots ||
        q.slot[1] >= P.n_slots || (unsigned long long)q.out_offset + (unsigned long long)(w * h * 3 / 2) > P.out_bytes)
        return;
    const int sub = (q.sub8 == 1 || nl == 2) ? 8 : 4;
    int ls[2], k = 0;
    for (int l = 0; l < 2; l++)
        if (q.slot[l] >= 0) { aff_subblock_mvs(q, l, sub, s_mv[warp][k], lane); ls[k++] = l; }
    __syncwarp();
    pel *o = P.out + q.out_offset;
    // luma: 16-phase filters per sub-block MV, a lane per column of a band of sub-blocks
    const int tasks = w * (h / sub);
    for (int t = lane; t < tasks; t += 32) {
        const int c = t % w, by = (t / w) * sub, bx = c & ~(sub - 1);
        int acc[8];
        for (int u = 0; u < k; u++) {
            const s32 *m = s_mv[warp][u][c >> 2][by >> 2];
            const int qx = ((q.x + bx) << 4) + m[0], qy = ((q.y + by) << 4) + m[1];
            const pel *plane = P.planes[q.slot[ls[u]] * 16];
            int v[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
            if (sub == 8) aff_luma_column<8>(plane, P.i_ref, P.W, P.H, qx, qy, c - bx, v);
            else aff_luma_column<4>(plane, P.i_ref, P.W, P.H, qx, qy, c - bx, v);
#pragma unroll
            for (int i = 0; i < 8; i++) acc[i] = u ? (acc[i] + v[i] + 1) >> 1 : v[i];
        }
        for (int i = 0; i < sub; i++) o[(by + i) * w + c] = (pel)acc[i];
    }
    o += w * h;
    // chroma: 4x4 blocks per 8x8 luma with the rounded mean of their four 4x4 MVs
    const int wc = w >> 1, hc = h >> 1;
    for (int pl = 0; pl < 2; pl++, o += wc * hc)
        for (int i = lane; i < wc * hc; i += 32) {
            const int j = i / wc, c = i - j * wc;
            const int lx = (c >> 2) << 3, ly = (j >> 2) << 3, us = lx >> 2, vs = ly >> 2;
            int v = 0;
            for (int t = 0; t < k; t++) {
                const s32 (*m)[16][2] = s_mv[warp][t];
                const s32 mx = (m[us][vs][0] + m[us + 1][vs][0] + m[us][vs + 1][0] + m[us + 1][vs + 1][0] + 2) >> 2;
                const s32 my = (m[us][vs][1] + m[us + 1][vs][1] + m[us][vs + 1][1] + m[us + 1][vs + 1][1] + 2) >> 2;
                const int qx = ((q.x + lx) << 4) + mx, qy = ((q.y + ly) << 4) + my;
                const int cx = min(max(qx >> 5, -64 - 2), (P.W + 4) >> 1), cy = min(max(qy >> 5, -64 - 2), (P.H + 4) >> 1);
                const pel *s = P.chroma[q.slot[ls[t]] * 2 + pl] + (long long)(cy + (j & 3)) * P.i_c + cx + (c & 3);
                const int sv = aff_chroma_sample(s, P.i_c, qx & 31, qy & 31);
                v = t ? (v + sv + 1) >> 1 : sv;
            }
            o[i] = (pel)v;
        }
}

int launch_mc_affine(int W, int H, const pel *const *planes, int n_slots, int i_ref, int pad,
                     const pel *const *chroma, int i_c, int pad_c, const void *reqs, int n, pel *out,
                     unsigned long long out_bytes, cudaStream_t st)
{
    if (!planes || !chroma || !reqs || !out || n < 0) return set_status(UC_ERR_ARG, "mc_affine: null argument");
    if (n_slots < 1 || n_slots > UAVS3E_CUDA_TZ_MAX_SLOTS || W < 16 || H < 16)
        return set_status(UC_ERR_ARG, "mc_affine: slots / picture size");
    // luma taps reach 132 + 3 samples before the picture, chroma 66 + 1
    if (pad < 144 || pad_c < 72 || i_ref < W + 2 * pad || i_c < (W >> 1) + 2 * pad_c)
        return set_status(UC_ERR_ARG, "mc_affine: padding (luma >= 144, chroma >= 72) / strides");
    if (n == 0) return UC_OK;
    McParams P;
    memset(&P, 0, sizeof(P));
    for (int i = 0; i < n_slots * 16; i++) {
        if (!planes[i]) return set_status(UC_ERR_ARG, "mc_affine: null plane");
        P.planes[i] = planes[i];
    }
    for (int i = 0; i < n_slots * 2; i++) {
        if (!chroma[i]) return set_status(UC_ERR_ARG, "mc_affine: null chroma plane");
        P.chroma[i] = chroma[i];
    }
    P.i_ref = i_ref; P.i_c = i_c; P.n_slots = n_slots; P.W = W; P.H = H;
    P.n = n; P.out = out; P.out_bytes = out_bytes;
    prof_begin(PROF_MC, st);
    k_mc_affine<<<(unsigned)((n + AFF_WARPS - 1) / AFF_WARPS), 32 * AFF_WARPS, 0, st>>>(P, (const AffReq *)reqs);
    UC_CHECK(cudaGetLastError());
    count_launch(1);
    prof_end(PROF_MC, st);
    return UC_OK;
}

int launch_mc_cu(int W, int H, const pel *const *planes, int n_slots, int i_ref, int pad, const pel *const *chroma,
                 int i_c, int pad_c, const void *reqs, int n, pel *out, unsigned long long out_bytes, cudaStream_t st)
{
    if (!planes || !chroma || !reqs || !out || n < 0) return set_status(UC_ERR_ARG, "mc_cu: null argument");
    if (n_slots < 1 || n_slots > UAVS3E_CUDA_TZ_MAX_SLOTS || W < 8 || H < 8)
        return set_status(UC_ERR_ARG, "mc_cu: slots / picture size");
    // reads reach 132 luma samples before the picture and 67 chroma samples (clipped positions,
    // filter taps), and up to 68 / 36 beyond its far edges
    if (pad < 144 || pad_c < 72 || i_ref < W + 2 * pad || i_c < (W >> 1) + 2 * pad_c)
        return set_status(UC_ERR_ARG, "mc_cu: padding (luma >= 144, chroma >= 72) / strides");
    if (n == 0) return UC_OK;
    McParams P;
    memset(&P, 0, sizeof(P));
    for (int i = 0; i < n_slots * 16; i++) {
        if (!planes[i]) return set_status(UC_ERR_ARG, "mc_cu: null plane");
        P.planes[i] = planes[i];
    }
    for (int i = 0; i < n_slots * 2; i++) {
        if (!chroma[i]) return set_status(UC_ERR_ARG, "mc_cu: null chroma plane");
        P.chroma[i] = chroma[i];
    }
    P.i_ref = i_ref; P.i_c = i_c; P.n_slots = n_slots; P.W = W; P.H = H;
    P.reqs = (const McReq *)reqs; P.n = n; P.out = out; P.out_bytes = out_bytes;
    prof_begin(PROF_MC, st);
    k_mc_cu<<<(unsigned)((n + MC_WARPS - 1) / MC_WARPS), 32 * MC_WARPS, 0, st>>>(P);
    UC_CHECK(cudaGetLastError());
    count_launch(1);
    prof_end(PROF_MC, st);
    return UC_OK;
}

}  // namespace uc

using namespace uc;

extern "C" UAVS3E_CUDA_API int uavs3e_cuda_mc_affine_device(int width, int height, const uint8_t *const *d_planes,
                                                            int n_slots, int i_ref, int pad,
                                                            const uint8_t *const *d_chroma, int i_c, int pad_c,
                                                            const uavs3e_cuda_affine_req_t *d_reqs, int n,
                                                            uint8_t *d_out, size_t out_bytes, void *stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    return launch_mc_affine(width, height, d_planes, n_slots, i_ref, pad, d_chroma, i_c, pad_c, d_reqs, n, d_out,
                            (unsigned long long)out_bytes, (cudaStream_t)stream);
}

extern "C" UAVS3E_CUDA_API int uavs3e_cuda_mc_cu_device(int width, int height, const uint8_t *const *d_planes,
                                                        int n_slots, int i_ref, int pad,
                                                        const uint8_t *const *d_chroma, int i_c, int pad_c,
                                                        const uavs3e_cuda_mc_req_t *d_reqs, int n, uint8_t *d_out,
                                                        size_t out_bytes, void *stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    return launch_mc_cu(width, height, d_planes, n_slots, i_ref, pad, d_chroma, i_c, pad_c, d_reqs, n, d_out,
                        (unsigned long long)out_bytes, (cudaStream_t)stream);
}
