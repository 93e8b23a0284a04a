// CU motion compensation for lists of CUs: com_mc_cu (src/com_mc.c:140-200) with hp_flag 0 --
// luma copied from the reference's quarter-sample plane (com_mc_blk_luma :41-87), chroma by the
// 4-tap filters at 1/8-sample positions (com_mc_blk_chroma :103-138: copy, ipflt H_4 / V_4,
// ipflt_ext EXT_4), the two lists averaged (pel_avrg) -- bit-exact with the reference.
//
// One warp per CU; lanes walk the CU's samples in raster order, so every store of the warp is
// one contiguous run of the output buffer.
#include "common.cuh"
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
        for (int i = lane; i < w * h; i += 32) {
            const int j = i / w, c = i - j * w;
            int v = src[0][j * P.i_ref + c];
            if (k == 2) v = (v + src[1][j * P.i_ref + c] + 1) >> 1;
            o[i] = (pel)v;
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
            for (int i = lane; i < wc * hc; i += 32) {
                const int j = i / wc, c = i - j * wc;
                int v = mc_chroma_sample(src[0] + j * P.i_c + c, P.i_c, dx[0], dy[0]);
                if (k == 2) v = (v + mc_chroma_sample(src[1] + j * P.i_c + c, P.i_c, dx[1], dy[1]) + 1) >> 1;
                o[i] = (pel)v;
            }
        }
    }
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
