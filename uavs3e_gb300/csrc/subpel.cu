// Frame-level quarter-sample interpolation: the 15 fractional luma planes of a padded
// reference picture, bit-exact with com_if_luma_frame (src/com_mc.c:760-800) including the
// edge padding that follows it (com_img_padding(img, 1, 4), src/com_util.c:148-160).
//
// Each output sample of a padded plane equals the filter value at its position clamped to
// [-4, W+3] x [-4, H+3] (the padding replicates that region outward), so one launch writes
// every sample of all 15 planes exactly once: HBM traffic is one read of the integer plane
// plus 15 plane writes.
#include "common.cuh"
#include "uavs3e_cuda_internal.h"

namespace uc {

constexpr int SP_TW = 64;        // output tile width
constexpr int SP_TH = 16;        // output tile height
constexpr int SP_RAW_W = SP_TW + 8;
constexpr int SP_RAW_H = SP_TH + 7;

__global__ void __launch_bounds__(256)
k_subpel_planes(const pel *__restrict__ src, int stride, int W, int H, int pad, PlaneSet15 out, int vec4)
{
    __shared__ pel raw[SP_RAW_H][SP_RAW_W];
    __shared__ s16 hs[3][SP_RAW_H][SP_TW];
    __shared__ int ccol[SP_TW];

    const int x0 = -pad + blockIdx.x * SP_TW;
    const int y0 = -pad + blockIdx.y * SP_TH;
    const int xe = min(x0 + SP_TW - 1, W + pad - 1);
    const int ye = min(y0 + SP_TH - 1, H + pad - 1);
    const int cxs = min(max(x0, -4), W + 3), cxe = min(max(xe, -4), W + 3);
    const int cys = min(max(y0, -4), H + 3), cye = min(max(ye, -4), H + 3);
    const int rw = cxe - cxs + 8, rh = cye - cys + 8;
    const int tid = threadIdx.x;

    for (int i = tid; i < rh * rw; i += blockDim.x) {
        int r = i / rw, c = i % rw;
        raw[r][c] = src[(cys - 3 + r) * stride + (cxs - 3 + c)];
    }
    if (tid < SP_TW) ccol[tid] = min(max(x0 + tid, -4), W + 3) - cxs;
    __syncthreads();

    // horizontal 8-tap sums (kept as s16, 8-bit: no rounding shift) at every window row for
    // each output column's clamped source column
    for (int i = tid; i < rh * SP_TW; i += blockDim.x) {
        int r = i / SP_TW, c = i % SP_TW;
        int cc = ccol[c];
        int t1 = 0, t2 = 0, t3 = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            int v = raw[r][cc + k];
            t1 += v * kLumaTaps[1][k];
            t2 += v * kLumaTaps[2][k];
            t3 += v * kLumaTaps[3][k];
        }
        hs[0][r][c] = (s16)t1;
        hs[1][r][c] = (s16)t2;
        hs[2][r][c] = (s16)t3;
    }
    __syncthreads();

    const int r = tid >> 4;            // output row in tile
    const int c0 = (tid & 15) * 4;     // first of 4 output columns
    const int y = y0 + r;
    if (y > ye) return;
    const int i0 = min(max(y, -4), H + 3) - cys;   // window row of (clamped y) - 3

    u32 pk[15];
#pragma unroll
    for (int q = 0; q < 15; q++) pk[q] = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int c = c0 + j;
        const int cc = ccol[c] + 3;
        // (0, dx): rounded horizontal value
#pragma unroll
        for (int f = 1; f <= 3; f++) {
            int v = clip255((hs[f - 1][i0 + 3][c] + 32) >> 6);
            pk[f - 1] |= (u32)v << (8 * j);
        }
        // (dy, 0): vertical 8-tap on the integer samples
#pragma unroll
        for (int f = 1; f <= 3; f++) {
            int t = 0;
#pragma unroll
            for (int k = 0; k < 8; k++) t += raw[i0 + k][cc] * kLumaTaps[f][k];
            pk[f * 4 - 1] |= (u32)clip255((t + 32) >> 6) << (8 * j);
        }
        // (dy, dx): vertical 8-tap on the s16 horizontal sums, (sum + 2^11) >> 12
#pragma unroll
        for (int dx = 1; dx <= 3; dx++) {
            int hv[8];
#pragma unroll
            for (int k = 0; k < 8; k++) hv[k] = hs[dx - 1][i0 + k][c];
#pragma unroll
            for (int dy = 1; dy <= 3; dy++) {
                int t = 0;
#pragma unroll
                for (int k = 0; k < 8; k++) t += hv[k] * kLumaTaps[dy][k];
                pk[dy * 4 + dx - 1] |= (u32)clip255((t + 2048) >> 12) << (8 * j);
            }
        }
    }
    const int x = x0 + c0;
    const long long row = (long long)y * stride;
    if (vec4 && x + 3 <= xe) {
#pragma unroll
        for (int q = 0; q < 15; q++) *(u32 *)(out.p[q] + row + x) = pk[q];
    } else {
        for (int j = 0; j < 4; j++) {
            if (x + j > xe) break;
#pragma unroll
            for (int q = 0; q < 15; q++) out.p[q][row + x + j] = (pel)(pk[q] >> (8 * j));
        }
    }
}

int launch_subpel_planes(const pel *src, int stride, int W, int H, int pad, const PlaneSet15 &out, cudaStream_t st)
{
    if (!src || W <= 0 || H <= 0 || pad < 8 || stride < W + 2 * pad) return set_status(UC_ERR_ARG, "subpel_planes: bad geometry");
    int vec4 = (stride % 4) == 0;
    for (int q = 0; q < 15; q++) {
        if (!out.p[q]) return set_status(UC_ERR_ARG, "subpel_planes: null plane");
        if (((uintptr_t)(out.p[q] - pad)) % 4) vec4 = 0;
    }
    dim3 grid((W + 2 * pad + SP_TW - 1) / SP_TW, (H + 2 * pad + SP_TH - 1) / SP_TH);
    prof_begin(PROF_SUBPEL, st);
    k_subpel_planes<<<grid, 256, 0, st>>>(src, stride, W, H, pad, out, vec4);
    UC_CHECK(cudaGetLastError());
    count_launch(1);
    prof_end(PROF_SUBPEL, st);
    return UC_OK;
}

}  // namespace uc
