// Learned CU-partition / intra-mode pruning network: kernels for training and inference.
//
// The network sees one 64x64 luma CTU plus a constant QP plane and predicts split flags at the
// 64, 32 and 16 levels and an intra-mode shortlist per 16x16 cell.  Four 3x3 convolutions
// (stride 2, ReLU; 2 -> 16 -> 32 -> 32 -> 64 channels, 64x64 -> 4x4) feed a 1x1 head with 48
// outputs per cell: [split16, split32 part, split64 part, 33 mode logits, 12 unused].
//
// Convolutions are implicit GEMMs on the bf16 tensor cores with FP32 accumulation
// (mma.sync m16n8k16): forward (rows = output pixels, K = taps x input channels), data gradient
// (rows = input pixels, K = taps x output channels, with the previous layer's ReLU mask applied
// on store) and weight gradient (rows = output channels, K = output pixels, split over CTAs with
// FP32 atomics).  Activations are NHWC bf16, weights [Cout][K] bf16 with FP32 master copies
// updated by Adam.
#include "common.cuh"
#include "uavs3e_cuda_internal.h"
#include "../../include/uavs3e_cuda.h"

#include <cuda_bf16.h>

namespace uc {

typedef __nv_bfloat16 bf16;

struct ConvShape {
    int B, Hin, Win, Cin, Hout, Wout, Cout;
    int ks, stride, pad;
    int K;       // ks * ks * Cin (taps x channels)
    int Kp;      // K rounded up to a multiple of 16 (weight row length)
};

__device__ __forceinline__ u32 pack_bf16(bf16 lo, bf16 hi)
{
    return (u32)__bfloat16_as_ushort(lo) | ((u32)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const u32 (&a)[4], const u32 (&b)[2])
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// im2col element pair (k, k+1) of output pixel m (k even; the pair shares a tap because Cin is
// even): two input channels of one input pixel, or 0 outside the picture / beyond K
__device__ __forceinline__ u32 fwd_pair(const bf16 *x, const ConvShape &S, int m, int k)
{
    if (k >= S.K) return 0u;
    const int hw = S.Hout * S.Wout;
    const int b = m / hw, r = m - b * hw, oy = r / S.Wout, ox = r - oy * S.Wout;
    const int tap = k / S.Cin, ci = k - tap * S.Cin;
    const int ky = tap / S.ks, kx = tap - ky * S.ks;
    const int iy = oy * S.stride + ky - S.pad, ix = ox * S.stride + kx - S.pad;
    if (iy < 0 || iy >= S.Hin || ix < 0 || ix >= S.Win) return 0u;
    return *reinterpret_cast<const u32 *>(x + (((size_t)b * S.Hin + iy) * S.Win + ix) * S.Cin + ci);
}

// data-gradient gather: for input pixel m and k = tap * Cout + co (co even), the output
// gradients (co, co+1) of the output pixel that read input pixel m through that tap
__device__ __forceinline__ u32 dgrad_pair(const bf16 *dy, const ConvShape &S, int m, int k)
{
    const int hw = S.Hin * S.Win;
    const int b = m / hw, r = m - b * hw, iy = r / S.Win, ix = r - iy * S.Win;
    const int tap = k / S.Cout, co = k - tap * S.Cout;
    const int ky = tap / S.ks, kx = tap - ky * S.ks;
    const int ty = iy + S.pad - ky, tx = ix + S.pad - kx;
    if (ty < 0 || tx < 0 || ty % S.stride || tx % S.stride) return 0u;
    const int oy = ty / S.stride, ox = tx / S.stride;
    if (oy >= S.Hout || ox >= S.Wout) return 0u;
    return *reinterpret_cast<const u32 *>(dy + (((size_t)b * S.Hout + oy) * S.Wout + ox) * S.Cout + co);
}

// one warp per 16 x 64 output tile (rows x columns); columns beyond N are skipped
// MODE 0: forward, y = act(x (*) w + bias), rows = output pixels, N = Cout, y bf16 or f32
// MODE 1: data gradient, dx = mask(x_in) * (dy (*) w^T), rows = input pixels, N = Cin
template <int MODE>
__global__ void __launch_bounds__(128) k_conv_gemm(ConvShape S, const bf16 *src, const bf16 *wmat, int wrow,
                                                     const float *bias, void *dst, int dst_f32, int relu,
                                                     const bf16 *mask)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int M = MODE == 0 ? S.B * S.Hout * S.Wout : S.B * S.Hin * S.Win;
    const int N = MODE == 0 ? S.Cout : S.Cin;
    const int K = MODE == 0 ? S.Kp : S.ks * S.ks * S.Cout;
    const int m0 = (blockIdx.x * 4 + (threadIdx.x >> 5)) * 16;
    const int n_base = blockIdx.y * 64;
    if (m0 >= M) return;
    float acc[8][4];
#pragma unroll
    for (int f = 0; f < 8; f++)
#pragma unroll
        for (int i = 0; i < 4; i++) acc[f][i] = 0.f;
    for (int k0 = 0; k0 < K; k0 += 16) {
        u32 a[4];
        const int ka = k0 + 2 * t;
        if (MODE == 0) {
            a[0] = fwd_pair(src, S, m0 + g, ka);
            a[1] = fwd_pair(src, S, m0 + g + 8, ka);
            a[2] = fwd_pair(src, S, m0 + g, ka + 8);
            a[3] = fwd_pair(src, S, m0 + g + 8, ka + 8);
        } else {
            a[0] = dgrad_pair(src, S, m0 + g, ka);
            a[1] = dgrad_pair(src, S, m0 + g + 8, ka);
            a[2] = dgrad_pair(src, S, m0 + g, ka + 8);
            a[3] = dgrad_pair(src, S, m0 + g + 8, ka + 8);
        }
#pragma unroll
        for (int f = 0; f < 8; f++) {
            const int n = n_base + f * 8 + g;
            if (n_base + f * 8 >= N) break;
            u32 b[2];
            const bf16 *wr = wmat + (size_t)n * wrow;
            b[0] = *reinterpret_cast<const u32 *>(wr + ka);
            b[1] = *reinterpret_cast<const u32 *>(wr + ka + 8);
            mma_bf16(acc[f], a, b);
        }
    }
#pragma unroll
    for (int f = 0; f < 8; f++) {
        if (n_base + f * 8 >= N) break;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int m = m0 + g + 8 * h, n = n_base + f * 8 + 2 * t;
            float v0 = acc[f][2 * h], v1 = acc[f][2 * h + 1];
            if (MODE == 0) {
                v0 += bias[n]; v1 += bias[n + 1];
                if (relu) { v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); }
            } else {
                // the layer input is the previous layer's ReLU output: zero where it was clipped
                const u32 xm = *reinterpret_cast<const u32 *>(mask + (size_t)m * N + n);
                if (!(xm & 0x7FFFu)) v0 = 0.f;
                if (!(xm & 0x7FFF0000u)) v1 = 0.f;
            }
            if (dst_f32) {
                float *o = (float *)dst + (size_t)m * N + n;
                o[0] = v0; o[1] = v1;
            } else {
                *reinterpret_cast<u32 *>((bf16 *)dst + (size_t)m * N + n) =
                    pack_bf16(__float2bfloat16(v0), __float2bfloat16(v1));
            }
        }
    }
}

// im2col element of output pixel m, k (scalar)
__device__ __forceinline__ bf16 fwd_elem(const bf16 *x, const ConvShape &S, int m, int k)
{
    if (k >= S.K) return __float2bfloat16(0.f);
    const int hw = S.Hout * S.Wout;
    const int b = m / hw, r = m - b * hw, oy = r / S.Wout, ox = r - oy * S.Wout;
    const int tap = k / S.Cin, ci = k - tap * S.Cin;
    const int ky = tap / S.ks, kx = tap - ky * S.ks;
    const int iy = oy * S.stride + ky - S.pad, ix = ox * S.stride + kx - S.pad;
    if (iy < 0 || iy >= S.Hin || ix < 0 || ix >= S.Win) return __float2bfloat16(0.f);
    return x[(((size_t)b * S.Hin + iy) * S.Win + ix) * S.Cin + ci];
}

// weight gradient dw[co][k] += sum_m dy[m][co] x_col[m][k] over this CTA's chunk of rows m;
// one warp per 16 (co) x 8 (k) tile, grid.z splits the output pixels
constexpr int WG_CHUNK = 512;

__global__ void __launch_bounds__(128) k_conv_wgrad(ConvShape S, const bf16 *dy, const bf16 *x, float *dw)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int M = S.B * S.Hout * S.Wout;
    const int tile = blockIdx.x * 4 + (threadIdx.x >> 5);
    const int n_tiles_k = S.Kp / 8;
    const int co0 = (tile / n_tiles_k) * 16, k0 = (tile % n_tiles_k) * 8;
    if (co0 >= S.Cout) return;
    const int mb = blockIdx.z * WG_CHUNK, me = min(M, mb + WG_CHUNK);
    float acc[4] = { 0.f, 0.f, 0.f, 0.f };
    for (int m = mb; m < me; m += 16) {
        u32 a[4], b[2];
        const int r0 = m + 2 * t, r1 = r0 + 1, r2 = r0 + 8, r3 = r0 + 9;
        const bf16 *d0 = dy + (size_t)r0 * S.Cout, *d1 = dy + (size_t)r1 * S.Cout;
        const bf16 *d2 = dy + (size_t)r2 * S.Cout, *d3 = dy + (size_t)r3 * S.Cout;
        a[0] = pack_bf16(d0[co0 + g], d1[co0 + g]);
        a[1] = pack_bf16(d0[co0 + g + 8], d1[co0 + g + 8]);
        a[2] = pack_bf16(d2[co0 + g], d3[co0 + g]);
        a[3] = pack_bf16(d2[co0 + g + 8], d3[co0 + g + 8]);
        b[0] = pack_bf16(fwd_elem(x, S, r0, k0 + g), fwd_elem(x, S, r1, k0 + g));
        b[1] = pack_bf16(fwd_elem(x, S, r2, k0 + g), fwd_elem(x, S, r3, k0 + g));
        mma_bf16(acc, a, b);
    }
    float *o0 = dw + (size_t)(co0 + g) * S.Kp + k0 + 2 * t;
    float *o1 = dw + (size_t)(co0 + g + 8) * S.Kp + k0 + 2 * t;
    atomicAdd(o0, acc[0]); atomicAdd(o0 + 1, acc[1]);
    atomicAdd(o1, acc[2]); atomicAdd(o1 + 1, acc[3]);
}

// bias gradient db[co] += sum_m dy[m][co]
__global__ void k_conv_bgrad(const bf16 *dy, int M, int C, float *db)
{
    const int co = threadIdx.x % C, lane_rows = blockDim.x / C;
    float s = 0.f;
    for (int m = blockIdx.x * lane_rows + threadIdx.x / C; m < M; m += gridDim.x * lane_rows)
        s += __bfloat162float(dy[(size_t)m * C + co]);
    atomicAdd(&db[co], s);
}

// wt[ci][tap * Cout + co] = w[co][tap * Cin + ci] (the data gradient's weight matrix)
__global__ void k_transpose_w(const bf16 *w, int Cout, int Cin, int taps, int Kp, bf16 *wt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Cout * Cin * taps) return;
    const int co = i % Cout, r = i / Cout, tap = r % taps, ci = r / taps;
    wt[(size_t)ci * taps * Cout + tap * Cout + co] = w[(size_t)co * Kp + tap * Cin + ci];
}

// network input: 64x64 luma of CTU (cx, cy) of the picture (edge samples repeated beyond the
// picture) as (p - 128) / 64, and the constant plane (qp - 32) / 8
__global__ void k_cnn_input(const pel *pic, int stride, int W, int H, const int *ctu_xy, int qp, bf16 *x0)
{
    const int b = blockIdx.x, p = threadIdx.x;   // 256 threads, 16 samples each
    const int cx = ctu_xy[2 * b], cy = ctu_xy[2 * b + 1];
    for (int i = p; i < 4096; i += blockDim.x) {
        const int y = min(cy + (i >> 6), H - 1), x = min(cx + (i & 63), W - 1);
        const float v = ((float)pic[(size_t)y * stride + x] - 128.f) / 64.f;
        *reinterpret_cast<u32 *>(x0 + ((size_t)b * 4096 + i) * 2) =
            pack_bf16(__float2bfloat16(v), __float2bfloat16(((float)qp - 32.f) / 8.f));
    }
}

// head losses of one CTU: logits [16 cells][40]; labels: split64, split32[4], split16[16],
// mode[16].  BCE on split16 = cell channel 0, split32 = mean of channel 1 over the quadrant's 4
// cells, split64 = mean of channel 2 over all cells; softmax cross-entropy on channels 3..35.
// Writes dlogits (bf16, scaled by 1/B) and adds the CTU's loss parts to loss[4].
constexpr int HEAD_C = 48;

__global__ void k_cnn_head_loss(const float *logits, const u8 *labels, int B, bf16 *dlog, float *loss)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const float *L = logits + (size_t)b * 16 * HEAD_C;
    const u8 *lab = labels + (size_t)b * 40;    // [0] s64, [1..4] s32, [5..20] s16, [21..36] mode
    bf16 *D = dlog + (size_t)b * 16 * HEAD_C;
    const float inv = 1.f / B;
    float l64 = 0.f, l32 = 0.f, l16 = 0.f, lm = 0.f;
    float grad[16][HEAD_C];
#pragma unroll 1
    for (int c = 0; c < 16; c++)
        for (int k = 0; k < HEAD_C; k++) grad[c][k] = 0.f;
    {   // split64
        float s = 0.f;
        for (int c = 0; c < 16; c++) s += L[c * HEAD_C + 2];
        s /= 16.f;
        const float p = 1.f / (1.f + expf(-s)), y = (float)lab[0];
        l64 = fmaxf(s, 0.f) - s * y + log1pf(expf(-fabsf(s)));
        for (int c = 0; c < 16; c++) grad[c][2] = (p - y) / 16.f;
    }
    for (int q = 0; q < 4; q++) {   // split32, quadrant q = (qy, qx) of 2x2 cells
        const int qy = q >> 1, qx = q & 1;
        float s = 0.f;
        for (int dy = 0; dy < 2; dy++)
            for (int dx = 0; dx < 2; dx++) s += L[((2 * qy + dy) * 4 + 2 * qx + dx) * HEAD_C + 1];
        s /= 4.f;
        const float p = 1.f / (1.f + expf(-s)), y = (float)lab[1 + q];
        l32 += fmaxf(s, 0.f) - s * y + log1pf(expf(-fabsf(s)));
        for (int dy = 0; dy < 2; dy++)
            for (int dx = 0; dx < 2; dx++) grad[(2 * qy + dy) * 4 + 2 * qx + dx][1] = (p - y) / 4.f / 4.f;
    }
    for (int c = 0; c < 16; c++) {   // split16 and modes
        const float s = L[c * HEAD_C + 0];
        const float p = 1.f / (1.f + expf(-s)), y = (float)lab[5 + c];
        l16 += fmaxf(s, 0.f) - s * y + log1pf(expf(-fabsf(s)));
        grad[c][0] = (p - y) / 16.f;
        float mx = -1e30f;
        for (int k = 0; k < 33; k++) mx = fmaxf(mx, L[c * HEAD_C + 3 + k]);
        float z = 0.f;
        for (int k = 0; k < 33; k++) z += expf(L[c * HEAD_C + 3 + k] - mx);
        const int ym = lab[21 + c];
        lm += logf(z) + mx - L[c * HEAD_C + 3 + ym];
        for (int k = 0; k < 33; k++) grad[c][3 + k] = (expf(L[c * HEAD_C + 3 + k] - mx) / z - (k == ym ? 1.f : 0.f)) / 16.f;
    }
    l32 /= 4.f; l16 /= 16.f; lm /= 16.f;
    for (int c = 0; c < 16; c++)
        for (int k = 0; k < HEAD_C; k++) D[c * HEAD_C + k] = __float2bfloat16(grad[c][k] * inv);
    atomicAdd(&loss[0], l64 * inv);
    atomicAdd(&loss[1], l32 * inv);
    atomicAdd(&loss[2], l16 * inv);
    atomicAdd(&loss[3], lm * inv);
}

// Adam on FP32 master weights; refreshes the bf16 copy.  Entries of a weight row beyond the
// layer's K stay 0 (their gradient is 0 and they start at 0).
__global__ void k_adam(float *w, float *m, float *v, const float *g, bf16 *wb, int n, float lr, float b1, float b2,
                       float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi; v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
}

static bool conv_shape(int B, int Hin, int Win, int Cin, int Cout, int ks, int stride, int Kp, ConvShape &S)
{
    S.B = B; S.Hin = Hin; S.Win = Win; S.Cin = Cin; S.Cout = Cout; S.ks = ks; S.stride = stride;
    S.pad = ks / 2;
    S.Hout = (Hin + 2 * S.pad - ks) / stride + 1;
    S.Wout = (Win + 2 * S.pad - ks) / stride + 1;
    S.K = ks * ks * Cin;
    S.Kp = Kp;
    return B > 0 && Cin >= 2 && !(Cin & 1) && Cout >= 16 && !(Cout % 8) && Kp >= S.K && !(Kp % 16) &&
           (B * S.Hout * S.Wout) % 16 == 0 && (B * Hin * Win) % 16 == 0 && (ks == 1 || ks == 3) &&
           (ks * ks * Cout) % 16 == 0;
}

}  // namespace uc

using namespace uc;

extern "C" {

UAVS3E_CUDA_API int uavs3e_cuda_cnn_conv_fwd(const void *x, const void *w, const float *bias, void *y, int y_f32,
                                             int B, int Hin, int Win, int Cin, int Cout, int ks, int stride, int Kp,
                                             int relu, void *stream)
{
    int r = ensure_init();
    if (r) return r;
    ConvShape S;
    if (!x || !w || !bias || !y || !conv_shape(B, Hin, Win, Cin, Cout, ks, stride, Kp, S))
        return set_status(UC_ERR_ARG, "cnn_conv_fwd: shape");
    const int M = B * S.Hout * S.Wout;
    dim3 grid((M / 16 + 3) / 4, (Cout + 63) / 64);
    k_conv_gemm<0><<<grid, 128, 0, (cudaStream_t)stream>>>(S, (const bf16 *)x, (const bf16 *)w, Kp, bias, y, y_f32,
                                                            relu, nullptr);
    UC_CHECK(cudaGetLastError());
    count_launch(1);
    return UC_OK;
}

UAVS3E_CUDA_API int uavs3e_cuda_cnn_conv_dgrad(const void *dy, const void *w, const void *x, void *dx, void *wt_scratch,
                                               int B, int Hin, int Win, int Cin, int Cout, int ks, int stride, int Kp,
                                               void *stream)
{
    int r = ensure_init();
    if (r) return r;
    ConvShape S;
    if (!dy || !w || !x || !dx || !wt_scratch || Cin % 8 || !conv_shape(B, Hin, Win, Cin, Cout, ks, stride, Kp, S))
        return set_status(UC_ERR_ARG, "cnn_conv_dgrad: shape");
    cudaStream_t st = (cudaStream_t)stream;
    const int taps = ks * ks, nw = Cout * Cin * taps;
    k_transpose_w<<<(nw + 255) / 256, 256, 0, st>>>((const bf16 *)w, Cout, Cin, taps, Kp, (bf16 *)wt_scratch);
    UC_CHECK(cudaGetLastError());
    const int M = B * Hin * Win;
    dim3 grid((M / 16 + 3) / 4, (Cin + 63) / 64);
    k_conv_gemm<1><<<grid, 128, 0, st>>>(S, (const bf16 *)dy, (const bf16 *)wt_scratch, taps * Cout, nullptr, dx, 0, 0,
                                         (const bf16 *)x);
    UC_CHECK(cudaGetLastError());
    count_launch(2);
    return UC_OK;
}

UAVS3E_CUDA_API int uavs3e_cuda_cnn_conv_wgrad(const void *dy, const void *x, float *dw, float *db, int B, int Hin,
                                               int Win, int Cin, int Cout, int ks, int stride, int Kp, void *stream)
{
    int r = ensure_init();
    if (r) return r;
    ConvShape S;
    if (!dy || !x || !dw || !db || Cout % 16 || Cout > 256 || !conv_shape(B, Hin, Win, Cin, Cout, ks, stride, Kp, S))
        return set_status(UC_ERR_ARG, "cnn_conv_wgrad: shape");
    cudaStream_t st = (cudaStream_t)stream;
    const int M = B * S.Hout * S.Wout;
    UC_CHECK(cudaMemsetAsync(dw, 0, (size_t)Cout * Kp * sizeof(float), st));
    UC_CHECK(cudaMemsetAsync(db, 0, (size_t)Cout * sizeof(float), st));
    const int tiles = (Cout / 16) * (Kp / 8);
    dim3 grid((tiles + 3) / 4, 1, (M + WG_CHUNK - 1) / WG_CHUNK);
    k_conv_wgrad<<<grid, 128, 0, st>>>(S, (const bf16 *)dy, (const bf16 *)x, dw);
    UC_CHECK(cudaGetLastError());
    const int rows = 256 / Cout;
    k_conv_bgrad<<<std::min(1024, (M + rows - 1) / rows), rows * Cout, 0, st>>>((const bf16 *)dy, M, Cout, db);
    UC_CHECK(cudaGetLastError());
    count_launch(2);
    return UC_OK;
}

UAVS3E_CUDA_API int uavs3e_cuda_cnn_input(const uint8_t *d_pic, int stride, int width, int height, const int *d_ctu_xy,
                                          int n, int qp, void *x0, void *stream)
{
    int r = ensure_init();
    if (r) return r;
    if (!d_pic || !d_ctu_xy || !x0 || n <= 0) return set_status(UC_ERR_ARG, "cnn_input");
    k_cnn_input<<<n, 256, 0, (cudaStream_t)stream>>>(d_pic, stride, width, height, d_ctu_xy, qp, (bf16 *)x0);
    UC_CHECK(cudaGetLastError());
    count_launch(1);
    return UC_OK;
}

UAVS3E_CUDA_API int uavs3e_cuda_cnn_head_loss(const float *logits, const uint8_t *labels, int B, void *dlogits,
                                              float *loss, void *stream)
{
    int r = ensure_init();
    if (r) return r;
    if (!logits || !labels || !dlogits || !loss || B <= 0) return set_status(UC_ERR_ARG, "cnn_head_loss");
    cudaStream_t st = (cudaStream_t)stream;
    UC_CHECK(cudaMemsetAsync(loss, 0, 4 * sizeof(float), st));
    k_cnn_head_loss<<<(B + 63) / 64, 64, 0, st>>>(logits, labels, B, (bf16 *)dlogits, loss);
    UC_CHECK(cudaGetLastError());
    count_launch(1);
    return UC_OK;
}

UAVS3E_CUDA_API int uavs3e_cuda_cnn_adam(float *w, float *m, float *v, const float *g, void *w_bf16, int n, float lr,
                                         float b1, float b2, float eps, int step, void *stream)
{
    int r = ensure_init();
    if (r) return r;
    if (!w || !m || !v || !g || n <= 0 || step < 1) return set_status(UC_ERR_ARG, "cnn_adam");
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_adam<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(w, m, v, g, (bf16 *)w_bf16, n, lr, b1, b2, eps, c1, c2);
    UC_CHECK(cudaGetLastError());
    count_launch(1);
    return UC_OK;
}

}  // extern "C"
