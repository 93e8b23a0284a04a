// Learned CU-partition / intra-mode pruning network: kernels for training and inference.
//
// The network sees one 64x64 luma CTU plus a constant QP plane and predicts split flags at the
// 64, 32 and 16 levels and an intra-mode shortlist per 16x16 cell.  Four 3x3 convolutions
// (stride 2, ReLU; 2 -> 16 -> 32 -> 32 -> 64 channels, 64x64 -> 4x4) feed a 1x1 head with 48
// outputs per cell: [split16, split32 part, split64 part, 33 mode logits, 12 unused].
//
// Convolutions are implicit GEMMs on the 5th-generation tensor cores (tcgen05.mma, bf16 x bf16
// with FP32 accumulation in tensor memory): forward (rows = output pixels, K = taps x input
// channels), data gradient (rows = input pixels, K = taps x output channels, with the previous
// layer's ReLU mask applied on store) and weight gradient, computed transposed (rows = taps x
// input channels, N = output channels, K = output pixels, split over CTAs with FP32 atomics).  A
// CTA of 128 threads owns a 128-row tile: it gathers the operands chunk by chunk (64 columns of
// K) into shared memory in the MMA's K-major layout, one thread issues the MMAs into a TMEM
// accumulator of 128 lanes x N columns, and the four warps read their 32 lanes back for the
// epilogue.  Activations are NHWC bf16, weights [Cout][K] bf16 with FP32 master copies updated
// by Adam.
#include "common.cuh"
#include "tma.cuh"
#include "umma.cuh"
#include "uavs3e_cuda_internal.h"
#include "../../include/uavs3e_cuda.h"

#include <cuda_bf16.h>
#include <string.h>
#include <algorithm>

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

// ---------------------------------------------------------------- tensor-core GEMM tiles

constexpr int TC_M = 128;        // rows of a tile (the MMA's M)
constexpr int TC_KC = 64;        // columns of K gathered per chunk
constexpr int TC_THREADS = 128;
constexpr int WG_CHUNK = 512;    // output pixels per CTA of the weight gradient
constexpr uint32_t TC_POLLS = 1u << 22;
// dynamic shared memory reserved (unused) by every launch so that at most 7 CTAs share an SM:
// their TMEM accumulators (at most 64 columns each) then always fit the SM's 512 columns and
// no CTA waits in its allocation
constexpr int TC_SMEM_RESERVE = 8 * 1024;
static __device__ unsigned int g_tc_timeouts;   // CTAs that gave up waiting for their MMAs

struct TcArgs {
    ConvShape S;
    const bf16 *src;     // MODE 0: x; MODE 1: dy; MODE 2: x (the pixel rows' inputs)
    const bf16 *wmat;    // MODE 0: w [Cout][Kp]; MODE 1: w^T [Cin][taps*Cout]; MODE 2: dy
    int wrow;            // row length of wmat (MODE 0 / 1)
    const float *bias;
    void *dst; int dst_f32, relu;
    const bf16 *mask;    // MODE 1: the layer input (ReLU output of the previous layer)
    float *dw;           // MODE 2
};

// MODE 0: forward, y = act(x (*) w + bias), rows = output pixels, N = Cout
// MODE 1: data gradient, dx = mask(x_in) * (dy (*) w^T), rows = input pixels, N = Cin
// MODE 2: weight gradient, dw^T[k][co] += sum over this CTA's output pixels of x_col[m][k] dy[m][co]
template <int MODE>
__global__ void __launch_bounds__(TC_THREADS) k_conv_tc(const TcArgs T)
{
    __shared__ __align__(128) unsigned char sa[TC_M * TC_KC * 2];
    __shared__ __align__(128) unsigned char sb[64 * TC_KC * 2];
    __shared__ __align__(8) u64 bar;
    __shared__ u32 s_tmem;
    // index tables: the tile's rows (one per thread) and the chunk's columns, decomposed once
    // instead of per gathered element (MODE 0: rows = output pixels {b Hin, oy s - pad, ox s - pad},
    // column pairs = {ky, kx, ci}; MODE 1: rows = input pixels {b Hout, iy + pad, ix + pad},
    // column pairs = {ky, kx, co}; MODE 2: rows = {ky, kx, ci}, columns = output pixels as MODE 0's
    // rows); .w = 1 where the row / column exists
    __shared__ int4 s_row[TC_M];
    __shared__ int4 s_col[TC_KC];
    const ConvShape &S = T.S;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int N = MODE == 0 ? S.Cout : MODE == 1 ? S.Cin : S.Cout;
    const int ncols = N <= 32 ? 32 : 64;
    // rows of the tile and the reduction range
    int M, K, r0, kb = 0;
    if (MODE == 0) { M = S.B * S.Hout * S.Wout; K = S.Kp; r0 = blockIdx.x * TC_M; }
    else if (MODE == 1) { M = S.B * S.Hin * S.Win; K = S.ks * S.ks * S.Cout; r0 = blockIdx.x * TC_M; }
    else { M = S.Kp; r0 = blockIdx.x * TC_M; kb = blockIdx.y * WG_CHUNK;
           K = min(WG_CHUNK, S.B * S.Hout * S.Wout - kb); K = (K + 15) & ~15; }
    const u32 bar_a = smem_u32(&bar);
    if (warp == 0) tmem_alloc(smem_u32(&s_tmem), (u32)ncols);
    if (tid == 0) {
        mbar_init(bar_a, 1);
        mbar_fence_init();
    }
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    const u32 tmem = s_tmem;
    const u32 idesc = umma_idesc_bf16(TC_M, N);
    u32 phase = 0;
    bool ok = true;
    const int npix = MODE == 2 ? S.B * S.Hout * S.Wout : 0;
    // output pixel p -> {b Hin, oy s - pad, ox s - pad, exists}
    auto out_pixel = [&](int p, int n) {
        if (p >= n) return make_int4(0, 0, 0, 0);
        const int hw = S.Hout * S.Wout, b = p / hw, rr = p - b * hw, oy = rr / S.Wout, ox = rr - oy * S.Wout;
        return make_int4(b * S.Hin, oy * S.stride - S.pad, ox * S.stride - S.pad, 1);
    };
    {
        const int row = r0 + tid;   // TC_THREADS == TC_M: one row per thread
        if (MODE == 0) {
            s_row[tid] = out_pixel(row, M);
        } else if (MODE == 1) {
            if (row < M) {
                const int hw = S.Hin * S.Win, b = row / hw, rr = row - b * hw, iy = rr / S.Win, ix = rr - iy * S.Win;
                s_row[tid] = make_int4(b * S.Hout, iy + S.pad, ix + S.pad, 1);
            } else {
                s_row[tid] = make_int4(0, 0, 0, 0);
            }
        } else {
            if (row < S.K) {
                const int tap = row / S.Cin, ci = row - tap * S.Cin, ky = tap / S.ks;
                s_row[tid] = make_int4(ky, tap - ky * S.ks, ci, 1);
            } else {
                s_row[tid] = make_int4(0, 0, 0, 0);
            }
        }
    }
    const int sshift = S.stride == 2 ? 1 : 0;   // the network's strides are 1 and 2

    for (int k0 = 0; k0 < K && ok; k0 += TC_KC) {
        const int kc = min(TC_KC, K - k0);         // a multiple of 16
        const int kq = kc >> 3;                    // 16-byte units per row
        // the chunk's column table (the previous chunk's MMAs have completed: see the wait below)
        if (MODE == 2) {
            for (int j = tid; j < kc; j += TC_THREADS) s_col[j] = out_pixel(kb + k0 + j, npix);
        } else {
            const int cdiv = MODE == 0 ? S.Cin : S.Cout, kmax = MODE == 0 ? S.K : K;
            for (int j = tid; j < (kc >> 1); j += TC_THREADS) {
                const int k = k0 + 2 * j;
                if (k < kmax) {
                    const int tap = k / cdiv, c = k - tap * cdiv, ky = tap / S.ks;
                    s_col[j] = make_int4(ky, tap - ky * S.ks, c, 1);
                } else {
                    s_col[j] = make_int4(0, 0, 0, 0);
                }
            }
        }
        __syncthreads();
        // A: TC_M rows x kc columns; 8 consecutive threads write one 128-byte core matrix
        for (int u = tid; u < TC_M * kq; u += TC_THREADS) {
            const int r = (u & 7) + 8 * ((u >> 3) / kq), q = (u >> 3) % kq;
            const int4 R = s_row[r];
            u32 v[4];
            if (MODE == 0) {
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const int4 Cc = s_col[4 * q + i];
                    const int iy = R.y + Cc.x, ix = R.z + Cc.y;
                    v[i] = (R.w & Cc.w) && iy >= 0 && iy < S.Hin && ix >= 0 && ix < S.Win
                               ? *reinterpret_cast<const u32 *>(T.src + ((size_t)(R.x + iy) * S.Win + ix) * S.Cin + Cc.z)
                               : 0u;
                }
            } else if (MODE == 1) {
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const int4 Cc = s_col[4 * q + i];
                    // the output pixel that read input pixel R through tap (ky, kx)
                    const int ty = R.y - Cc.x, tx = R.z - Cc.y;
                    const bool hit = (R.w & Cc.w) && ty >= 0 && tx >= 0 &&
                                     (sshift ? !((ty | tx) & 1) : S.stride == 1 || (ty % S.stride == 0 && tx % S.stride == 0));
                    const int oy = sshift ? ty >> 1 : S.stride == 1 ? ty : ty / S.stride;
                    const int ox = sshift ? tx >> 1 : S.stride == 1 ? tx : tx / S.stride;
                    v[i] = hit && oy < S.Hout && ox < S.Wout
                               ? *reinterpret_cast<const u32 *>(T.src + ((size_t)(R.x + oy) * S.Wout + ox) * S.Cout + Cc.z)
                               : 0u;
                }
            } else {
                // row r = input-column index (tap, ci) of x_col, columns = output pixels kb + k0 + 8q + j
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    bf16 e[2];
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const int4 Cc = s_col[8 * q + 2 * i + h];
                        const int iy = Cc.y + R.x, ix = Cc.z + R.y;
                        e[h] = (R.w & Cc.w) && iy >= 0 && iy < S.Hin && ix >= 0 && ix < S.Win
                                   ? T.src[((size_t)(Cc.x + iy) * S.Win + ix) * S.Cin + R.z]
                                   : __float2bfloat16(0.f);
                    }
                    v[i] = pack_bf16(e[0], e[1]);
                }
            }
            *reinterpret_cast<uint4 *>(sa + umma_tile_off(r, 8 * q, kc)) = make_uint4(v[0], v[1], v[2], v[3]);
        }
        // B: N rows x kc columns
        for (int u = tid; u < N * kq; u += TC_THREADS) {
            const int n = (u & 7) + 8 * ((u >> 3) / kq), q = (u >> 3) % kq;
            uint4 v;
            if (MODE != 2) {
                v = *reinterpret_cast<const uint4 *>(T.wmat + (size_t)n * T.wrow + k0 + 8 * q);
            } else {
                u32 w[4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const int m = kb + k0 + 8 * q + 2 * i;
                    const bf16 z = __float2bfloat16(0.f);
                    const bf16 e0 = m < npix ? T.wmat[(size_t)m * S.Cout + n] : z;
                    const bf16 e1 = m + 1 < npix ? T.wmat[(size_t)(m + 1) * S.Cout + n] : z;
                    w[i] = pack_bf16(e0, e1);
                }
                v = make_uint4(w[0], w[1], w[2], w[3]);
            }
            *reinterpret_cast<uint4 *>(sb + umma_tile_off(n, 8 * q, kc)) = v;
        }
        // the operands written by the threads become visible to the tensor core
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after_sync();
            const u32 a0 = smem_u32(sa), b0 = smem_u32(sb);
            for (int s = 0; s < (kc >> 4); s++)
                umma_bf16(tmem, umma_desc(a0 + 256 * s, 128, kc * 16), umma_desc(b0 + 256 * s, 128, kc * 16), idesc,
                          (k0 | s) != 0);
            umma_commit(bar_a);
        }
        // the chunk's MMAs must complete before the next chunk overwrites the operands
        const bool done = mbar_wait_bounded(bar_a, phase, TC_POLLS);
        phase ^= 1;
        ok = !__syncthreads_or(!done);
        if (!ok) {
            if (tid == 0) atomicAdd(&g_tc_timeouts, 1u);
            mbar_wait_bounded(bar_a, phase ^ 1, TC_POLLS);   // the commit may still arrive
        }
    }
    tc_fence_after_sync();

    if (ok) {
        // epilogue: warp w holds rows 32w .. 32w + 31 of the tile in TMEM lanes of its quarter
        const int r = 32 * warp + lane;
        for (int c = 0; c < N; c += 16) {
            float v[16];
            tmem_ld16(tmem + ((u32)(32 * warp) << 16) + (u32)c, v);
            if (MODE == 0) {
                const int m = r0 + r;
                if (m < M) {
#pragma unroll
                    for (int i = 0; i < 16; i += 2) {
                        float v0 = v[i] + T.bias[c + i], v1 = v[i + 1] + T.bias[c + i + 1];
                        if (T.relu) { v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); }
                        if (T.dst_f32) {
                            float *o = (float *)T.dst + (size_t)m * N + c + i;
                            o[0] = v0; o[1] = v1;
                        } else {
                            *reinterpret_cast<u32 *>((bf16 *)T.dst + (size_t)m * N + c + i) =
                                pack_bf16(__float2bfloat16(v0), __float2bfloat16(v1));
                        }
                    }
                }
            } else if (MODE == 1) {
                const int m = r0 + r;
                if (m < M) {
#pragma unroll
                    for (int i = 0; i < 16; i += 2) {
                        // the layer input is the previous layer's ReLU output: zero where it was clipped
                        const u32 xm = *reinterpret_cast<const u32 *>(T.mask + (size_t)m * N + c + i);
                        const float v0 = (xm & 0x7FFFu) ? v[i] : 0.f, v1 = (xm & 0x7FFF0000u) ? v[i + 1] : 0.f;
                        *reinterpret_cast<u32 *>((bf16 *)T.dst + (size_t)m * N + c + i) =
                            pack_bf16(__float2bfloat16(v0), __float2bfloat16(v1));
                    }
                }
            } else {
                const int kk = r0 + r;
                if (kk < S.Kp) {
#pragma unroll
                    for (int i = 0; i < 16; i++) atomicAdd(T.dw + (size_t)(c + i) * S.Kp + kk, v[i]);
                }
            }
        }
    }
    tc_fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, (u32)ncols);
}

// bias gradient db[co] += sum_m dy[m][co]: a CTA of 256 threads walks rows m in steps of
// rows = 256 / C (thread t < rows C takes channel t % C of row t / C), sums its channels in shared
// memory and adds them to db with one atomic per channel
__global__ void __launch_bounds__(256) k_conv_bgrad(const bf16 *dy, int M, int C, float *db)
{
    __shared__ float s_part[256];
    const int co = threadIdx.x % C, rows = 256 / C, r0 = threadIdx.x / C;
    float s = 0.f;
    if (r0 < rows)   // C = 48 leaves the last 16 threads idle
        for (int m = blockIdx.x * rows + r0; m < M; m += gridDim.x * rows) s += __bfloat162float(dy[(size_t)m * C + co]);
    s_part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x < C) {
        float t = 0.f;
        for (int r = 0; r < rows; r++) t += s_part[r * C + threadIdx.x];
        atomicAdd(&db[threadIdx.x], t);
    }
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

__global__ void __launch_bounds__(256) k_cnn_head_loss(const float *logits, const u8 *labels, int B, bf16 *dlog,
                                                        float *loss)
{
    // a half-warp per CTU, a lane per 4x4 cell c = cy * 4 + cx; the split sums over the CTU and
    // over each 2x2-cell quadrant are shuffles within the half-warp (quadrant cells are lanes
    // c, c ^ 1, c ^ 4, c ^ 5)
    const int t = blockIdx.x * blockDim.x + threadIdx.x, b = t >> 4, c = t & 15;
    const bool act = b < B;
    const float *L = logits + ((size_t)(act ? b : 0) * 16 + c) * HEAD_C;
    const u8 *lab = labels + (size_t)(act ? b : 0) * 40;   // [0] s64, [1..4] s32, [5..20] s16, [21..36] mode
    const float inv = 1.f / B;
    auto bce = [](float s, float y) { return fmaxf(s, 0.f) - s * y + log1pf(expf(-fabsf(s))); };
    // split64: the mean of the 16 cells' part
    float s64 = L[2];
#pragma unroll
    for (int d = 1; d < 16; d <<= 1) s64 += __shfl_xor_sync(0xffffffffu, s64, d);
    s64 /= 16.f;
    const float y64 = (float)lab[0];
    // split32: the mean over the cell's quadrant
    const int q = (c >> 3) * 2 + ((c & 3) >> 1);
    float s32 = L[1];
    s32 += __shfl_xor_sync(0xffffffffu, s32, 1);
    s32 += __shfl_xor_sync(0xffffffffu, s32, 4);
    s32 /= 4.f;
    const float y32 = (float)lab[1 + q];
    // split16 and the 33 mode logits of the cell
    const float s16 = L[0], y16 = (float)lab[5 + c];
    float mx = -1e30f;
    for (int k = 0; k < 33; k++) mx = fmaxf(mx, L[3 + k]);
    float z = 0.f;
    for (int k = 0; k < 33; k++) z += expf(L[3 + k] - mx);
    const int ym = lab[21 + c];
    float part[4] = { c == 0 ? bce(s64, y64) : 0.f, (c == 0 || c == 2 || c == 8 || c == 10) ? bce(s32, y32) / 4.f : 0.f,
                      bce(s16, y16) / 16.f, (logf(z) + mx - L[3 + ym]) / 16.f };
    if (act) {
        bf16 *D = dlog + ((size_t)b * 16 + c) * HEAD_C;
        const float p16 = 1.f / (1.f + expf(-s16)), p32 = 1.f / (1.f + expf(-s32)), p64 = 1.f / (1.f + expf(-s64));
        D[0] = __float2bfloat16((p16 - y16) / 16.f * inv);
        D[1] = __float2bfloat16((p32 - y32) / 4.f / 4.f * inv);
        D[2] = __float2bfloat16((p64 - y64) / 16.f * inv);
        for (int k = 0; k < 33; k++)
            D[3 + k] = __float2bfloat16((expf(L[3 + k] - mx) / z - (k == ym ? 1.f : 0.f)) / 16.f * inv);
        for (int k = 36; k < HEAD_C; k++) D[k] = __float2bfloat16(0.f);
    }
    // the loss parts summed over the warp (two CTUs), one atomic per part and warp
#pragma unroll
    for (int i = 0; i < 4; i++) {
        float v = act ? part[i] * inv : 0.f;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
        if ((threadIdx.x & 31) == 0) atomicAdd(&loss[i], v);
    }
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
    if (!x || !w || !bias || !y || Cout % 16 || Cout > 64 || !conv_shape(B, Hin, Win, Cin, Cout, ks, stride, Kp, S))
        return set_status(UC_ERR_ARG, "cnn_conv_fwd: shape");
    const int M = B * S.Hout * S.Wout;
    TcArgs T;
    memset(&T, 0, sizeof(T));
    T.S = S; T.src = (const bf16 *)x; T.wmat = (const bf16 *)w; T.wrow = Kp; T.bias = bias;
    T.dst = y; T.dst_f32 = y_f32; T.relu = relu;
    k_conv_tc<0><<<(M + TC_M - 1) / TC_M, TC_THREADS, TC_SMEM_RESERVE, (cudaStream_t)stream>>>(T);
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
    if (!dy || !w || !x || !dx || !wt_scratch || Cin % 16 || Cin > 64 ||
        !conv_shape(B, Hin, Win, Cin, Cout, ks, stride, Kp, S))
        return set_status(UC_ERR_ARG, "cnn_conv_dgrad: shape");
    cudaStream_t st = (cudaStream_t)stream;
    const int taps = ks * ks, nw = Cout * Cin * taps;
    k_transpose_w<<<(nw + 255) / 256, 256, 0, st>>>((const bf16 *)w, Cout, Cin, taps, Kp, (bf16 *)wt_scratch);
    UC_CHECK(cudaGetLastError());
    const int M = B * Hin * Win;
    TcArgs T;
    memset(&T, 0, sizeof(T));
    T.S = S; T.src = (const bf16 *)dy; T.wmat = (const bf16 *)wt_scratch; T.wrow = taps * Cout;
    T.dst = dx; T.mask = (const bf16 *)x;
    k_conv_tc<1><<<(M + TC_M - 1) / TC_M, TC_THREADS, TC_SMEM_RESERVE, st>>>(T);
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
    if (!dy || !x || !dw || !db || Cout % 16 || Cout > 64 || !conv_shape(B, Hin, Win, Cin, Cout, ks, stride, Kp, S))
        return set_status(UC_ERR_ARG, "cnn_conv_wgrad: shape");
    cudaStream_t st = (cudaStream_t)stream;
    const int M = B * S.Hout * S.Wout;
    UC_CHECK(cudaMemsetAsync(dw, 0, (size_t)Cout * Kp * sizeof(float), st));
    UC_CHECK(cudaMemsetAsync(db, 0, (size_t)Cout * sizeof(float), st));
    TcArgs T;
    memset(&T, 0, sizeof(T));
    T.S = S; T.src = (const bf16 *)x; T.wmat = (const bf16 *)dy; T.dw = dw;
    dim3 grid((Kp + TC_M - 1) / TC_M, (M + WG_CHUNK - 1) / WG_CHUNK);
    k_conv_tc<2><<<grid, TC_THREADS, TC_SMEM_RESERVE, st>>>(T);
    UC_CHECK(cudaGetLastError());
    k_conv_bgrad<<<std::min(1024, (M + 255) / 256), 256, 0, st>>>((const bf16 *)dy, M, Cout, db);
    UC_CHECK(cudaGetLastError());
    count_launch(2);
    return UC_OK;
}

// CTAs of the tensor-core convolutions that gave up waiting for their MMAs since the last call
// (their outputs were not written)
UAVS3E_CUDA_API int uavs3e_cuda_cnn_timeouts(void)
{
    int r = ensure_init();
    if (r) return r;
    unsigned int n = 0, zero = 0;
    UC_CHECK(cudaMemcpyFromSymbol(&n, g_tc_timeouts, sizeof(n)));
    UC_CHECK(cudaMemcpyToSymbol(g_tc_timeouts, &zero, sizeof(zero)));
    return (int)n;
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
    k_cnn_head_loss<<<(B * 16 + 255) / 256, 256, 0, st>>>(logits, labels, B, (bf16 *)dlogits, loss);
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
