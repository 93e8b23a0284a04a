// Learned CU-partition / intra-mode pruning network: kernels for training and inference.
//
// The network sees one 64x64 luma CTU plus a constant QP plane and predicts split flags at the
// 64, 32 and 16 levels and an intra-mode shortlist per 16x16 cell.  Four 3x3 convolutions
// (stride 2, ReLU; 2 -> 16 -> 32 -> 32 -> 64 channels, 64x64 -> 4x4) feed a 1x1 head with 48
// outputs per cell: [split16, split32 part, split64 part, 33 mode logits, 12 unused].
//
// Convolutions are implicit GEMMs on the 5th-generation tensor cores (tcgen05.mma, bf16 x bf16
// with FP32 accumulation in tensor memory): forward (rows = output pixels, K = taps x input
// channels), data gradient (rows = the input pixels of one stride phase class, K = the taps that
// class reaches x output channels, with the previous layer's ReLU mask applied on store) and
// weight gradient, computed transposed (rows = taps x input channels plus a row of ones for the
// bias gradient, N = output channels, K = output pixels, split over CTAs with FP32 atomics).  A
// CTA of 128 threads owns a 128-row tile: it gathers the operands chunk by chunk (64 columns of
// K) into shared memory in the MMA's no-swizzle layouts (K-major for the forward and data
// gradient, MN-major for the weight gradient, whichever makes 8 channels of one pixel one
// 16-byte load), one thread issues the MMAs into a TMEM accumulator of 128 lanes x N columns,
// and the four warps read their 32 lanes back for the epilogue.  Activations are NHWC bf16,
// weights [Cout][K] bf16 with FP32 master copies updated by Adam.
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

// ---------------------------------------------------------------- tensor-core GEMM tiles

constexpr int TC_M = 128;        // rows of a tile (the MMA's M)
constexpr int TC_KC = 64;        // columns of K gathered per chunk
constexpr int TC_THREADS = 128;
constexpr int WG_CHUNK = 512;    // most output pixels per CTA of the weight gradient
constexpr uint32_t TC_POLLS = 1u << 22;
// the static shared memory of a CTA (operand tiles and index tables, about 26 KB) lets at most 8
// CTAs share an SM (228 KB, plus 1 KB per CTA for the system): their TMEM accumulators (at most
// 64 columns each) then always fit the SM's 512 columns and no CTA waits in its allocation
constexpr int TC_STATIC_SMEM = TC_M * TC_KC * 2 + 64 * TC_KC * 2 + TC_M * 8 + TC_KC * 16;
static_assert(9 * (TC_STATIC_SMEM + 1024) > 228 * 1024, "more than 8 CTAs per SM would oversubscribe TMEM");
static __device__ unsigned int g_tc_timeouts;   // CTAs that gave up waiting for their MMAs

struct TcArgs {
    ConvShape S;
    const bf16 *src;     // MODE 0: x; MODE 1: dy; MODE 2: x (the pixel rows' inputs)
    const bf16 *wmat;    // MODE 0 / 1: w [Cout][Kp]; MODE 2: dy
    int wrow;            // row length of wmat (MODE 0 / 1: Kp)
    const float *bias;
    void *dst; int dst_f32, relu;
    const bf16 *mask;    // MODE 1: the layer input (ReLU output of the previous layer)
    float *dw, *db;      // MODE 2
    int ncls;            // MODE 1: phase classes (stride^2) and the first tile of each (+ the total)
    int cls_tile0[5];
    int wg_chunk;        // MODE 2: output pixels per CTA (a multiple of 64, at most WG_CHUNK)
};

// MODE 0: forward, y = act(x (*) w + bias), rows = output pixels, N = Cout
// MODE 1: data gradient, dx = mask(x_in) * (dy (*) w^T), N = Cin.  The input pixels are split into
//         the stride x stride phase classes (iy % stride, ix % stride): a pixel of one class is
//         read only through the taps (ky, kx) with (iy + pad - ky) and (ix + pad - kx) divisible by
//         the stride, so each class is a dense GEMM with K = its taps x Cout (at stride 2 with 3x3
//         taps: 1, 2, 2 or 4 taps instead of 9); a CTA takes 128 rows of one class
// MODE 2: weight gradient, dw^T[k][co] += sum over this CTA's output pixels of x_col[m][k] dy[m][co];
//         row K of x_col^T is a row of ones, so the same MMAs give the bias gradient
//         db[co] = sum_m dy[m][co].  Both operands are stored MN-major (the 8 channels of one pixel
//         are one 16-byte row of a core matrix), so each 16 bytes is one load from the NHWC tensors
// VEC: the 8 channels of a unit are contiguous (MODE 1, or Cin a multiple of 8) and gathered by
// one 16-byte load; otherwise by 4-byte channel pairs
template <int MODE, bool VEC>
__global__ void __launch_bounds__(TC_THREADS, 7) k_conv_tc(const TcArgs T)
{
    __shared__ __align__(128) unsigned char sa[TC_M * TC_KC * 2];
    __shared__ __align__(128) unsigned char sb[64 * TC_KC * 2];
    __shared__ __align__(8) u64 bar;
    __shared__ u32 s_tmem;
    // index tables, decomposed once instead of per gathered element.  A gathered element is
    // src[base + delta]: the pixel side of the product gives base and a mask of its taps (bit
    // ky ks + kx) that lie inside the picture, the (tap, channel) side gives delta and its tap:
    //   MODE 0: rows = output pixels {base, mask}; columns per 8 (per 2 when Cin is not a
    //           multiple of 8) = {delta, tap};
    //   MODE 1: rows = the class's input pixels {base, mask}; columns per 8 = {delta, tap, co};
    //   MODE 2: rows = (tap, ci) {delta, tap}; columns = output pixels {base, mask}.
    // Rows and columns that do not exist have mask 0 or tap 31 (never in a mask).
    __shared__ int2 s_row[TC_M];
    __shared__ int4 s_col[TC_KC];
    __shared__ int s_pix[TC_M];   // MODE 1: the row's input pixel, -1 past the class's rows
    const ConvShape &S = T.S;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int N = MODE == 0 ? S.Cout : MODE == 1 ? S.Cin : S.Cout;
    const int ncols = N <= 32 ? 32 : 64;
    const int sshift = S.stride == 2 ? 1 : 0;   // strides 1 and 2
    // rows of the tile and the reduction range
    int M, K, r0, kb = 0;
    int py = 0, px = 0, Hc = 0, Wc = 0, ky0 = 0, kx0 = 0, nkx = 1;
    if (MODE == 0) {
        M = S.B * S.Hout * S.Wout; K = S.Kp; r0 = blockIdx.x * TC_M;
    } else if (MODE == 1) {
        int cls = 0;
        while (cls + 1 < T.ncls && (int)blockIdx.x >= T.cls_tile0[cls + 1]) cls++;
        py = cls >> sshift; px = cls - (py << sshift);
        Hc = (S.Hin - py + S.stride - 1) >> sshift; Wc = (S.Win - px + S.stride - 1) >> sshift;
        ky0 = (py + S.pad) & sshift; kx0 = (px + S.pad) & sshift;
        const int nky = (S.ks - ky0 + S.stride - 1) >> sshift;
        nkx = (S.ks - kx0 + S.stride - 1) >> sshift;
        M = S.B * Hc * Wc; K = nky * nkx * S.Cout; r0 = (blockIdx.x - T.cls_tile0[cls]) * TC_M;
    } else {
        M = S.K + 1; r0 = blockIdx.x * TC_M; kb = blockIdx.y * T.wg_chunk;
        K = min(T.wg_chunk, S.B * S.Hout * S.Wout - kb); K = (K + 15) & ~15;
    }
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
    const u32 idesc = umma_idesc_bf16(TC_M, N, MODE == 2, MODE != 0);
    u32 phase = 0;
    bool ok = true;
    const int npix = MODE == 2 ? S.B * S.Hout * S.Wout : 0;
    constexpr bool vec = VEC;
    const int rowK = MODE == 2 ? S.K - r0 : -1;      // MODE 2: the tile row of the ones row (bias)
    // MODE 2: 8-row groups of the tile that hold a (tap, channel) row or the ones row; the groups
    // past them are zero in every chunk, so they are cleared once here and never gathered
    const int ng = MODE == 2 ? min(TC_M / 8, (M - r0 + 7) >> 3) : TC_M / 8;
    if (MODE == 2 && ng < TC_M / 8)
        for (int i = tid; i < TC_M * TC_KC * 2 / 16; i += TC_THREADS)
            reinterpret_cast<uint4 *>(sa)[i] = make_uint4(0u, 0u, 0u, 0u);
    // t / ng and t / (N / 8) for t < 8 ng and t < N as multiply-shifts (exact in those ranges)
    const u32 ng_inv = (65536u + ng - 1) / ng, nh_inv = (65536u + (N >> 3) - 1) / (N >> 3);
    // output pixel p -> {offset of its window's corner (oy s - pad, ox s - pad), mask of its taps
    // inside the picture}; {0, 0} past n
    auto out_pixel = [&](int p, int n) {
        if (p >= n) return make_int2(0, 0);
        const int hw = S.Hout * S.Wout, b = p / hw, rr = p - b * hw, oy = rr / S.Wout, ox = rr - oy * S.Wout;
        const int y0 = oy * S.stride - S.pad, x0 = ox * S.stride - S.pad;
        // the taps inside are the rows ky in [ylo, yhi] x the columns kx in [xlo, xhi]
        const int ylo = max(0, -y0), yhi = min(S.ks - 1, S.Hin - 1 - y0);
        const int xlo = max(0, -x0), xhi = min(S.ks - 1, S.Win - 1 - x0);
        const int cols = ((1 << (xhi + 1)) - 1) & ~((1 << xlo) - 1);
        int mask = 0;
        for (int ky = ylo; ky <= yhi; ky++) mask |= cols << (ky * S.ks);
        return make_int2(((b * S.Hin + y0) * S.Win + x0) * S.Cin, xlo <= xhi ? mask : 0);
    };
    // column k of x_col (tap, input channel) -> {delta from the window's corner, tap}; tap 31 past K
    auto tap_col = [&](int k) {
        if (k >= S.K) return make_int2(0, 31);
        const int tap = k / S.Cin, c = k - tap * S.Cin, ky = tap / S.ks, kx = tap - ky * S.ks;
        return make_int2((ky * S.Win + kx) * S.Cin + c, tap);
    };
    {
        const int row = r0 + tid;   // TC_THREADS == TC_M: one row per thread
        if (MODE == 0) {
            s_row[tid] = out_pixel(row, M);
        } else if (MODE == 1) {
            if (row < M) {
                const int hw = Hc * Wc, b = row / hw, rr = row - b * hw, j = rr / Wc, i = rr - j * Wc;
                const int iy = (j << sshift) + py, ix = (i << sshift) + px;
                // the class's taps reach output pixel (ay - ky / s, ax - kx / s), s = 1 or 2
                const int ay = (iy + S.pad) >> sshift, ax = (ix + S.pad) >> sshift;
                int mask = 0;
                for (int ky = ky0; ky < S.ks; ky += S.stride)
                    for (int kx = kx0; kx < S.ks; kx += S.stride) {
                        const int oy = ay - (ky >> sshift), ox = ax - (kx >> sshift);
                        if (oy >= 0 && oy < S.Hout && ox >= 0 && ox < S.Wout) mask |= 1 << (ky * S.ks + kx);
                    }
                s_row[tid] = make_int2(((b * S.Hout + ay) * S.Wout + ax) * S.Cout, mask);
                s_pix[tid] = (b * S.Hin + iy) * S.Win + ix;
            } else {
                s_row[tid] = make_int2(0, 0);
                s_pix[tid] = -1;
            }
        } else {
            s_row[tid] = tap_col(row);
        }
    }

    for (int k0 = 0; k0 < K && ok; k0 += TC_KC) {
        const int kc = min(TC_KC, K - k0);         // a multiple of 16
        const int kq = kc >> 3;                    // 8-column groups
        // the chunk's column table (the previous chunk's MMAs have completed: see the wait below)
        if (MODE == 2) {
            for (int j = tid; j < kc; j += TC_THREADS) {
                const int2 P = out_pixel(kb + k0 + j, npix);
                s_col[j] = make_int4(P.x, P.y, 0, 0);
            }
        } else if (MODE == 1) {
            if (tid < kq) {
                const int k = k0 + 8 * tid, t = k / S.Cout, co = k - t * S.Cout, tyi = t / nkx;
                const int ky = ky0 + (tyi << sshift), kx = kx0 + ((t - tyi * nkx) << sshift);
                s_col[tid] = make_int4(-((ky >> sshift) * S.Wout + (kx >> sshift)) * S.Cout + co, ky * S.ks + kx, co, 0);
            }
        } else {
            const int per = vec ? 8 : 2;           // columns per table entry
            for (int j = tid; j < kc / per; j += TC_THREADS) {
                const int2 D = tap_col(k0 + per * j);
                s_col[j] = make_int4(D.x, D.y, 0, 0);
            }
        }
        __syncthreads();
        // A: TC_M rows x kc columns, 16 bytes per unit, loaded for the thread's units first and
        // stored after.  MODE 0 / 1 (K-major): unit u = 8 columns of one row, 8 consecutive threads
        // fill one 128-byte core matrix.  MODE 2 (MN-major): unit u = 8 rows of one column.
        {
            const int nunits = MODE == 2 ? ng * kc : TC_M * kq;
            // MODE 0 / 1 with kq = 2, 4 or 8 (kq divides 16): unit u = tid + 128 i has the column group
            // (tid / 8) % kq for every i and row (tid % 8) + 8 ((tid / 8) / kq) + i (128 / kq), so the
            // column entry is read once
            const bool qfix = MODE != 2 && vec && (kq & (kq - 1)) == 0;
            const int lkq = 31 - __clz(kq);
            const int qf = (tid >> 3) & (kq - 1);
            const int4 Cq = s_col[qfix ? qf : 0];
            // units are loaded in batches of UB before they are stored (the weight gradient's
            // units hold more state: 4 keep it within the registers of 7 CTAs per SM)
            constexpr int UB = MODE == 2 ? 4 : 8;
#pragma unroll
            for (int i0 = 0; i0 < 8; i0 += UB) {
                uint4 va[UB];
                u32 off[UB];
#pragma unroll
                for (int j = 0; j < UB; j++) {
                    const int i = i0 + j, u = tid + i * TC_THREADS;
                    va[j] = make_uint4(0, 0, 0, 0);
                    off[j] = 0;
                    if (u >= nunits) continue;
                    if (MODE != 2) {
                        const int r = qfix ? (tid & 7) + 8 * ((tid >> 3) >> lkq) + (i << (7 - lkq)) : (u & 7) + 8 * ((u >> 3) / kq);
                        const int q = qfix ? qf : (u >> 3) % kq;
                        const int2 R = s_row[r];
                        off[j] = umma_tile_off(r, 8 * q, kc);
                        if (vec) {
                            const int4 Cc = qfix ? Cq : s_col[q];
                            if ((R.y >> Cc.y) & 1) va[j] = *reinterpret_cast<const uint4 *>(T.src + (R.x + Cc.x));
                        } else {
                            // MODE 0 with Cin not a multiple of 8: column pairs (two channels of one tap)
                            u32 v[4];
#pragma unroll
                            for (int e = 0; e < 4; e++) {
                                const int4 Cc = s_col[4 * q + e];
                                v[e] = (R.y >> Cc.y) & 1 ? *reinterpret_cast<const u32 *>(T.src + (R.x + Cc.x)) : 0u;
                            }
                            va[j] = make_uint4(v[0], v[1], v[2], v[3]);
                        }
                    } else {
                        const int kk = u & 7, t8 = u >> 3, kg = (int)(((u32)t8 * ng_inv) >> 16), g = t8 - kg * ng;
                        const int k = 8 * kg + kk;
                        const int4 Cc = s_col[k];
                        off[j] = (u32)(kg * (TC_M * 16) + g * 128 + kk * 16);
                        if (vec && 8 * g == rowK) {
                            // K is a multiple of 8 here: the ones row starts a group of 8 rows
                            va[j] = make_uint4(Cc.y ? 0x3F80u : 0u, 0u, 0u, 0u);
                        } else if (vec) {
                            const int2 R = s_row[8 * g];
                            if ((Cc.y >> R.y) & 1) va[j] = *reinterpret_cast<const uint4 *>(T.src + (Cc.x + R.x));
                        } else {
                            // row pairs (2e, 2e + 1) are channels (ci, ci + 1) of one tap (Cin and K
                            // are even): one 4-byte load each; the ones row K is the low half of a pair
                            u32 v[4];
#pragma unroll
                            for (int e = 0; e < 4; e++) {
                                const int rr = 8 * g + 2 * e;
                                const int2 R = s_row[rr];
                                v[e] = rr == rowK ? (Cc.y ? 0x3F80u : 0u)
                                       : (Cc.y >> R.y) & 1 ? *reinterpret_cast<const u32 *>(T.src + (Cc.x + R.x)) : 0u;
                            }
                            va[j] = make_uint4(v[0], v[1], v[2], v[3]);
                        }
                    }
                }
#pragma unroll
                for (int j = 0; j < UB; j++)
                    if (tid + (i0 + j) * TC_THREADS < nunits) *reinterpret_cast<uint4 *>(sa + off[j]) = va[j];
            }
        }
        // B: N rows x kc columns.  MODE 0: rows of the weight matrix (K-major).  MODE 1: the weights
        // w[co][tap Cin + ci] as they are stored, MN-major (unit = 8 input channels of one (tap,
        // co) column).  MODE 2: dy, MN-major (unit = 8 output channels of one pixel)
        {
            const int nh = N >> 3;
            const int nunits = MODE != 0 ? nh * kc : N * kq;
            uint4 vb[4];
            u32 off[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int u = tid + i * TC_THREADS;
                vb[i] = make_uint4(0, 0, 0, 0);
                off[i] = 0;
                if (u >= nunits) continue;
                if (MODE == 0) {
                    const int n = (u & 7) + 8 * ((u >> 3) / kq), q = (u >> 3) % kq;
                    off[i] = umma_tile_off(n, 8 * q, kc);
                    vb[i] = *reinterpret_cast<const uint4 *>(T.wmat + (size_t)n * T.wrow + k0 + 8 * q);
                } else {
                    const int t8 = u >> 3, kg = (int)(((u32)t8 * nh_inv) >> 16), h = t8 - kg * nh, k = 8 * kg + (u & 7);
                    off[i] = (u32)(kg * (N * 16) + h * 128 + (u & 7) * 16);
                    if (MODE == 1) {
                        const int4 Cc = s_col[kg];   // {delta, tap, co}
                        vb[i] = *reinterpret_cast<const uint4 *>(T.wmat + (size_t)(Cc.z + (u & 7)) * T.wrow +
                                                                 Cc.y * S.Cin + 8 * h);
                    } else {
                        const int m = kb + k0 + k;
                        if (m < npix) vb[i] = *reinterpret_cast<const uint4 *>(T.wmat + (size_t)m * S.Cout + 8 * h);
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < 4; i++)
                if (tid + i * TC_THREADS < nunits) *reinterpret_cast<uint4 *>(sb + off[i]) = vb[i];
        }
        // the operands written by the threads become visible to the tensor core
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after_sync();
            const u32 a0 = smem_u32(sa), b0 = smem_u32(sb);
            for (int s = 0; s < (kc >> 4); s++) {
                // one MMA per 16 columns of K: two core matrices along K
                const u64 ad = MODE == 2 ? umma_desc_mn(a0 + 2 * (TC_M * 16) * s, 128, TC_M * 16)
                                         : umma_desc(a0 + 256 * s, 128, kc * 16);
                const u64 bd = MODE != 0 ? umma_desc_mn(b0 + 2 * (N * 16) * s, 128, N * 16)
                                         : umma_desc(b0 + 256 * s, 128, kc * 16);
                umma_bf16(tmem, ad, bd, idesc, (k0 | s) != 0);
            }
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
        // (a data-gradient class without taps, K = 0, has no accumulator: its rows are 0)
        const int r = 32 * warp + lane;
        for (int c = 0; c < N; c += 16) {
            float v[16];
            if (K > 0) {
                tmem_ld16(tmem + ((u32)(32 * warp) << 16) + (u32)c, v);
            } else {
#pragma unroll
                for (int i = 0; i < 16; i++) v[i] = 0.f;
            }
            // the row's 16 columns are 32 (bf16) or 64 (FP32) contiguous bytes, N a multiple of 16:
            // 16-byte loads and stores
            if (MODE == 0) {
                const int m = r0 + r;
                if (m < M) {
#pragma unroll
                    for (int i = 0; i < 16; i++) {
                        v[i] += T.bias[c + i];
                        if (T.relu) v[i] = fmaxf(v[i], 0.f);
                    }
                    if (T.dst_f32) {
                        float4 *o = reinterpret_cast<float4 *>((float *)T.dst + (size_t)m * N + c);
#pragma unroll
                        for (int j = 0; j < 4; j++) o[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
                    } else {
                        u32 p[8];
#pragma unroll
                        for (int j = 0; j < 8; j++) p[j] = pack_bf16(__float2bfloat16(v[2 * j]), __float2bfloat16(v[2 * j + 1]));
                        uint4 *o = reinterpret_cast<uint4 *>((bf16 *)T.dst + (size_t)m * N + c);
                        o[0] = make_uint4(p[0], p[1], p[2], p[3]);
                        o[1] = make_uint4(p[4], p[5], p[6], p[7]);
                    }
                }
            } else if (MODE == 1) {
                const int m = s_pix[r];
                if (m >= 0) {
                    // the layer input is the previous layer's ReLU output: zero where it was clipped
                    const uint4 *xm4 = reinterpret_cast<const uint4 *>(T.mask + (size_t)m * N + c);
                    const uint4 xa = xm4[0], xb = xm4[1];
                    const u32 xm[8] = {xa.x, xa.y, xa.z, xa.w, xb.x, xb.y, xb.z, xb.w};
                    u32 p[8];
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        const float v0 = (xm[j] & 0x7FFFu) ? v[2 * j] : 0.f, v1 = (xm[j] & 0x7FFF0000u) ? v[2 * j + 1] : 0.f;
                        p[j] = pack_bf16(__float2bfloat16(v0), __float2bfloat16(v1));
                    }
                    uint4 *o = reinterpret_cast<uint4 *>((bf16 *)T.dst + (size_t)m * N + c);
                    o[0] = make_uint4(p[0], p[1], p[2], p[3]);
                    o[1] = make_uint4(p[4], p[5], p[6], p[7]);
                }
            } else {
                const int kk = r0 + r;
                if (kk < S.K) {
#pragma unroll
                    for (int i = 0; i < 16; i++) atomicAdd(T.dw + (size_t)(c + i) * S.Kp + kk, v[i]);
                } else if (kk == S.K) {
#pragma unroll
                    for (int i = 0; i < 16; i++) atomicAdd(T.db + c + i, v[i]);
                }
            }
        }
    }
    tc_fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, (u32)ncols);
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

// the 16-byte gathers and epilogue stores address 8 channels at a time from the tensors' bases
static bool aligned16(const void *p) { return ((uintptr_t)p & 15) == 0; }

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
           (stride == 1 || stride == 2) && (ks * ks * Cout) % 16 == 0 &&
           // element offsets are 32-bit
           (long long)B * Hin * Win * Cin < (1ll << 31) && (long long)B * S.Hout * S.Wout * Cout < (1ll << 31);
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
    if (!aligned16(x) || !aligned16(w) || !aligned16(y)) return set_status(UC_ERR_ARG, "cnn_conv_fwd: alignment");
    const int M = B * S.Hout * S.Wout;
    TcArgs T;
    memset(&T, 0, sizeof(T));
    T.S = S; T.src = (const bf16 *)x; T.wmat = (const bf16 *)w; T.wrow = Kp; T.bias = bias;
    T.dst = y; T.dst_f32 = y_f32; T.relu = relu;
    if (Cin % 8 == 0)
        k_conv_tc<0, true><<<(M + TC_M - 1) / TC_M, TC_THREADS, 0, (cudaStream_t)stream>>>(T);
    else
        k_conv_tc<0, false><<<(M + TC_M - 1) / TC_M, TC_THREADS, 0, (cudaStream_t)stream>>>(T);
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
    (void)wt_scratch;   // the weights are read in place (MN-major); kept for the ABI
    if (!dy || !w || !x || !dx || Cin % 16 || Cin > 64 || Cout % 16 || !conv_shape(B, Hin, Win, Cin, Cout, ks, stride, Kp, S))
        return set_status(UC_ERR_ARG, "cnn_conv_dgrad: shape");
    if (!aligned16(dy) || !aligned16(w) || !aligned16(x) || !aligned16(dx))
        return set_status(UC_ERR_ARG, "cnn_conv_dgrad: alignment");
    cudaStream_t st = (cudaStream_t)stream;
    TcArgs T;
    memset(&T, 0, sizeof(T));
    T.S = S; T.src = (const bf16 *)dy; T.wmat = (const bf16 *)w; T.wrow = Kp;
    T.dst = dx; T.mask = (const bf16 *)x;
    // the input pixels' phase classes (iy % stride, ix % stride), each a run of 128-row tiles
    T.ncls = stride * stride;
    T.cls_tile0[0] = 0;
    for (int c = 0; c < T.ncls; c++) {
        const int py = c / stride, px = c % stride;
        const int rows = B * ((Hin - py + stride - 1) / stride) * ((Win - px + stride - 1) / stride);
        T.cls_tile0[c + 1] = T.cls_tile0[c] + (rows + TC_M - 1) / TC_M;
    }
    if (T.cls_tile0[T.ncls] == 0) return set_status(UC_ERR_ARG, "cnn_conv_dgrad: shape");
    k_conv_tc<1, true><<<T.cls_tile0[T.ncls], TC_THREADS, 0, st>>>(T);
    UC_CHECK(cudaGetLastError());
    count_launch(1);
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
    if (!aligned16(dy) || !aligned16(x)) return set_status(UC_ERR_ARG, "cnn_conv_wgrad: alignment");
    cudaStream_t st = (cudaStream_t)stream;
    const int M = B * S.Hout * S.Wout;
    UC_CHECK(cudaMemsetAsync(dw, 0, (size_t)Cout * Kp * sizeof(float), st));
    UC_CHECK(cudaMemsetAsync(db, 0, (size_t)Cout * sizeof(float), st));
    TcArgs T;
    memset(&T, 0, sizeof(T));
    T.S = S; T.src = (const bf16 *)x; T.wmat = (const bf16 *)dy; T.dw = dw; T.db = db;
    // rows: the K (tap, input channel) rows and the ones row of the bias gradient; the pixels are
    // split into chunks small enough that the launch still has 4 CTAs per SM (down to 64 pixels)
    const int rowtiles = (S.K + 1 + TC_M - 1) / TC_M;
    int sms = 0, dev = 0;
    UC_CHECK(cudaGetDevice(&dev));
    UC_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    T.wg_chunk = WG_CHUNK;
    while (T.wg_chunk > 64 && rowtiles * ((M + T.wg_chunk - 1) / T.wg_chunk) < 4 * sms) T.wg_chunk >>= 1;
    dim3 grid(rowtiles, (M + T.wg_chunk - 1) / T.wg_chunk);
    if (Cin % 8 == 0)
        k_conv_tc<2, true><<<grid, TC_THREADS, 0, st>>>(T);
    else
        k_conv_tc<2, false><<<grid, TC_THREADS, 0, st>>>(T);
    UC_CHECK(cudaGetLastError());
    count_launch(1);
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
