// Shared device/host helpers of libuavs3e_cuda (sm_103a, 8-bit luma).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

typedef uint8_t  pel;
typedef int8_t   s8;
typedef int16_t  s16;
typedef int32_t  s32;
typedef int64_t  s64;
typedef uint8_t  u8;
typedef uint16_t u16;
typedef uint32_t u32;
typedef uint64_t u64;

// status codes shared with include/uavs3e_cuda.h
#define UC_OK              0
#define UC_ERR_ARG        -101
#define UC_ERR_MEMORY     -102
#define UC_ERR_UNSUPPORTED -103
#define UC_ERR_CUDA       -110
#define UC_ERR_NOT_INIT   -111
#define UC_ERR_TIMEOUT    -112

namespace uc {

// record a failure in the library's sticky status (capi.cu); returns the code
int set_status(int code, const char *what);
int check_cuda(cudaError_t e, const char *what);

#define UC_CHECK(call)                                                       \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) return uc::check_cuda(e_, #call);             \
    } while (0)

// 8-tap luma filters (quarter-sample phases 0..3), src/com_tables.c:149-154
__device__ __constant__ static const s8 kLumaTaps[4][8] = {
    { 0, 0, 0, 64, 0, 0, 0, 0 },
    { -1, 4, -10, 57, 19, -7, 3, -1 },
    { -1, 4, -11, 40, 40, -11, 4, -1 },
    { -1, 3, -7, 19, 57, -10, 4, -1 },
};

__device__ __forceinline__ int clip255(int v) { return min(255, max(0, v)); }

// sum over the four byte lanes of |a - b|, accumulated into c (PTX video instruction)
__device__ __forceinline__ u32 sad4(u32 a, u32 b, u32 c)
{
    u32 d;
    asm("vabsdiff4.u32.u32.u32.add %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

// smallest value over the warp (every lane receives it)
__device__ __forceinline__ u64 warp_min_u64(u64 v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        u64 t = __shfl_xor_sync(0xffffffffu, v, o);
        v = t < v ? t : v;
    }
    return v;
}

// 4 bytes starting `sh` bytes (0..3) into the 8-byte little-endian pair (lo, hi)
__device__ __forceinline__ u32 align4(u32 lo, u32 hi, u32 sh)
{
    return __funnelshift_r(lo, hi, sh * 8);
}

// in-register Walsh-Hadamard butterflies
template <int N>
__device__ __forceinline__ void wht(int *v)
{
#pragma unroll
    for (int h = 1; h < N; h <<= 1)
#pragma unroll
        for (int i = 0; i < N; i += 2 * h)
#pragma unroll
            for (int j = i; j < i + h; j++) {
                int a = v[j], b = v[j + h];
                v[j] = a + b;
                v[j + h] = a - b;
            }
}

// 2-D WHT of an N x N difference tile held in registers, row-major
template <int N>
__device__ __forceinline__ void wht2d(int *d)
{
#pragma unroll
    for (int r = 0; r < N; r++) wht<N>(d + r * N);
#pragma unroll
    for (int c = 0; c < N; c++) {
        int col[N];
#pragma unroll
        for (int r = 0; r < N; r++) col[r] = d[r * N + c];
        wht<N>(col);
#pragma unroll
        for (int r = 0; r < N; r++) d[r * N + c] = col[r];
    }
}

// difference tile o - p of N x N samples
template <int N>
__device__ __forceinline__ void load_diff(int *d, const pel *o, int io, const pel *p, int ip)
{
#pragma unroll
    for (int r = 0; r < N; r++)
#pragma unroll
        for (int c = 0; c < N; c++) d[r * N + c] = (int)o[r * io + c] - (int)p[r * ip + c];
}

// com_had's normalisation of a 2:1 tile, (int)((double)s / sq * 2.0) for s >= 0 and sq = the
// host's sqrt(128) (16x8 / 8x16 tiles) or sqrt(32) (8x4 / 4x8), src/com_cost.c:344-710.  With
// k = had_scale_k(sq) = round(2^41 / sq), s k / 2^40 equals 2 s / sq to within 2^-17 for
// s < 2^23, so wherever its fraction lies at least 2^-16 from an integer its integer part is the
// double expression's value (a unit test checks every s < 2^23); the products nearer an integer
// (about 3 in 10^5) and larger s take the double expression itself.  A double division costs far
// more on this GPU than the 64-bit multiply.
__host__ __device__ __forceinline__ u64 had_scale_k(double sq) { return (u64)(2199023255552.0 / sq + 0.5); }

__device__ __forceinline__ u32 had_scale(int s, double sq, u64 k)
{
    const u64 prod = (u64)(u32)s * k;
    const u64 frac = prod & ((1ull << 40) - 1);
    if ((u32)s < (1u << 23) && frac >= (1ull << 24) && frac <= (1ull << 40) - (1ull << 24)) return (u32)(prod >> 40);
    return (u32)(int)((double)s / sq * 2.0);
}

// Hadamard SATD of a tw x th tile (com_had_4x4/8x8/16x8/8x16/8x4/4x8, src/com_cost.c:176-710).
// The 16-point (8-point) transform of a [left|right] row is [H(l)+H(r), H(l)-H(r)], so a
// 16x8 tile's coefficient magnitudes are |A+B| and |A-B| for the 8x8 transforms A, B of its
// halves, and |a+b| + |a-b| = 2 max(|a|, |b|).  sq32/sq128 are the host's sqrt(32), sqrt(128).
__device__ __forceinline__ u32 satd_tile(int tw, int th, const pel *o, int io, const pel *p, int ip,
                                         double sq32, double sq128)
{
    if (tw == 8 && th == 8) {
        int d[64];
        load_diff<8>(d, o, io, p, ip);
        wht2d<8>(d);
        int s = 0;
#pragma unroll
        for (int i = 0; i < 64; i++) s += abs(d[i]);
        return (u32)((s + 2) >> 2);
    }
    if (tw == 4 && th == 4) {
        int d[16];
        load_diff<4>(d, o, io, p, ip);
        wht2d<4>(d);
        int s = 0;
#pragma unroll
        for (int i = 0; i < 16; i++) s += abs(d[i]);
        return (u32)((s + 1) >> 1);
    }
    if (tw * th == 128) {
        int a[64], b[64];
        int bo = tw == 16 ? 8 : 8 * io, bp = tw == 16 ? 8 : 8 * ip;
        load_diff<8>(a, o, io, p, ip);
        wht2d<8>(a);
        load_diff<8>(b, o + bo, io, p + bp, ip);
        wht2d<8>(b);
        int s = 0;
#pragma unroll
        for (int i = 0; i < 64; i++) s += 2 * max(abs(a[i]), abs(b[i]));
        return (u32)(int)((double)s / sq128 * 2.0);
    }
    {   // 8x4 / 4x8
        int a[16], b[16];
        int bo = tw == 8 ? 4 : 4 * io, bp = tw == 8 ? 4 : 4 * ip;
        load_diff<4>(a, o, io, p, ip);
        wht2d<4>(a);
        load_diff<4>(b, o + bo, io, p + bp, ip);
        wht2d<4>(b);
        int s = 0;
#pragma unroll
        for (int i = 0; i < 16; i++) s += 2 * max(abs(a[i]), abs(b[i]));
        return (u32)(int)((double)s / sq32 * 2.0);
    }
}

// com_had tile shape for a w x h block (src/com_cost.c:712-812)
__host__ __device__ __forceinline__ void had_tile_shape(int w, int h, int *tw, int *th)
{
    if (w == h) { *tw = w == 4 ? 4 : 8; *th = *tw; }
    else if (w > h) { if (h == 4 || (h & 7)) { *tw = 8; *th = 4; } else { *tw = 16; *th = 8; } }
    else { if (w == 4 || (w & 7)) { *tw = 4; *th = 8; } else { *tw = 8; *th = 16; } }
}

// One pass of com_had tile rows over the warp: lanes in groups of TH hold one row each of a TW x TH
// tile (row = lane % TH), rows transformed in registers, columns by butterflies across the group.
// Tiles of 2:1 shape combine their two square halves as |a + b| + |a - b| = 2 max(|a|, |b|)
// (com_had_16x8 / _8x16 / _8x4 / _4x8, src/com_cost.c:344-710).  had_tile_sum returns the tile's
// magnitude sum, had_tile_rows its SATD, in every lane of the group (0 for inactive groups).
template <int TW, int TH>
__device__ __forceinline__ int had_tile_sum(const pel *o, const pel *p, bool active, int lane)
{
    constexpr bool WIDE = TW > TH, TALL = TW < TH;
    constexpr int N = WIDE ? TW / 2 : TW;            // points of each row transform
    constexpr int V = TALL ? TH / 2 : TH;            // points of the column transform
    int a[N], b[N];
#pragma unroll
    for (int i = 0; i < N; i++) {
        a[i] = active ? (int)o[i] - (int)p[i] : 0;
        b[i] = (WIDE && active) ? (int)o[N + i] - (int)p[N + i] : 0;
    }
    wht<N>(a);
    if (WIDE) wht<N>(b);
#pragma unroll
    for (int m = 1; m < V; m <<= 1) {
        const bool hi = lane & m;
#pragma unroll
        for (int i = 0; i < N; i++) {
            const int pa = __shfl_xor_sync(0xffffffffu, a[i], m);
            a[i] = hi ? pa - a[i] : a[i] + pa;
            if (WIDE) {
                const int pb = __shfl_xor_sync(0xffffffffu, b[i], m);
                b[i] = hi ? pb - b[i] : b[i] + pb;
            }
        }
    }
    int s = 0;
    if (TALL) {                                       // the other half of the 16 (8) rows
        const bool top = !(lane & V);
#pragma unroll
        for (int i = 0; i < N; i++) {
            const int e = __shfl_xor_sync(0xffffffffu, a[i], V);
            s += top ? 2 * max(abs(a[i]), abs(e)) : 0;
        }
    } else {
#pragma unroll
        for (int i = 0; i < N; i++) s += WIDE ? 2 * max(abs(a[i]), abs(b[i])) : abs(a[i]);
    }
#pragma unroll
    for (int m = 1; m < TH; m <<= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
    return s;
}

// com_had's normalisation of a tile's magnitude sum: 4x4 (s+1)>>1, 8x8 (s+2)>>2, 2:1 tiles
// (int)(s / sqrt(w h) * 2.0) in double
template <int TW, int TH>
__device__ __forceinline__ u32 had_tile_norm(int s, double sq32, double sq128, u64 k32, u64 k128)
{
    if (TW == TH) return (u32)(TW == 8 ? (s + 2) >> 2 : (s + 1) >> 1);
    return TW * TH == 128 ? had_scale(s, sq128, k128) : had_scale(s, sq32, k32);
}

template <int TW, int TH>
__device__ __forceinline__ u32 had_tile_rows(const pel *o, int io, const pel *p, int ip, bool active, int lane,
                                            double sq32, double sq128, u64 k32, u64 k128)
{
    return had_tile_norm<TW, TH>(had_tile_sum<TW, TH>(o, p, active, lane), sq32, sq128, k32, k128);
}


}  // namespace uc
