// Affine motion-compensation helpers shared by the affine CU prediction (mc.cu) and the affine
// motion search (affme.cu): the 1/16-sample luma filters and the sub-block MV rounding.
#pragma once
#include "common.cuh"

namespace uc {

// 1/16-sample luma filters (com_tbl_mc_l_coeff_hp, src/com_tables.c:130-147)
__device__ __constant__ static const s8 kMcLumaHp[16][8] = {
    { 0, 0, 0, 64, 0, 0, 0, 0 },      { 0, 1, -3, 63, 4, -2, 1, 0 },     { -1, 2, -5, 62, 8, -3, 1, 0 },
    { -1, 3, -8, 60, 13, -4, 1, 0 },   { -1, 4, -10, 58, 17, -5, 1, 0 },  { -1, 4, -11, 52, 26, -8, 3, -1 },
    { -1, 3, -9, 47, 31, -10, 4, -1 }, { -1, 4, -11, 45, 34, -10, 4, -1 }, { -1, 4, -11, 40, 40, -11, 4, -1 },
    { -1, 4, -10, 34, 45, -11, 4, -1 }, { -1, 4, -10, 31, 47, -9, 3, -1 }, { -1, 3, -8, 26, 52, -11, 4, -1 },
    { 0, 1, -5, 17, 58, -10, 4, -1 },  { 0, 1, -4, 13, 60, -8, 3, -1 },   { 0, 1, -3, 8, 62, -5, 2, -1 },
    { 0, 1, -2, 4, 63, -3, 1, 0 },
};

// the same rows packed 4 signed taps per word (taps 0..3, taps 4..7), for dp4a, in global memory
// so that lanes reading different phases do not serialise as they would on the constant cache
__device__ static const u32 kMcLumaHpPacked[16][2] = {
    { 0x40000000u, 0x00000000u }, { 0x3ffd0100u, 0x0001fe04u }, { 0x3efb02ffu, 0x0001fd08u }, { 0x3cf803ffu, 0x0001fc0du },
    { 0x3af604ffu, 0x0001fb11u }, { 0x34f504ffu, 0xff03f81au }, { 0x2ff703ffu, 0xff04f61fu }, { 0x2df504ffu, 0xff04f622u },
    { 0x28f504ffu, 0xff04f528u }, { 0x22f604ffu, 0xff04f52du }, { 0x1ff604ffu, 0xff03f72fu }, { 0x1af803ffu, 0xff04f534u },
    { 0x11fb0100u, 0xff04f63au }, { 0x0dfc0100u, 0xff03f83cu }, { 0x08fd0100u, 0xff02fb3eu }, { 0x04fe0100u, 0x0001fd3fu },
};

// sum of 4 unsigned bytes of a times 4 signed bytes of b, plus c
__device__ __forceinline__ int dp4a_us(u32 a, u32 b, int c)
{
    int d;
    asm("dp4a.u32.s32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

// one luma sample of com_mc_blk_luma with hp_flag 1: always filtered from the integer plane
// (the reference's plane shortcut tests dy == 0 and dy == 8 together and never applies)
__device__ __forceinline__ int aff_luma_sample(const pel *s, int is, int dx, int dy)
{
    if (!dx && !dy) return s[0];
    if (!dy) {
        int v = 0;
#pragma unroll
        for (int t = 0; t < 8; t++) v += s[t - 3] * kMcLumaHp[dx][t];
        return min(255, max(0, (v + 32) >> 6));
    }
    if (!dx) {
        int v = 0;
#pragma unroll
        for (int t = 0; t < 8; t++) v += s[(t - 3) * is] * kMcLumaHp[dy][t];
        return min(255, max(0, (v + 32) >> 6));
    }
    int v = 0;
#pragma unroll
    for (int t = 0; t < 8; t++) {
        const pel *r = s + (t - 3) * is;
        int hs = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) hs += r[k - 3] * kMcLumaHp[dx][k];
        v += (int)(s16)hs * kMcLumaHp[dy][t];
    }
    return min(255, max(0, (v + 2048) >> 12));
}

// com_mv_rounding_s32 with right shift 7: magnitude rounded to 1/16 sample
__device__ __forceinline__ s32 aff_round7(s32 v) { return v >= 0 ? (v + 64) >> 7 : -((-v + 64) >> 7); }

}  // namespace uc
