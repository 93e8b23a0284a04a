// Affine motion-compensation helpers shared by the affine CU prediction (mc.cu) and the affine
// motion search (affme.cu): the 1/16-sample luma filters and the sub-block MV rounding.  The
// reference's com_mc_blk_luma with hp_flag 1 always filters from the integer plane (its plane
// shortcut tests dy == 0 and dy == 8 together and never applies).
#pragma once
#include "common.cuh"

namespace uc {

// 1/16-sample luma filters (com_tbl_mc_l_coeff_hp, src/com_tables.c:130-147), the rows packed 4
// signed taps per word (taps 0..3, taps 4..7) for dp4a, in global memory so that lanes reading
// different phases do not serialise as they would on the constant cache
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

// One column of a sub-block of com_mc_blk_luma with hp_flag 1: the SUB samples at column dc of
// the sub-block whose 1/16-sample position is (qx, qy), clipped as the reference clips it to
// [-MAX_CU_SIZE - 4, picture size + 4].  The 8-tap horizontal filter of SUB + 7 rows (two dp4a
// per row on the row's 8 bytes), then the vertical filter of those sums.  The reference's copy and
// 1-D cases are this 2-D formula with the phase-0 taps {0,0,0,64,0,0,0,0}: 64 s through
// (v + 2048) >> 12 gives (s * 64 + 32) >> 6 exactly, so one path serves all four.  The aligned
// word loads reach at most 3 samples beyond each end of the 8-tap window (inside a 144-sample
// padding at the clipped positions).
template <int SUB>
__device__ __forceinline__ void aff_luma_column(const pel *plane, int i_ref, int W, int H, int qx, int qy, int dc,
                                                int *out)
{
    const int sx = min(max(qx >> 4, -128 - 4), W + 4), sy = min(max(qy >> 4, -128 - 4), H + 4);
    const u32 hlo = kMcLumaHpPacked[qx & 15][0], hhi = kMcLumaHpPacked[qx & 15][1];
    const u32 vlo = kMcLumaHpPacked[qy & 15][0], vhi = kMcLumaHpPacked[qy & 15][1];
    int cv[8];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        cv[k] = (int)(s8)(u8)(vlo >> (8 * k));
        cv[k + 4] = (int)(s8)(u8)(vhi >> (8 * k));
    }
    const pel *s = plane + (long long)(sy - 3) * i_ref + sx + dc - 3;
    int hs[SUB + 7];
#pragma unroll
    for (int r = 0; r < SUB + 7; r++) {
        const unsigned long long a = (unsigned long long)(s + (long long)r * i_ref);
        const u32 *aw = (const u32 *)(a & ~3ull);
        const u32 sh = (u32)(a & 3) * 8;
        const u32 w0 = aw[0], w1 = aw[1], w2 = aw[2];
        hs[r] = dp4a_us(__funnelshift_r(w1, w2, sh), hhi, dp4a_us(__funnelshift_r(w0, w1, sh), hlo, 0));
    }
#pragma unroll
    for (int o = 0; o < SUB; o++) {
        int v = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) v += hs[o + k] * cv[k];
        out[o] = min(255, max(0, (v + 2048) >> 12));
    }
}

// com_mv_rounding_s32 with right shift 7: magnitude rounded to 1/16 sample
__device__ __forceinline__ s32 aff_round7(s32 v) { return v >= 0 ? (v + 64) >> 7 : -((-v + 64) >> 7); }

}  // namespace uc
