// Luma intra prediction evaluated per sample (device), bit-exact with com_intra_pred
// (src/com_ipred.c:733-779) and the C kernel-table entries it dispatches to.
//
// Every sample of every mode is a closed-form function of the neighbour array and a few
// per-block constants, so a CTA can compute any subset of (mode, sample) pairs in parallel:
//   - DC: one per-block average (ipred_dc, :130-162);
//   - plane: per-block slopes b, c and origin (ipred_plane, :164-210);
//   - bilinear: the running sums of ipred_bi (:256-310) in closed form;
//   - angular: the generic x / xy / y kernels (ipred_ang_x :844, ipred_ang_xy :1138,
//     xPredIntraAngAdi_Y :1003) -- the specialised table entries equal them except mode 10
//     and 26 (no end-of-reference clamp) and mode 32 (its own padding of the filtered line,
//     xPredIntraAngAdi_Y_32 :1103);
//   - IPF (ipf_core :615, ipf_core_s16 :669): a per-sample blend with the left/top
//     references, applied to the unfiltered value of the same sample.
#pragma once
#include "common.cuh"

namespace uc {

__device__ __constant__ static const s8 kDirDxDy[2][33][2] = {
    { {0,0},{0,0},{0,0},{11,2},{2,0},{11,3},{1,0},{93,7},{1,1},{93,8},{1,2},{1,3},{0,0},{1,3},{1,2},
      {93,8},{1,1},{93,7},{1,0},{11,3},{2,0},{11,2},{4,0},{8,0},{0,0},{8,0},{4,0},{11,2},{2,0},{11,3},
      {1,0},{93,7},{1,1} },
    { {0,0},{0,0},{0,0},{93,8},{1,1},{93,7},{1,0},{11,3},{2,0},{11,2},{4,0},{8,0},{0,0},{8,0},{4,0},
      {11,2},{2,0},{11,3},{1,0},{93,7},{1,1},{93,8},{1,2},{1,3},{0,0},{1,3},{1,2},{93,8},{1,1},{93,7},
      {1,0},{11,3},{2,0} },
};

__device__ __constant__ static const u8 kIpfParam[5][10] = {
    { 24, 6, 2, 0, 0, 0, 0, 0, 0, 0 },
    { 44, 25, 14, 8, 4, 2, 1, 1, 0, 0 },
    { 40, 27, 19, 13, 9, 6, 4, 3, 2, 1 },
    { 36, 27, 21, 16, 12, 9, 7, 5, 4, 3 },
    { 52, 44, 37, 31, 26, 22, 18, 15, 13, 11 },
};

__host__ __device__ __forceinline__ int ilog2i(int v) { return 31 - __builtin_clz((unsigned)v); }
__device__ __forceinline__ int ilog2d(int v) { return 31 - __clz(v); }

// per-block constants of one CU's neighbour array (s = centre of the array)
struct IpredBlock {
    int w, h, lw, lh, avail, bd;
    int dc;                       // ipred_dc value
    int pl_b, pl_c, pl_t;         // plane slopes / origin
    int bi_a, bi_b, bi_wt;        // bilinear corner values and weight
};

__device__ __forceinline__ void ipred_block_setup(const pel *s, int w, int h, int avail, int bd, IpredBlock &B)
{
    B.w = w; B.h = h; B.lw = ilog2d(w); B.lh = ilog2d(h); B.avail = avail; B.bd = bd;
    // DC
    int dc = 0;
    if (avail & 2) {
        for (int i = 0; i < h; i++) dc += s[-i - 1];
        if (avail & 1) {
            for (int j = 0; j < w; j++) dc += s[j + 1];
            dc = (dc + ((w + h) >> 1)) * (4096 / (w + h)) >> 12;
        } else {
            dc = (dc + (h >> 1)) >> B.lh;
        }
    } else if (avail & 1) {
        for (int j = 0; j < w; j++) dc += s[j + 1];
        dc = (dc + (w >> 1)) >> B.lw;
    } else {
        dc = 1 << (bd - 1);
    }
    B.dc = dc;
    // plane
    const int mult[5] = { 13, 17, 5, 11, 23 }, shf[5] = { 7, 10, 11, 15, 19 };
    int w2 = w >> 1, h2 = h >> 1, iw = B.lw - 2, ih = B.lh - 2;
    int ch = 0, cv = 0;
    for (int x = 1; x <= w2; x++) ch += x * (s[w2 + x] - s[w2 - x]);
    for (int y = 1; y <= h2; y++) cv += y * (s[-h2 - y] - s[-h2 + y]);
    int a = (s[-h] + s[w]) << 4;
    B.pl_b = ((ch << 5) * mult[iw] + (1 << (shf[iw] - 1))) >> shf[iw];
    B.pl_c = ((cv << 5) * mult[ih] + (1 << (shf[ih] - 1))) >> shf[ih];
    B.pl_t = a - (h2 - 1) * B.pl_c - (w2 - 1) * B.pl_b + 16;
    // bilinear
    const int tbl_wc[6] = { -1, 21, 13, 7, 4, 2 };
    int ish = min(B.lw, B.lh);
    int wc = tbl_wc[B.lw > B.lh ? B.lw - B.lh : B.lh - B.lw];
    int ba = s[w], bb = s[-h];
    int bc = (w == h) ? (ba + bb + 1) >> 1 : (((ba << B.lw) + (bb << B.lh)) * wc + (1 << (ish + 5))) >> (ish + 6);
    B.bi_a = ba; B.bi_b = bb; B.bi_wt = (bc << 1) - ba - bb;
}

__device__ __forceinline__ int ang_ctx(int mode, int xy, int d, int *off)
{
    int mult = kDirDxDy[xy][mode][0], sh = kDirDxDy[xy][mode][1];
    int dn = d * mult >> sh;
    *off = ((d * mult * 32) >> sh) - dn * 32;
    return dn;
}

__device__ __forceinline__ int f4tap(int p0, int p1, int p2, int p3, int off)
{
    return (p0 * (32 - off) + p1 * (64 - off) + p2 * (32 + off) + p3 * off + 64) >> 7;
}

// unfiltered angular sample (modes 3..11, 13..23, 25..32; 12/24 are handled by the caller)
__device__ __forceinline__ int ang_sample(const pel *s, int mode, int w, int h, int i, int j)
{
    if (mode < 12) {
        int off, idx = ang_ctx(mode, 0, j + 1, &off);
        int pw = mode == 10 ? w : min(w, 2 * w - idx + 1);
        const pel *p;
        if (pw <= 0) p = s + 2 * w;
        else p = s + idx + min(i, pw - 1);
        return f4tap(p[0], p[1], p[2], p[3], off);
    }
    if (mode < 24) {
        int oy, xs = ang_ctx(mode, 1, i + 1, &oy);
        int yy = j - xs;
        if (yy <= -1) {
            int ox, ix = ang_ctx(mode, 0, j + 1, &ox);
            const pel *px = s - ix + i;
            return (px[2] * (32 - ox) + px[1] * (64 - ox) + px[0] * (32 + ox) + px[-1] * ox + 64) >> 7;
        }
        return (s[-yy - 2] * (32 - oy) + s[-yy - 1] * (64 - oy) + s[-yy] * (32 + oy) + s[-yy + 1] * oy + 64) >> 7;
    }
    if (mode == 32) {
        int rs = min(h / 2 + w - 1, h);
        int n = (j >> 1) + i;
        int b;
        if (n >= rs) b = -1 - 2 * rs + 1;          // the pad value: filtered line 1 at rs - 1
        else b = (j & 1) ? -3 - 2 * n : -2 - 2 * n;
        if (n >= rs) return (s[-1 - 2 * rs] + 2 * s[-2 - 2 * rs] + s[-3 - 2 * rs] + 2) >> 2;
        return (s[b] + 2 * s[b - 1] + s[b - 2] + 2) >> 2;
    }
    int off, xs = ang_ctx(mode, 1, i + 1, &off);
    int idx = -j - xs;
    if (mode != 26) idx = max(-2 * h, idx);
    return f4tap(s[idx], s[idx - 1], s[idx - 2], s[idx - 3], off);
}

// final prediction sample of com_intra_pred(ipm, ipf) at (i, j); with CW, CH > 0 the block is
// known at compile time to be CW x CH at 8 bits (B's size fields are then not read)
template <int CW = 0, int CH = 0>
__device__ __forceinline__ int ipred_sample(const pel *s, const IpredBlock &B, int ipm, int ipf, int i, int j)
{
    constexpr bool K = CW > 0 && CH > 0;
    const int w = K ? CW : B.w, h = K ? CH : B.h, mx = K ? 255 : (1 << B.bd) - 1;
    const int blw = K ? ilog2d(CW) : B.lw, blh = K ? ilog2d(CH) : B.lh;
    int v;
    bool s16path = false;
    if (ipm == 1) {                                         // plane
        v = (B.pl_t + j * B.pl_c + i * B.pl_b) >> 5;
        s16path = true;
    } else if (ipm == 2) {                                  // bilinear
        int lxy = blw + blh + 1, offs = 1 << (blw + blh);
        int up = s[i + 1], le = s[-j - 1];
        int predx = (le << blw) + (i + 1) * (B.bi_a - le);
        int refup = (up << blh) + (j + 1) * (B.bi_b - up);
        v = ((predx << blh) + (refup << blw) + i * j * B.bi_wt + offs) >> lxy;
        s16path = true;
    } else if (ipm == 0) {
        v = B.dc;
    } else if (ipm == 12) {
        v = s[1 + i];
    } else if (ipm == 24) {
        v = s[-1 - j];
    } else {
        v = ang_sample(s, ipm, w, h, i, j);
    }
    if (s16path && !ipf) return min(mx, max(0, v));
    if (!ipf) return v;
    // IPF ranges (ipf_core / ipf_core_s16)
    int ih = blw - 2, iv = blh - 2;
    int vr = min(h, 10), hr = min(w, 10);
    if (ih > 4) { ih = 4; hr = 0; }
    if (iv > 4) { iv = 4; vr = 0; }
    if (ipm >= 3 && ipm <= 18) vr = 0;
    if (ipm > 18) hr = 0;
    int cl = i < hr ? kIpfParam[ih][i] : 0;
    int ct = j < vr ? kIpfParam[iv][j] : 0;
    if (j < vr || i < hr) v = (cl * s[-j - 1] + ct * s[1 + i] + (64 - cl - ct) * v + 32) >> 6;
    if (s16path) v = min(mx, max(0, v));
    return v;
}

}  // namespace uc
