/*
 * oracle.c -- CPU restatement of uavs3e's mode-decision kernels (8-bit luma).
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Each function cites the reference function whose
 * algorithm it restates; file:line are relative to the uavs3e source tree.  The code is
 * written for clarity, not speed, except where a batched workload would otherwise not
 * finish in seconds (those loops use OpenMP).
 */
#include "oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MIN(a, b) ((a) < (b) ? (a) : (b))
#define MAX(a, b) ((a) > (b) ? (a) : (b))
#define CLIP3(lo, hi, v) MAX((lo), MIN((hi), (v)))
#define ABSI(a) ((a) < 0 ? -(a) : (a))

static int ilog2(int v) { int r = 0; while ((1 << (r + 1)) <= v) r++; return r; }

/* =============================================================================== tables */

/* 8-tap luma / 4-tap chroma quarter/eighth-sample filters, src/com_tables.c:149-154,191-200 */
static const s8 MC_L[4][8] = {
    { 0, 0, 0, 64, 0, 0, 0, 0 },
    { -1, 4, -10, 57, 19, -7, 3, -1 },
    { -1, 4, -11, 40, 40, -11, 4, -1 },
    { -1, 3, -7, 19, 57, -10, 4, -1 },
};
static const s8 MC_C[8][4] = {
    { 0, 64, 0, 0 }, { -4, 62, 6, 0 }, { -6, 56, 15, -1 }, { -5, 47, 25, -3 },
    { -4, 36, 36, -4 }, { -3, 25, 47, -5 }, { -1, 15, 56, -6 }, { 0, 6, 62, -4 },
};

/* intra angle steps {multiplier, shift}: [0] along x for row offsets, [1] along y for column
 * offsets; src/com_tables.c:402-423 */
static const s8 DIR_DXDY[2][33][2] = {
    { {0,0},{0,0},{0,0},{11,2},{2,0},{11,3},{1,0},{93,7},{1,1},{93,8},{1,2},{1,3},{0,0},{1,3},{1,2},
      {93,8},{1,1},{93,7},{1,0},{11,3},{2,0},{11,2},{4,0},{8,0},{0,0},{8,0},{4,0},{11,2},{2,0},{11,3},
      {1,0},{93,7},{1,1} },
    { {0,0},{0,0},{0,0},{93,8},{1,1},{93,7},{1,0},{11,3},{2,0},{11,2},{4,0},{8,0},{0,0},{8,0},{4,0},
      {11,2},{2,0},{11,3},{1,0},{93,7},{1,1},{93,8},{1,2},{1,3},{0,0},{1,3},{1,2},{93,8},{1,1},{93,7},
      {1,0},{11,3},{2,0} },
};

/* intra prediction filter weights per block-size class, src/com_ipred.c:607-613 */
static const u8 IPF_PARAM[5][10] = {
    { 24, 6, 2, 0, 0, 0, 0, 0, 0, 0 },
    { 44, 25, 14, 8, 4, 2, 1, 1, 0, 0 },
    { 40, 27, 19, 13, 9, 6, 4, 3, 2, 1 },
    { 36, 27, 21, 16, 12, 9, 7, 5, 4, 3 },
    { 52, 44, 37, 31, 26, 22, 18, 15, 13, 11 },
};

/* quantiser scale per QP, src/quant.c:56-67 */
static const u16 Q_SCALE[80] = {
    16302, 15024, 13777, 12634, 11626, 10624, 9742, 8958, 8192, 7512, 6889, 6305, 5793, 5303, 4878, 4467,
    4091, 3756, 3444, 3161, 2894, 2654, 2435, 2235, 2048, 1878, 1722, 1579, 1449, 1329, 1218, 1117,
    1024, 939, 861, 790, 724, 664, 609, 558, 512, 470, 430, 395, 362, 332, 304, 279,
    256, 235, 215, 197, 181, 166, 152, 140, 128, 116, 108, 99, 91, 83, 76, 69,
    64, 59, 54, 49, 45, 41, 38, 35, 32, 30, 27, 25, 23, 21, 19, 18,
};
/* dequantiser scale and shift per QP, src/com_itdq.c:770-793 */
static const u32 DQ_SCALE[80] = {
    32768, 36061, 38968, 42495, 46341, 50535, 55437, 60424, 32932, 35734, 38968, 42495, 46177, 50535, 55109, 59933,
    65535, 35734, 38968, 42577, 46341, 50617, 55027, 60097, 32809, 35734, 38968, 42454, 46382, 50576, 55109, 60056,
    65535, 35734, 38968, 42495, 46320, 50515, 55109, 60076, 65535, 35744, 38968, 42495, 46341, 50535, 55099, 60087,
    65535, 35734, 38973, 42500, 46341, 50535, 55109, 60097, 32771, 35734, 38965, 42497, 46341, 50535, 55109, 60099,
    32768, 36061, 38968, 42495, 46341, 50535, 55437, 60424, 32932, 35734, 38968, 42495, 46177, 50535, 55109, 59933,
};
static const u8 DQ_SHIFT[80] = {
    14, 14, 14, 14, 14, 14, 14, 14, 13, 13, 13, 13, 13, 13, 13, 13, 13, 12, 12, 12, 12, 12, 12, 12,
    11, 11, 11, 11, 11, 11, 11, 11, 11, 10, 10, 10, 10, 10, 10, 10, 10, 9, 9, 9, 9, 9, 9, 9,
    9, 8, 8, 8, 8, 8, 8, 8, 7, 7, 7, 7, 7, 7, 7, 7, 6, 6, 6, 6, 6, 6, 6, 6, 5, 5, 5, 5, 5, 5, 5, 5,
};
/* 4x4 alternative transform and 8x8 secondary transform kernels, src/com_tables.c:98-110 */
static const s8 C4_TRANS[4][4] = { { 34, 58, 72, 81 }, { 77, 69, -7, -75 }, { 79, -33, -75, 58 }, { 55, -84, 73, -28 } };
static const s8 C8_TRANS[4][4] = { { 123, -35, -8, -3 }, { -32, -120, 30, 10 }, { 14, 25, 123, -22 }, { 8, 13, 19, 126 } };

static s8   DCT_TM[7][3 * 64 * 64];     /* [log2n][type][k][n] */
static int  DCT2_FOLD[7][64 * 64];       /* effective DCT2 matrix of the partial butterflies */
static int  DCT87_EFF[2][7][64 * 64];    /* effective DCT8 / DST7 matrices */
static u16 *SCAN[7][7];
static s32  RDOQ_ERR_SCALE[80][6];
static double TBL_SQRT[2];
static int  g_init = 0;

/* DCT2 / DCT8 / DST7 integer matrices: s = sqrt(N)*32 times the orthonormal basis, rounded
 * half away from zero; src/com_tables.c:222-278 */
static void build_dct_tables(void)
{
    const double PI = 3.14159265358979323846;
    for (int L = 1; L <= 6; L++) {
        int c = 1 << L;
        double s = sqrt((double)c) * 32;
        s8 *T = DCT_TM[L];
        for (int k = 0; k < c; k++) {
            for (int n = 0; n < c; n++) {
                double w0 = k == 0 ? sqrt(0.5) : 1;
                double v = cos(PI * (n + 0.5) * k / c) * w0 * sqrt(2.0 / c);
                T[0 * c * c + k * c + n] = (s8)(s * v + (v > 0 ? 0.5 : -0.5));
                v = cos(PI * (k + 0.5) * (n + 0.5) / (c + 0.5)) * sqrt(2.0 / (c + 0.5));
                T[1 * c * c + k * c + n] = (s8)(s * v + (v > 0 ? 0.5 : -0.5));
                v = sin(PI * (k + 0.5) * (n + 1) / (c + 0.5)) * sqrt(2.0 / (c + 0.5));
                T[2 * c * c + k * c + n] = (s8)(s * v + (v > 0 ? 0.5 : -0.5));
            }
        }
    }
    TBL_SQRT[0] = sqrt(4.0 * 8.0);
    TBL_SQRT[1] = sqrt(16.0 * 8.0);
}

/*
 * The reference's DCT2 butterflies (src/transform.c:57-251 forward, src/com_itdq.c:47-262
 * inverse) read only the first N/2^(l+1) entries of each matrix row and rebuild the rest from
 * the even/odd symmetry.  This computes the matrix they effectively apply, by running the
 * even/odd decomposition on unit vectors: row k uses the difference vector of level ctz(k)+1,
 * rows 0 and N/2 the final 2-entry sum vector.  With exact integer arithmetic (and mod-2^32
 * wrap-around) the matrix form gives the butterfly's results bit for bit.
 */
static void build_dct2_fold(void)
{
    for (int L = 2; L <= 6; L++) {
        int N = 1 << L;
        const s8 *tm = DCT_TM[L];
        int *F = DCT2_FOLD[L];
        for (int n = 0; n < N; n++) {
            int S[7][64], D[7][64];
            for (int i = 0; i < N; i++) S[0][i] = i == n;
            for (int l = 1; l < L; l++) {
                int len = N >> (l - 1);
                for (int i = 0; i < len / 2; i++) {
                    S[l][i] = S[l - 1][i] + S[l - 1][len - 1 - i];
                    D[l][i] = S[l - 1][i] - S[l - 1][len - 1 - i];
                }
            }
            for (int k = 0; k < N; k++) {
                const int *V; int len;
                if (k == 0 || k == N / 2) { V = S[L - 1]; len = 2; }
                else { int j = __builtin_ctz(k); V = D[j + 1]; len = N >> (j + 1); }
                int acc = 0;
                for (int i = 0; i < len; i++) acc += tm[k * N + i] * V[i];
                F[k * N + n] = acc;
            }
        }
    }
}

/* effective DCT8 (t=0) / DST7 (t=1) matrices: the 4-point kernels use fast forms built from
 * row 0 of the table (src/transform.c:416-432, 545-562; inverse src/com_itdq.c:428-452,
 * 543-566); larger sizes use the table as is. */
static void build_dct87(void)
{
    for (int L = 2; L <= 6; L++) {
        int N = 1 << L;
        for (int t = 0; t < 2; t++) {
            const s8 *tab = DCT_TM[L] + (t == 0 ? 1 : 2) * N * N;
            int *M = DCT87_EFF[t][L];
            if (N == 4) {
                int a = tab[0], b = tab[1], c = tab[2], d = tab[3];
                if (t == 0) {       /* DCT8 fast form uses b, c, d of row 0 */
                    int r[4][4] = { { c + d, b, c, d }, { b, 0, -b, -b }, { c, -b, -d, c + d }, { d, -b, c + d, -c } };
                    memcpy(M, r, sizeof(r));
                } else {            /* DST7 fast form uses a, b, c of row 0 */
                    int r[4][4] = { { a, b, c, a + b }, { c, c, 0, -c }, { a + b, -a, -c, b }, { b, -(a + b), c, -a } };
                    memcpy(M, r, sizeof(r));
                }
            } else {
                for (int i = 0; i < N * N; i++) M[i] = tab[i];
            }
        }
    }
}

/* zig-zag scan, src/com_util.c:1220-1268 */
static void build_scan(void)
{
    for (int ly = 1; ly <= 6; ly++) {
        for (int lx = 1; lx <= 6; lx++) {
            int sx = 1 << lx, sy = 1 << ly;
            u16 *s = (u16 *)malloc(sizeof(u16) * sx * sy);
            int pos = 0;
            s[pos++] = 0;
            for (int l = 1; l < sx + sy - 1; l++) {
                if (l & 1) {
                    int x = MIN(l, sx - 1), y = MAX(0, l - (sx - 1));
                    for (; x >= 0 && y < sy; x--, y++) s[pos++] = (u16)(y * sx + x);
                } else {
                    int y = MIN(l, sy - 1), x = MAX(0, l - (sy - 1));
                    for (; y >= 0 && x < sx; x++, y--) s[pos++] = (u16)(y * sx + x);
                }
            }
            SCAN[lx][ly] = s;
        }
    }
}

/* RDOQ error scale, src/quant.c:69-83 (8-bit) */
static void build_rdoq(void)
{
    for (int qp = 0; qp < 80; qp++) {
        for (int i = 0; i < 6; i++) {
            int tr_shift = 15 - 8 - (i + 1);
            double e = pow(2.0, 15 - tr_shift);
            e = e / Q_SCALE[qp] / 1;
            RDOQ_ERR_SCALE[qp][i] = (s32)(e * (double)(1 << 20));
        }
    }
}

void orc_init(void)
{
    if (g_init) return;
    build_dct_tables();
    build_dct2_fold();
    build_dct87();
    build_scan();
    build_rdoq();
    g_init = 1;
}

const s8 *orc_dct_table(int log2n) { orc_init(); return DCT_TM[log2n]; }
const u16 *orc_scan(int log2w, int log2h) { orc_init(); return SCAN[log2w][log2h]; }
const s8 *orc_mc_luma_coef(void) { return &MC_L[0][0]; }
const s8 *orc_mc_chroma_coef(void) { return &MC_C[0][0]; }
u16 orc_quant_scale(int qp) { return Q_SCALE[qp]; }
u32 orc_dq_scale(int qp) { return DQ_SCALE[qp]; }
u32 orc_dq_shift(int qp) { return DQ_SHIFT[qp]; }
s32 orc_rdoq_err_scale(int qp, int i) { orc_init(); return RDOQ_ERR_SCALE[qp][i]; }
double orc_tbl_sqrt(int i) { orc_init(); return TBL_SQRT[i]; }

/* MV-bits table (exp-Golomb-like lengths): tab[0]=1, |v| in [2^(e-1)-1, 2^e-2] -> 2e bits;
 * src/inter.c:2029-2057.  tab points at 2*offset+1 entries; the centre is tab[offset]. */
void orc_mvbits_table(u8 *tab, int offset)
{
    u8 *c = tab + offset;
    memset(tab, 0, (size_t)(2 * offset + 1));
    c[0] = 1;
    c[-1] = c[1] = 2;
    c[-2] = c[2] = 3;
    for (int e = 2;; e++) {
        int imax = MIN((1 << e) - 1, offset), imin = (1 << (e - 1)) - 1;
        for (int i = imin; i < imax; i++) c[-i] = c[i] = (u8)(e << 1);
        if (imax == offset) break;
    }
}

/* ================================================================================ costs */

/* DEFINE_SAD / DEFINE_SSD, src/com_cost.c:40-58, 117-137 */
u32 orc_sad(int w, int h, const pel *o, int io, const pel *p, int ip)
{
    u32 s = 0;
    for (int y = 0; y < h; y++, o += io, p += ip)
        for (int x = 0; x < w; x++) s += (u32)ABSI(o[x] - p[x]);
    return s;
}

u64 orc_ssd(int w, int h, const pel *o, int io, const pel *p, int ip)
{
    u64 s = 0;
    for (int y = 0; y < h; y++, o += io, p += ip)
        for (int x = 0; x < w; x++) { int d = o[x] - p[x]; s += (u64)(d * d); }
    return s;
}

/* in-place Walsh-Hadamard transform of n values with the given stride */
static void wht(int *v, int n, int stride)
{
    for (int h = 1; h < n; h <<= 1)
        for (int i = 0; i < n; i += h << 1)
            for (int j = i; j < i + h; j++) {
                int a = v[j * stride], b = v[(j + h) * stride];
                v[j * stride] = a + b;
                v[(j + h) * stride] = a - b;
            }
}

/*
 * Hadamard SATD of one tw x th tile, com_had_4x4/8x8/16x8/8x16/8x4/4x8
 * (src/com_cost.c:176-710).  Those functions apply complete 2-D Walsh-Hadamard transforms
 * whose butterfly order only permutes and negates outputs, so the sum of magnitudes equals
 * that of any WHT ordering.  Normalisation: 4x4 (s+1)>>1, 8x8 (s+2)>>2, 16x8/8x16 and
 * 8x4/4x8 (int)(s / sqrt(tw*th) * 2.0) in double.
 */
u32 orc_satd_tile(int tw, int th, const pel *o, int io, const pel *p, int ip)
{
    orc_init();
    int d[128];
    for (int y = 0; y < th; y++)
        for (int x = 0; x < tw; x++) d[y * tw + x] = o[y * io + x] - p[y * ip + x];
    for (int y = 0; y < th; y++) wht(d + y * tw, tw, 1);
    for (int x = 0; x < tw; x++) wht(d + x, th, tw);
    int s = 0;
    for (int i = 0; i < tw * th; i++) s += ABSI(d[i]);
    if (tw == 4 && th == 4) return (u32)((s + 1) >> 1);
    if (tw == 8 && th == 8) return (u32)((s + 2) >> 2);
    if (tw * th == 128) return (u32)(int)(s / TBL_SQRT[1] * 2.0);
    return (u32)(int)(s / TBL_SQRT[0] * 2.0);
}

/* com_had tiling by block shape, src/com_cost.c:712-812.  Square blocks whose side is not a
 * multiple of 8 (resp. 16) take a single 4x4 (resp. 8x8) tile at the top-left. */
u32 orc_had(int w, int h, const pel *o, int io, const pel *p, int ip, int bd)
{
    int shift = bd - 8, tw, th;
    if (w == h) {
        if (w & 7) return orc_satd_tile(4, 4, o, io, p, ip) >> shift;
        if (w & 15) return orc_satd_tile(8, 8, o, io, p, ip) >> shift;
        tw = 8; th = 8;
    } else if (w > h) {
        if (h == 4 || (h & 7)) { tw = 8; th = 4; }
        else { tw = 16; th = 8; }
    } else {
        if (w == 4 || (w & 7)) { tw = 4; th = 8; }
        else { tw = 8; th = 16; }
    }
    int sum = 0;
    for (int y = 0; y < h; y += th)
        for (int x = 0; x < w; x += tw)
            sum += (int)orc_satd_tile(tw, th, o + y * io + x, io, p + y * ip + x, ip);
    return (u32)(sum >> shift);
}

/* calc_satd_intra, src/util.c:200-229: power-of-two sides go to com_had, 12/24/48 sides are
 * split into three equal segments */
u32 orc_satd_intra(int w, int h, const pel *o, const pel *p, int io, int ip, int bd)
{
    int sw = w, sh = h, nw = 1, nh = 1;
    if (w & (w - 1)) { nw = 3; sw = w / 3; }
    if (h & (h - 1)) { nh = 3; sh = h / 3; }
    if (nw == 1 && nh == 1) return orc_had(w, h, o, io, p, ip, bd);
    u32 c = 0;
    for (int j = 0; j < nh; j++)
        for (int i = 0; i < nw; i++)
            c += orc_had(sw, sh, o + sw * i + sh * j * io, io, p + sw * i + sh * j * ip, ip, bd);
    return c;
}

/* ==================================================================================== MC */

/* mc_if_cpy, src/com_mc.c:645-654 */
void orc_ipcpy(const pel *s, int is, pel *d, int id, int w, int h)
{
    for (int y = 0; y < h; y++, s += is, d += id) memcpy(d, s, (size_t)w);
}

/* separable one-dimensional filters: type 0 = 8-tap horizontal, 1 = 4-tap horizontal,
 * 2 = 8-tap vertical, 3 = 4-tap vertical; (sum + 32) >> 6 clipped to [0, max_val].
 * mc_if_hor_luma / mc_if_ver_luma / mc_if_hor_chroma / mc_if_ver_chroma,
 * src/com_mc.c:461-491, 553-583 */
void orc_ipflt(int type, const pel *s, int is, pel *d, int id, int w, int h, const s8 *c, int max_val)
{
    int taps = (type == 0 || type == 2) ? 8 : 4;
    int step = (type >= 2) ? is : 1;
    int back = taps / 2 - 1;
    for (int y = 0; y < h; y++, s += is, d += id)
        for (int x = 0; x < w; x++) {
            int sum = 0;
            for (int t = 0; t < taps; t++) sum += s[x + (t - back) * step] * c[t];
            d[x] = (pel)CLIP3(0, max_val, (sum + 32) >> 6);
        }
}

/* two-pass filters: horizontal into s16 rows (8-bit: no rounding shift), then vertical with
 * (sum + 2048) >> 12; type 0 = 8-tap luma, 1 = 4-tap chroma.  mc_if_hor_ver_luma /
 * mc_if_hor_ver_chroma, src/com_mc.c:493-551, 585-643 */
void orc_ipflt_ext(int type, const pel *s, int is, pel *d, int id, int w, int h, const s8 *cx, const s8 *cy, int max_val)
{
    int taps = type == 0 ? 8 : 4, back = taps / 2 - 1;
    int shift1 = max_val == 255 ? 0 : 2, shift2 = max_val == 255 ? 12 : 10;
    int add1 = (1 << shift1) >> 1, add2 = 1 << (shift2 - 1);
    int rows = h + taps - 1;
    s16 *tmp = (s16 *)malloc(sizeof(s16) * (size_t)rows * w);
    const pel *sp = s - back * is;
    for (int r = 0; r < rows; r++, sp += is)
        for (int x = 0; x < w; x++) {
            int sum = 0;
            for (int t = 0; t < taps; t++) sum += sp[x + t - back] * cx[t];
            tmp[r * w + x] = (s16)(shift1 ? (sum + add1) >> shift1 : sum);
        }
    for (int y = 0; y < h; y++, d += id)
        for (int x = 0; x < w; x++) {
            int sum = 0;
            for (int t = 0; t < taps; t++) sum += tmp[(y + t) * w + x] * cy[t];
            d[x] = (pel)CLIP3(0, max_val, (sum + add2) >> shift2);
        }
    free(tmp);
}

/* com_img_padding(img, 1, 4) on one plane, src/com_util.c:103-160: the region
 * [-4, W+4) x [-4, H+4) is replicated outward to the full padding */
static void pad_plane4(pel *p0, int width, int height, int pad, int stride)
{
    int ext = pad - 4, rw = width + 8, rh = height + 8;
    pel *a = p0 - 4 * stride - 4;
    for (int y = 0; y < rh; y++) {
        pel *row = a + y * stride;
        memset(row - ext, row[0], (size_t)ext);
        memset(row + rw, row[rw - 1], (size_t)ext);
    }
    for (int y = 1; y <= ext; y++) memcpy(a - ext - y * stride, a - ext, (size_t)stride);
    for (int y = 1; y <= ext; y++) memcpy(a + (rh - 1 + y) * stride - ext, a + (rh - 1) * stride - ext, (size_t)stride);
}

/*
 * com_if_luma_frame, src/com_mc.c:760-800 (8-bit):
 *   horizontal phases (0,dx) over [-8, W+8) x [-8, H+8): clip((t + 32) >> 6), t kept as s16;
 *   vertical phases (dy,0) from the integer plane over [-4, W+4) x [-4, H+4);
 *   diagonal phases (dy,dx) from the s16 rows: clip((sum + 2048) >> 12);
 *   then every fractional plane is edge-padded from its [-4, W+4) x [-4, H+4) region.
 */
void orc_if_luma_frame(pel *plane0, pel **planes15, int width, int height, int pad, int stride)
{
    int tw = width + 16, th = height + 16;
    s16 *tmp[3];
    for (int i = 0; i < 3; i++) tmp[i] = (s16 *)malloc(sizeof(s16) * (size_t)tw * th);
    for (int y = -8; y < height + 8; y++) {
        const pel *s = plane0 + y * stride;
        for (int x = -8; x < width + 8; x++)
            for (int f = 1; f <= 3; f++) {
                int t = 0;
                for (int k = 0; k < 8; k++) t += s[x + k - 3] * MC_L[f][k];
                tmp[f - 1][(y + 8) * tw + x + 8] = (s16)t;
                planes15[f - 1][y * stride + x] = (pel)CLIP3(0, 255, (t + 32) >> 6);
            }
    }
    for (int y = -4; y < height + 4; y++)
        for (int x = -4; x < width + 4; x++)
            for (int f = 1; f <= 3; f++) {
                int t = 0;
                for (int k = 0; k < 8; k++) t += plane0[(y + k - 3) * stride + x] * MC_L[f][k];
                planes15[f * 4 - 1][y * stride + x] = (pel)CLIP3(0, 255, (t + 32) >> 6);
            }
    for (int dx = 1; dx <= 3; dx++)
        for (int y = -4; y < height + 4; y++)
            for (int x = -4; x < width + 4; x++)
                for (int dy = 1; dy <= 3; dy++) {
                    int t = 0;
                    for (int k = 0; k < 8; k++) t += tmp[dx - 1][(y + k - 3 + 8) * tw + x + 8] * MC_L[dy][k];
                    planes15[dy * 4 + dx - 1][y * stride + x] = (pel)CLIP3(0, 255, (t + 2048) >> 12);
                }
    for (int i = 0; i < 15; i++) pad_plane4(planes15[i], width, height, pad, stride);
    for (int i = 0; i < 3; i++) free(tmp[i]);
}

/* ================================================================================ pel ops */

/* DEFINE_DIFF / DEFINE_AVRG / com_recon, src/com_util.c:3068-3129 */
void orc_pel_diff(int w, int h, const pel *o, int io, const pel *p, int ip, s16 *r, int ir)
{
    for (int y = 0; y < h; y++, o += io, p += ip, r += ir)
        for (int x = 0; x < w; x++) r[x] = (s16)(o[x] - p[x]);
}

void orc_pel_avrg(int w, int h, pel *d, int id, const pel *s1, const pel *s2)
{
    for (int y = 0; y < h; y++, d += id, s1 += w, s2 += w)
        for (int x = 0; x < w; x++) d[x] = (pel)((s1[x] + s2[x] + 1) >> 1);
}

void orc_recon(const s16 *resi, const pel *pred, int ipred, int w, int h, pel *rec, int irec, int cbf, int bd)
{
    int mx = (1 << bd) - 1;
    for (int y = 0; y < h; y++, pred += ipred, rec += irec)
        for (int x = 0; x < w; x++) rec[x] = cbf ? (pel)CLIP3(0, mx, resi[y * w + x] + pred[x]) : pred[x];
}

/* ================================================================================= intra */

/* com_intra_get_nbr (luma), src/com_ipred.c:40-112.  nb_out[ORC_NEIB_MID] is the corner,
 * +1.. the top row (then the top-right run), -1.. the left column (then bottom-left run);
 * extensions stop at the first SCU whose "coded" flag is clear and are padded with the last
 * sample; unavailable sides take 1 << (bd-1). */
void orc_intra_get_nbr(int x, int y, int w, int h, const pel *src, int s_src, const pel *top, int lcu_size, int avail,
                       pel *nb_out, int scup, const u8 *coded, int i_scu, int bd)
{
    int wsc = w >> 2, hsc = h >> 2, unit = 4, i;
    const pel *srcT = (y % lcu_size == 0) ? top : src - s_src;
    const pel *srcTL = srcT - 1, *srcL = src - 1;
    pel *dst = nb_out + ORC_NEIB_MID;
    int def = 1 << (bd - 1);
    int range = MAX(w, h) * 4 + 4;
    (void)x;
    if (avail & 1) {                                   /* AVAIL_UP */
        pel *up = dst + 1;
        const pel *t = srcT;
        memcpy(up, t, (size_t)w);
        up += w; t += w;
        const u8 *m = coded + scup - i_scu + wsc;
        for (i = 0; i < wsc; i++, up += unit, t += unit) {
            if (!m[i]) break;
            memcpy(up, t, (size_t)unit);
        }
        memset(up, up[-1], (size_t)(range - (w + i * unit)));
    } else {
        memset(dst + 1, def, (size_t)range);
    }
    if (avail & 2) {                                   /* AVAIL_LE */
        pel *left = dst - 1;
        const pel *s = srcL;
        for (i = 0; i < h; i++, s += s_src) *left-- = *s;
        const u8 *m = coded + scup - 1 + hsc * i_scu;
        for (i = 0; i < hsc; i++) {
            if (!m[i * i_scu]) break;
            for (int j = 0; j < unit; j++, s += s_src) *left-- = *s;
        }
        int pads = range - h - i * unit;
        memset(left - pads + 1, left[1], (size_t)pads);
    } else {
        memset(dst - range, def, (size_t)range);
    }
    if (avail & 4) dst[0] = srcTL[0];                   /* AVAIL_UP_LE */
    else if (avail & 1) dst[0] = srcTL[1];
    else if (avail & 2) dst[0] = srcL[0];
    else dst[0] = (pel)def;
}

static int ang_ctx(int mode, int xy, int d, int *off)
{
    int mult = DIR_DXDY[xy][mode][0], sh = DIR_DXDY[xy][mode][1];
    int dn = d * mult >> sh;
    *off = ((d * mult * 32) >> sh) - dn * 32;
    return dn;
}

static inline int f4(int p0, int p1, int p2, int p3, int off)
{
    return (p0 * (32 - off) + p1 * (64 - off) + p2 * (32 + off) + p3 * off + 64) >> 7;
}

/*
 * Angular prediction as installed in the C kernel table (src/com_ipred.c:1647-1693):
 *   modes 3..11: ipred_ang_x (:844), whose row reads stop at 2w (the specialisations for
 *     4/6/8 match it; mode 10's ipred_ang_x_10 does not clamp);
 *   modes 12..23: ipred_ang_xy (:1138) (the specialisations 13..23 match it);
 *   modes 24..32: xPredIntraAngAdi_Y (:1003), whose column reads stop at -2h (mode 26's
 *     specialisation does not clamp; mode 32 follows xPredIntraAngAdi_Y_32 (:1103) which
 *     pads its two filtered lines after min(h/2+w-1, h) entries).
 * s points at the neighbour-array centre.
 */
static void ang_core(const pel *s, pel *dst, int i_dst, int mode, int w, int h)
{
    if (mode < 12) {
        for (int j = 0; j < h; j++, dst += i_dst) {
            int off, idx = ang_ctx(mode, 0, j + 1, &off);
            int pw = mode == 10 ? w : MIN(w, 2 * w - idx + 1);
            int i;
            for (i = 0; i < pw; i++) {
                const pel *p = s + idx + i;
                dst[i] = (pel)f4(p[0], p[1], p[2], p[3], off);
            }
            if (pw <= 0) {
                dst[0] = (pel)f4(s[2 * w], s[2 * w + 1], s[2 * w + 2], s[2 * w + 3], off);
                pw = 1;
            }
            for (; i < w; i++) dst[i] = dst[pw - 1];
        }
    } else if (mode < 24) {
        for (int j = 0; j < h; j++, dst += i_dst) {
            int ox, ix = ang_ctx(mode, 0, j + 1, &ox);
            for (int i = 0; i < w; i++) {
                int oy, xs = ang_ctx(mode, 1, i + 1, &oy);
                int yy = j - xs;
                if (yy <= -1) {
                    const pel *px = s - ix + i;
                    dst[i] = (pel)((px[2] * (32 - ox) + px[1] * (64 - ox) + px[0] * (32 + ox) + px[-1] * ox + 64) >> 7);
                } else {
                    dst[i] = (pel)((s[-yy - 2] * (32 - oy) + s[-yy - 1] * (64 - oy) + s[-yy] * (32 + oy) + s[-yy + 1] * oy + 64) >> 7);
                }
            }
        }
    } else if (mode == 32) {
        int rs = MIN(h / 2 + w - 1, h);
        int padv = (s[-1 - 2 * rs] + 2 * s[-2 - 2 * rs] + s[-3 - 2 * rs] + 2) >> 2;
        for (int j = 0; j < h; j++, dst += i_dst)
            for (int i = 0; i < w; i++) {
                int n = (j >> 1) + i;
                if (n >= rs) { dst[i] = (pel)padv; continue; }
                int b = (j & 1) ? -3 - 2 * n : -2 - 2 * n;
                dst[i] = (pel)((s[b] + 2 * s[b - 1] + s[b - 2] + 2) >> 2);
            }
    } else {
        for (int j = 0; j < h; j++, dst += i_dst)
            for (int i = 0; i < w; i++) {
                int off, xs = ang_ctx(mode, 1, i + 1, &off);
                int idx = -j - xs;
                if (mode != 26) idx = MAX(-2 * h, idx);
                dst[i] = (pel)f4(s[idx], s[idx - 1], s[idx - 2], s[idx - 3], off);
            }
    }
}

void orc_ipred_ang(const pel *nb, pel *dst, int i_dst, int mode, int w, int h)
{
    ang_core(nb + ORC_NEIB_MID, dst, i_dst, mode, w, h);
}

/* ipred_dc, src/com_ipred.c:130-162 */
void orc_ipred_dc(const pel *nb, pel *dst, int i_dst, int w, int h, int avail, int bd)
{
    const pel *s = nb + ORC_NEIB_MID;
    int dc = 0;
    if (avail & 2) {
        for (int i = 0; i < h; i++) dc += s[-i - 1];
        if (avail & 1) {
            for (int j = 0; j < w; j++) dc += s[j + 1];
            dc = (dc + ((w + h) >> 1)) * (4096 / (w + h)) >> 12;
        } else {
            dc = (dc + (h >> 1)) >> ilog2(h);
        }
    } else if (avail & 1) {
        for (int j = 0; j < w; j++) dc += s[j + 1];
        dc = (dc + (w >> 1)) >> ilog2(w);
    } else {
        dc = 1 << (bd - 1);
    }
    for (int y = 0; y < h; y++, dst += i_dst) memset(dst, dc, (size_t)w);
}

/* plane prediction parameters, ipred_plane / ipred_plane_ipf, src/com_ipred.c:164-254 */
static void plane_params(const pel *s, int w, int h, int *pb, int *pc, int *ptemp)
{
    static const int mult[5] = { 13, 17, 5, 11, 23 }, shf[5] = { 7, 10, 11, 15, 19 };
    int w2 = w >> 1, h2 = h >> 1, iw = ilog2(w) - 2, ih = ilog2(h) - 2;
    int ch = 0, cv = 0;
    for (int x = 1; x <= w2; x++) ch += x * (s[w2 + x] - s[w2 - x]);
    for (int y = 1; y <= h2; y++) cv += y * (s[-h2 - y] - s[-h2 + y]);
    int a = (s[-h] + s[w]) << 4;
    int b = ((ch << 5) * mult[iw] + (1 << (shf[iw] - 1))) >> shf[iw];
    int c = ((cv << 5) * mult[ih] + (1 << (shf[ih] - 1))) >> shf[ih];
    *pb = b; *pc = c;
    *ptemp = a - (h2 - 1) * c - (w2 - 1) * b + 16;
}

void orc_ipred_plane(const pel *nb, pel *dst, int i_dst, int w, int h, int bd)
{
    int b, c, t, mx = (1 << bd) - 1;
    plane_params(nb + ORC_NEIB_MID, w, h, &b, &c, &t);
    for (int y = 0; y < h; y++, t += c, dst += i_dst) {
        int t2 = t;
        for (int x = 0; x < w; x++, t2 += b) dst[x] = (pel)CLIP3(0, mx, t2 >> 5);
    }
}

void orc_ipred_plane_ipf(const pel *nb, s16 *dst, int w, int h)
{
    int b, c, t;
    plane_params(nb + ORC_NEIB_MID, w, h, &b, &c, &t);
    for (int y = 0; y < h; y++, t += c, dst += w) {
        int t2 = t;
        for (int x = 0; x < w; x++, t2 += b) dst[x] = (s16)(t2 >> 5);
    }
}

/* bilinear prediction, ipred_bi / ipred_bi_ipf, src/com_ipred.c:256-368.  Written per
 * sample: the running sums of the reference reduce to
 *   predx  = (ref_le[y] << lw) + (x+1)*(a - ref_le[y])
 *   ref_up = (ref_up[x] << lh) + (y+1)*(b - ref_up[x])
 *   wxy    = x * y * wt   (the inner loop adds wy[y] = y*wt after each sample) */
static int bi_sample(const pel *s, int w, int h, int x, int y)
{
    static const int tbl_wc[6] = { -1, 21, 13, 7, 4, 2 };
    int lw = ilog2(w), lh = ilog2(h), ish = MIN(lw, lh), lxy = lw + lh + 1;
    int off = 1 << (lw + lh);
    int wc = tbl_wc[lw > lh ? lw - lh : lh - lw];
    int a = s[w], b = s[-h];
    int c = (w == h) ? (a + b + 1) >> 1 : (((a << lw) + (b << lh)) * wc + (1 << (ish + 5))) >> (ish + 6);
    int wt = (c << 1) - a - b;
    int up = s[x + 1], le = s[-y - 1];
    int predx = (le << lw) + (x + 1) * (a - le);
    int refup = (up << lh) + (y + 1) * (b - up);
    int wxy = x * y * wt;
    return ((predx << lh) + (refup << lw) + wxy + off) >> lxy;
}

void orc_ipred_bi(const pel *nb, pel *dst, int i_dst, int w, int h, int bd)
{
    int mx = (1 << bd) - 1;
    for (int y = 0; y < h; y++, dst += i_dst)
        for (int x = 0; x < w; x++) dst[x] = (pel)CLIP3(0, mx, bi_sample(nb + ORC_NEIB_MID, w, h, x, y));
}

void orc_ipred_bi_ipf(const pel *nb, s16 *dst, int w, int h)
{
    for (int y = 0; y < h; y++, dst += w)
        for (int x = 0; x < w; x++) dst[x] = (s16)bi_sample(nb + ORC_NEIB_MID, w, h, x, y);
}

/* intra prediction filter ranges, ipf_core / ipf_core_s16, src/com_ipred.c:615-731 */
static void ipf_ranges(int ipm, int w, int h, int *hr, int *vr, const u8 **hp, const u8 **vp)
{
    int ih = ilog2(w) - 2, iv = ilog2(h) - 2;
    int vrange = MIN(h, 10), hrange = MIN(w, 10);
    if (ih > 4) { ih = 4; hrange = 0; }
    if (iv > 4) { iv = 4; vrange = 0; }
    if (ipm >= 3 && ipm <= 18) vrange = 0;   /* IPD_DIA_L .. IPD_DIA_R */
    if (ipm > 18) hrange = 0;
    *hr = hrange; *vr = vrange;
    *hp = IPF_PARAM[ih]; *vp = IPF_PARAM[iv];
}

void orc_ipf_core(const pel *nb, pel *dst, int i_dst, int ipm, int w, int h, int bd)
{
    const pel *s = nb + ORC_NEIB_MID, *top = s + 1;
    int hr, vr; const u8 *hp, *vp;
    (void)bd;
    ipf_ranges(ipm, w, h, &hr, &vr, &hp, &vp);
    for (int r = 0; r < h; r++, dst += i_dst) {
        if (r < vr) {
            int ct = vp[r];
            for (int c = 0; c < w; c++) {
                int cl = c < hr ? hp[c] : 0;
                int cur = 64 - cl - ct;
                dst[c] = (pel)((cl * s[-r - 1] + ct * top[c] + cur * dst[c] + 32) >> 6);
            }
        } else {
            for (int c = 0; c < hr; c++) {
                int cl = hp[c];
                dst[c] = (pel)((cl * s[-r - 1] + (64 - cl) * dst[c] + 32) >> 6);
            }
        }
    }
}

void orc_ipf_core_s16(const pel *nb, pel *dst, int i_dst, const s16 *pred, int ipm, int w, int h, int bd)
{
    const pel *s = nb + ORC_NEIB_MID, *top = s + 1;
    int hr, vr, mx = (1 << bd) - 1; const u8 *hp, *vp;
    ipf_ranges(ipm, w, h, &hr, &vr, &hp, &vp);
    for (int r = 0; r < h; r++, dst += i_dst, pred += w) {
        for (int c = 0; c < w; c++) {
            int cl = (c < hr) ? hp[c] : 0;
            int ct = (r < vr) ? vp[r] : 0;
            int v;
            if (r < vr || c < hr) v = (cl * s[-r - 1] + ct * top[c] + (64 - cl - ct) * pred[c] + 32) >> 6;
            else v = pred[c];
            dst[c] = (pel)CLIP3(0, mx, v);
        }
    }
}

/* com_intra_pred, src/com_ipred.c:733-779 (dst stride = w) */
void orc_intra_pred(const pel *nb, pel *dst, int ipm, int w, int h, int bd, int avail, int ipf)
{
    const pel *s = nb + ORC_NEIB_MID;
    if (ipm != 1 && ipm != 2) {
        if (ipm == 12) {
            for (int y = 0; y < h; y++) memcpy(dst + y * w, s + 1, (size_t)w);
        } else if (ipm == 24) {
            for (int y = 0; y < h; y++) memset(dst + y * w, s[-1 - y], (size_t)w);
        } else if (ipm == 0) {
            orc_ipred_dc(nb, dst, w, w, h, avail, bd);
        } else {
            ang_core(s, dst, w, ipm, w, h);
        }
        if (ipf) orc_ipf_core(nb, dst, w, ipm, w, h, bd);
    } else if (ipf) {
        s16 tmp[64 * 64];
        if (ipm == 1) orc_ipred_plane_ipf(nb, tmp, w, h);
        else orc_ipred_bi_ipf(nb, tmp, w, h);
        orc_ipf_core_s16(nb, dst, w, tmp, ipm, w, h, bd);
    } else {
        if (ipm == 1) orc_ipred_plane(nb, dst, w, w, h, bd);
        else orc_ipred_bi(nb, dst, w, w, h, bd);
    }
}

/* ============================================================================ transforms */

static inline int rnd_of(int shift) { return shift > 0 ? 1 << (shift - 1) : 0; }

/*
 * Forward DCT2 of a w x h residual (trans_dct2_wXhY, src/transform.c:253-412):
 * rows with shift log2w + bd - 10, then columns with shift log2h + 5, each pass rounded and
 * truncated to s16.  64-point passes produce only the first 32 outputs, so for w or h = 64
 * only the top-left 32-wide / 32-high part of dst is written (the rest is left untouched).
 */
void orc_trans_dct2(int log2w, int log2h, const s16 *src, s16 *dst, int bd)
{
    orc_init();
    int w = 1 << log2w, h = 1 << log2h;
    int kw = MIN(w, 32), kh = MIN(h, 32);
    int sh1 = log2w + bd - 10, sh2 = log2h + 5;
    const int *FW = DCT2_FOLD[log2w], *FH = DCT2_FOLD[log2h];
    s16 *t = (s16 *)malloc(sizeof(s16) * (size_t)w * h);   /* t[u*h + y] */
    for (int y = 0; y < h; y++)
        for (int u = 0; u < kw; u++) {
            int acc = 0;
            for (int x = 0; x < w; x++) acc += FW[u * w + x] * src[y * w + x];
            t[u * h + y] = (s16)((acc + rnd_of(sh1)) >> sh1);
        }
    for (int u = 0; u < kw; u++)
        for (int v = 0; v < kh; v++) {
            int acc = 0;
            for (int y = 0; y < h; y++) acc += FH[v * h + y] * t[u * h + y];
            dst[v * w + u] = (s16)((acc + rnd_of(sh2)) >> sh2);
        }
    free(t);
}

/* forward DCT8 (type 0) / DST7 (type 1) pass, tx_dct8_pbN / tx_dst7_pbN,
 * src/transform.c:416-671: input rows of N, output transposed with stride `line` */
void orc_trans_dct8_dst7(int type, int log2n, const s16 *src, s16 *dst, int shift, int line)
{
    orc_init();
    int N = 1 << log2n;
    const int *M = DCT87_EFF[type][log2n];
    for (int i = 0; i < line; i++, src += N)
        for (int k = 0; k < N; k++) {
            int acc = 0;
            for (int n = 0; n < N; n++) acc += M[k * N + n] * src[n];
            dst[k * line + i] = (s16)((acc + rnd_of(shift)) >> shift);
        }
}

/* 4x4 alternative transform passes and 8x8-corner secondary transform,
 * xCTr_4_1d_Hor/Vert, xTr2nd_8_1d_Hor/Vert, src/transform.c:674-764 */
static void c4_fwd(const s16 *src, s16 *dst, int shift, int vert)
{
    int t[4][4], rnd = rnd_of(shift);
    for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) t[i][j] = src[i * 4 + j];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            int sum = rnd;
            for (int k = 0; k < 4; k++) sum += C4_TRANS[i][k] * (vert ? t[k][j] : t[j][k]);
            sum = CLIP3(-32768, 32767, sum >> shift);
            if (vert) dst[i * 4 + j] = (s16)sum; else dst[j * 4 + i] = (s16)sum;
        }
}

static void sec_fwd(s16 *src, int stride, int vert)
{
    int t[4][4];
    for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) t[i][j] = src[i * stride + j];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            int sum = 64;
            for (int k = 0; k < 4; k++) sum += C8_TRANS[i][k] * (vert ? t[k][j] : t[j][k]);
            sum = CLIP3(-32768, 32767, sum >> 7);
            if (vert) src[i * stride + j] = (s16)sum; else src[j * stride + i] = (s16)sum;
        }
}

/* transform(), src/transform.c:772-797 (luma TB) */
void orc_transform(int tb_nxn, int blk_idx, s16 *coef, const s16 *resi, int log2w, int log2h, int bd, int sec, int alt4)
{
    orc_init();
    int sh1 = log2w + bd - 10, sh2 = log2h + 5;
    if (alt4 && log2w == 2 && log2h == 2) {
        s16 t[16];
        c4_fwd(resi, t, sh1 + 1, 0);
        c4_fwd(t, coef, sh2 + 1, 1);
        return;
    }
    if (tb_nxn) {
        s16 t[64 * 64];
        orc_trans_dct8_dst7(blk_idx & 1, log2w, resi, t, sh1, 1 << log2h);
        orc_trans_dct8_dst7(blk_idx >> 1, log2h, t, coef, sh2, 1 << log2w);
    } else {
        orc_trans_dct2(log2w, log2h, resi, coef, bd);
    }
    if (sec >> 1) sec_fwd(coef, 1 << log2w, 1);
    if (sec & 1) sec_fwd(coef, 1 << log2w, 0);
}

/*
 * Inverse DCT2 (itrans_dct2_hH_wW, src/com_itdq.c:264-423): columns with shift 5 clipped to
 * s16, then rows with shift 20 - bd clipped to [-2^bd, 2^bd - 1].  64-point passes read only
 * the first 32 coefficients.
 */
void orc_itrans_dct2(int log2h, int log2w, const s16 *coef, s16 *resi, int bd)
{
    orc_init();
    int w = 1 << log2w, h = 1 << log2h;
    int kw = MIN(w, 32), kh = MIN(h, 32);
    int sh2 = 20 - bd, mx = (1 << bd) - 1, mn = -(1 << bd);
    const int *FW = DCT2_FOLD[log2w], *FH = DCT2_FOLD[log2h];
    s16 *t = (s16 *)malloc(sizeof(s16) * (size_t)w * h);   /* t[y*w + u] */
    for (int u = 0; u < kw; u++)
        for (int y = 0; y < h; y++) {
            int acc = 0;
            for (int v = 0; v < kh; v++) acc += FH[v * h + y] * coef[v * w + u];
            t[y * w + u] = (s16)CLIP3(-32768, 32767, (acc + 16) >> 5);
        }
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            int acc = 0;
            for (int u = 0; u < kw; u++) acc += FW[u * w + x] * t[y * w + u];
            resi[y * w + x] = (s16)CLIP3(mn, mx, (acc + (1 << (sh2 - 1))) >> sh2);
        }
    free(t);
}

/* inverse DCT8 / DST7 pass, itx_dct8_pbN / itx_dst7_pbN, src/com_itdq.c:428-653: input
 * column i (stride `line`) -> output row i of N samples */
void orc_itrans_dct8_dst7(int type, int log2n, const s16 *coef, s16 *blk, int shift, int line, int max_v, int min_v)
{
    orc_init();
    int N = 1 << log2n;
    const int *M = DCT87_EFF[type][log2n];
    for (int i = 0; i < line; i++, blk += N)
        for (int j = 0; j < N; j++) {
            int acc = 0;
            for (int k = 0; k < N; k++) acc += coef[k * line + i] * M[k * N + j];
            blk[j] = (s16)CLIP3(min_v, max_v, (acc + rnd_of(shift)) >> shift);
        }
}

static void c4_inv(const s16 *src, s16 *dst, int shift, int vert, int bd)
{
    int t[4][4], rnd = rnd_of(shift);
    int lo = vert ? -32768 : -(1 << bd), hi = vert ? 32767 : (1 << bd) - 1;
    for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) t[i][j] = src[i * 4 + j];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            int sum = rnd;
            for (int k = 0; k < 4; k++) sum += C4_TRANS[k][i] * (vert ? t[k][j] : t[j][k]);
            sum = CLIP3(lo, hi, sum >> shift);
            if (vert) dst[i * 4 + j] = (s16)sum; else dst[j * 4 + i] = (s16)sum;
        }
}

static void sec_inv(s16 *src, int stride, int vert)
{
    int t[4][4];
    for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) t[i][j] = src[i * stride + j];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            int sum = 64;
            for (int k = 0; k < 4; k++) sum += C8_TRANS[k][i] * (vert ? t[k][j] : t[j][k]);
            sum = CLIP3(-32768, 32767, sum >> 7);
            if (vert) src[i * stride + j] = (s16)sum; else src[j * stride + i] = (s16)sum;
        }
}

/* com_dquant / com_dquant_wq, src/com_itdq.c:807-871 */
void orc_dquant(int flat, const s16 *coef, s16 *out, const u8 *wq4, const u8 *wq8, int log2w, int log2h, int scale, int shift, int bd)
{
    int w = 1 << log2w, h = 1 << log2h;
    int off = shift == 0 ? 0 : 1 << (shift - 1);
    int refix = (log2w + log2h) & 1;
    (void)bd;
    if (flat) {
        int n = MIN(h, 32) * w;
        for (int i = 0; i < n; i++) {
            int lev = (coef[i] * scale + off) >> shift;
            lev = CLIP3(-32768, 32767, lev);
            out[i] = (s16)(refix ? (lev * 181 + 128) >> 8 : lev);
        }
        return;
    }
    const u8 *wq; int ish, istep, ww;
    if (log2w == 2 && log2h == 2) { wq = wq4; ish = 0; istep = 1; ww = 4; }
    else { wq = wq8; ish = MAX(log2w, log2h) - 3; istep = 1 << ish; ww = 8; }
    for (int i = 0; i < h; i++) {
        for (int j = 0; j < w; j++) {
            int weight = ((i | j) & 0xE0) ? 0 : wq[j >> ish];
            int lev = (int)((((((s64)((coef[i * w + j] * weight) >> 2)) * scale) >> 4) + off) >> shift);
            lev = CLIP3(-32768, 32767, lev);
            if (refix) lev = (lev * 181 + 128) >> 8;
            out[i * w + j] = (s16)lev;
        }
        if ((i + 1) % istep == 0) wq += ww;
    }
}

/* com_invqt -> com_inv_trans, src/com_itdq.c:747-881 (luma TB) */
void orc_invqt(int tb_nxn, int blk_idx, const s16 *coef, s16 *resi, const u8 *wq4, const u8 *wq8, int log2w, int log2h, int qp, int bd, int sec, int alt4)
{
    orc_init();
    s16 dq[64 * 64];
    int log2_size = (log2w + log2h) >> 1;
    int scale = (int)DQ_SCALE[qp];
    int shift = (int)DQ_SHIFT[qp] - (15 - bd - log2_size) + 1;
    orc_dquant(wq4 == NULL, coef, dq, wq4, wq8, log2w, log2h, scale, shift, bd);
    if (alt4 && log2w == 2 && log2h == 2) {
        s16 t[16];
        c4_inv(dq, t, 5, 1, bd);
        c4_inv(t, resi, 20 - bd + 2, 0, bd);
        return;
    }
    int stride = 1 << log2w;
    if (sec & 1) sec_inv(dq, stride, 0);
    if (sec >> 1) sec_inv(dq, stride, 1);
    if (tb_nxn) {
        s16 t[64 * 64];
        orc_itrans_dct8_dst7(blk_idx >> 1, log2h, dq, t, 5, 1 << log2w, 32767, -32768);
        orc_itrans_dct8_dst7(blk_idx & 1, log2w, t, resi, 20 - bd, 1 << log2h, (1 << bd) - 1, -(1 << bd));
    } else {
        orc_itrans_dct2(log2h, log2w, dq, resi, bd);
    }
}

/* quant_check / quant_rdoq (first RDOQ pass), src/com_itdq.c:910-954 */
int orc_quant_check(const s16 *coef, int num, int threshold)
{
    for (int i = 0; i < (num >> 2) * 4; i++)
        if (coef[i] > threshold || coef[i] < -threshold) return 0;
    return 1;
}

int orc_quant_rdoq(const s16 *coef, int num, int q_value, int q_bits, s32 err_scale, int precision_bits,
                   u32 *abs_coef, s16 *abs_level, s64 *uncoded_err)
{
    s32 add = 1 << (q_bits - 1);
    int last = -1;
    int thr = ((1 << (q_bits - 1)) - 1) / q_value + 1;
    for (int i = 0; i < num; i++) {
        int a = ABSI((int)coef[i]);
        if (a < thr) { abs_level[i] = 0; continue; }
        u32 ld = (u32)a * (u32)q_value;
        s64 err = ((s64)ld * err_scale) >> precision_bits;
        abs_level[i] = (s16)(u32)(((u64)ld + (u64)add) >> q_bits);
        abs_coef[i] = ld;
        uncoded_err[i] = err * err;
        last = i;
    }
    return last;
}

/* ===================================================================== batched: motion */

typedef struct { int minx, maxx, miny, maxy; } mvrange_t;

/* get_max_search_range with is_padding = 1, mvr 0, mvp 0 (src/me.c:502-527) clipped to the
 * [-range, range] full-search window */
static mvrange_t me_range(int x, int y, int W, int H, int range)
{
    int mto = MAX(W, H);                        /* ((((max(W,H) << 2) + 3) << 0) >> 2) */
    mvrange_t r;
    r.minx = MAX(-range, MAX(-128 + 1 - x, -mto + 4));
    r.miny = MAX(-range, MAX(-128 + 1 - y, -mto + 4));
    r.maxx = MIN(range, MIN(W - 1 - x, mto - 4));
    r.maxy = MIN(range, MIN(H - 1 - y, mto - 4));
    return r;
}

/* com_mc_blk_luma_pointer, src/com_mc.c:89-101 */
static const pel *mc_pointer(const pel *const *planes, int i_ref, int qx, int qy, int maxx, int maxy)
{
    int dx = qx & 3, dy = qy & 3;
    int x = CLIP3(-128 - 4, maxx, qx >> 2), y = CLIP3(-128 - 4, maxy, qy >> 2);
    return planes[dy * 4 + dx] + y * i_ref + x;
}

/*
 * Batched motion search for one block and one reference:
 *   integer full search of cost = (SAD << 16) + (bits(4dx) + bits(4dy)) * lambda_mv, strict
 *   '<' in raster order (dy outer, dx inner) so the first minimum wins
 *   (cost_sad + GET_MVBITS_IPEL_*, src/me.c:103-197);
 *   then me_sub_pel_search with SATD cost (subpel_cost_type 0, src/me.c:366-500): centre,
 *   8 half-sample points around the integer winner, 8 quarter-sample points around the
 *   half-sample winner, cost = bits * lambda_mv + (satd << 16).
 */
static void me_one(const pel *org, int i_org, const pel *const *pl, int i_ref, int W, int H,
                   const orc_me_block_t *b, int range, u32 lambda, const u8 *bits, orc_me_result_t *o)
{
    static const s8 HP[8][2] = { { -2, 0 }, { -2, 2 }, { 0, 2 }, { 2, 2 }, { 2, 0 }, { 2, -2 }, { 0, -2 }, { -2, -2 } };
    static const s8 QP[8][2] = { { -1, 0 }, { 0, 1 }, { 1, 0 }, { 0, -1 }, { -1, 1 }, { 1, 1 }, { -1, -1 }, { 1, -1 } };
    int x = b->x, y = b->y, w = b->w, h = b->h;
    const pel *o0 = org + y * i_org + x;
    const pel *ref = pl[0] + y * i_ref + x;
    mvrange_t r = me_range(x, y, W, H, range);
    u64 best = ~(u64)0; int bx = 0, by = 0; u32 bsad = 0;
    for (int dy = r.miny; dy <= r.maxy; dy++)
        for (int dx = r.minx; dx <= r.maxx; dx++) {
            u32 sad = orc_sad(w, h, o0, i_org, ref + dy * i_ref + dx, i_ref);
            u64 c = ((u64)sad << 16) + (u64)(bits[4 * dx] + bits[4 * dy]) * lambda;
            if (c < best) { best = c; bx = dx; by = dy; bsad = sad; }
        }
    o->mv_int[0] = (s16)bx; o->mv_int[1] = (s16)by; o->sad_int = bsad; o->cost_int = best;

    int maxx = W + 4, maxy = H + 4;
    int cx = bx * 4, cy = by * 4;
    u32 satd = orc_had(w, h, o0, i_org, ref + by * i_ref + bx, i_ref, 8);
    u64 cbest = (u64)((u32)(bits[cx] + bits[cy]) * lambda) + ((u64)satd << 16);
    int mx = cx, my = cy; u32 bsatd = satd;
    for (int i = 0; i < 8; i++) {
        int vx = cx + HP[i][0], vy = cy + HP[i][1];
        const pel *p = mc_pointer(pl, i_ref, vx + (x << 2), vy + (y << 2), maxx, maxy);
        u32 s = orc_had(w, h, o0, i_org, p, i_ref, 8);
        u64 c = (u64)((u32)(bits[vx] + bits[vy]) * lambda) + ((u64)s << 16);
        if (c < cbest) { cbest = c; mx = vx; my = vy; bsatd = s; }
    }
    cx = mx; cy = my;
    for (int i = 0; i < 8; i++) {
        int vx = cx + QP[i][0], vy = cy + QP[i][1];
        const pel *p = mc_pointer(pl, i_ref, vx + (x << 2), vy + (y << 2), maxx, maxy);
        u32 s = orc_had(w, h, o0, i_org, p, i_ref, 8);
        u64 c = (u64)((u32)(bits[vx] + bits[vy]) * lambda) + ((u64)s << 16);
        if (c < cbest) { cbest = c; mx = vx; my = vy; bsatd = s; }
    }
    o->mv_sub[0] = (s16)mx; o->mv_sub[1] = (s16)my; o->satd_sub = bsatd; o->cost_sub = cbest;
}

void orc_me_frame(const pel *org, int i_org, const pel *const *planes, int i_ref, int width, int height,
                  int n_refs, const orc_me_block_t *blocks, int n_blocks, int range, u32 lambda_mv,
                  orc_me_result_t *out, int threads)
{
    orc_init();
    int off = (MAX(width, height) << 2) + 3;
    u8 *tab = (u8 *)malloc((size_t)(2 * off + 1));
    orc_mvbits_table(tab, off);
    const u8 *bits = tab + off;
#ifdef _OPENMP
    if (threads < 1) threads = 1;
    #pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
#endif
    for (int i = 0; i < n_blocks * n_refs; i++) {
        int b = i / n_refs, r = i % n_refs;
        me_one(org, i_org, planes + r * 16, i_ref, width, height, &blocks[b], range, lambda_mv, bits, &out[i]);
    }
    (void)threads;
    free(tab);
}

/* ===================================================================== batched: intra */

/* hash of a level block: sum over positions of level * weight(raster position) mod 2^32, with
 * the odd weight (i * 0x9E3779B1 + 0x7F4A7C15) | 1: any single changed level, sign flip or
 * exchange of two different levels changes it */
u32 orc_level_hash(const s16 *lev, int n)
{
    u32 hsh = 0;
    for (int i = 0; i < n; i++)
        hsh += (u32)(int)lev[i] * (((u32)i * 0x9E3779B1u + 0x7F4A7C15u) | 1u);
    return hsh;
}

/* quantisation of the lattice: rdoq_quant_block's quant_check early-out and its first pass
 * (src/quant.c:196-231), with levels kept (no second RDOQ pass). Returns the signed levels. */
static void lattice_quant(const s16 *coef, s16 *lev, int log2w, int log2h, int qp, int is_intra, orc_lat_q_t *q)
{
    int w = 1 << log2w, h = 1 << log2h, n = w * h;
    int odd = (log2w + log2h) & 1;
    int ns_shift = odd ? 7 : 0, ns_scale = odd ? 181 : 1, ns_off = odd ? 64 : 0;
    int log2_size = (log2w + log2h) >> 1;
    int tr_shift = 15 - 8 - log2_size;
    int q_bits = 14 + tr_shift;
    int q_value = (Q_SCALE[qp] * ns_scale + ns_off) >> ns_shift;
    int used = 1 << (log2w + MIN(5, log2h));
    int offset = (is_intra ? 201 : 153) << (q_bits - 9);
    int nz_thr = ((((1 << q_bits) - offset) << 10) / q_value - 1) >> 10;
    memset(lev, 0, sizeof(s16) * (size_t)n);
    q->num_nz = 0; q->last_nz = -1; q->sum_abs = 0;
    if (orc_quant_check(coef, used, nz_thr)) { q->coef_hash = orc_level_hash(lev, n); return; }
    const u16 *scan = SCAN[log2w][log2h];
    int thr = ((1 << (q_bits - 1)) - 1) / q_value + 1;
    for (int i = 0; i < n; i++) {
        int pos = scan[i];
        int a = ABSI((int)coef[pos]);
        if (a < thr) continue;
        u32 ld = (u32)a * (u32)q_value;
        int l = (int)(s16)(u32)(((u64)ld + (u64)(1u << (q_bits - 1))) >> q_bits);
        if (!l) continue;
        lev[pos] = (s16)(coef[pos] < 0 ? -l : l);
        q->num_nz++; q->last_nz = (s16)i; q->sum_abs += (u32)l;
    }
    q->coef_hash = orc_level_hash(lev, n);
}

void orc_intra_lattice(const pel *org, int i_org, const pel *rec, int i_rec, int width, int height,
                       const orc_cu_t *cus, int n_cus, int ipf, const int *qps, int n_qp, int is_intra_slice,
                       u32 *satd_out, orc_lat_q_t *q_out, int threads)
{
    orc_init();
    int i_scu = (width >> 2) + 2, h_scu = (height >> 2) + 2;
    u8 *coded = (u8 *)calloc((size_t)i_scu * h_scu, 1);
    for (int y = 1; y <= (height >> 2); y++)
        for (int x = 1; x <= (width >> 2); x++) coded[y * i_scu + x] = 1;
#ifdef _OPENMP
    if (threads < 1) threads = 1;
    #pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
#endif
    for (int c = 0; c < n_cus; c++) {
        const orc_cu_t *cu = &cus[c];
        int x = cu->x, y = cu->y, w = cu->w, h = cu->h;
        int lw = ilog2(w), lh = ilog2(h);
        int avail = (y > 0 ? 1 : 0) | (x > 0 ? 2 : 0) | ((x > 0 && y > 0) ? 4 : 0);
        pel nb[ORC_NEIB_SIZE];
        int scup = (y >> 2) * i_scu + (x >> 2) + i_scu + 1;   /* map origin offset by the border */
        const pel *src = rec + y * i_rec + x;
        orc_intra_get_nbr(x, y, w, h, src, i_rec, src - i_rec, 1 << 30, avail, nb, scup, coded, i_scu, 8);
        const pel *o = org + y * i_org + x;
        pel pred[64 * 64], recon[64 * 64];
        s16 resi[64 * 64], coef[64 * 64], lev[64 * 64], rr[64 * 64];
        for (int m = 0; m < 33; m++) {
            orc_intra_pred(nb, pred, m, w, h, 8, avail, ipf);
            satd_out[c * 33 + m] = orc_satd_intra(w, h, o, pred, i_org, w, 8);
            orc_pel_diff(w, h, o, i_org, pred, w, resi, w);
            memset(coef, 0, sizeof(coef));
            orc_trans_dct2(lw, lh, resi, coef, 8);
            for (int q = 0; q < n_qp; q++) {
                orc_lat_q_t *qo = &q_out[((size_t)c * 33 + m) * n_qp + q];
                lattice_quant(coef, lev, lw, lh, qps[q], is_intra_slice, qo);
                if (qo->num_nz) {
                    orc_invqt(0, 0, lev, rr, NULL, NULL, lw, lh, qps[q], 8, 0, 0);
                    orc_recon(rr, pred, w, w, h, recon, w, 1, 8);
                } else {
                    orc_recon(rr, pred, w, w, h, recon, w, 0, 8);
                }
                qo->ssd = (u32)orc_ssd(w, h, o, i_org, recon, w);
            }
        }
    }
    (void)threads;
    free(coded);
}

/* ============================================================ batched: lookahead cost */

/* One motion search of loka_estimate_coding_cost: me_search_tz (src/me.c:529-568) on a 16x16
 * unit at integer resolution (curr_mvr 2), predictor (0,0), no bi-prediction, so the MV-bits
 * lookup GET_MVBITS_IPEL_* (inc/util.h:43-44) indexes the table with the integer MV itself. */
typedef struct {
    const pel *org; int i_org;          /* unit origin in the current picture            */
    const pel *ref; int i_ref;          /* co-located sample of the reference plane      */
    int minx, maxx, miny, maxy;         /* get_max_search_range, src/me.c:502-527        */
    u32 lambda;                         /* lambda_mv                                     */
    const u8 *bits;                     /* MV-bits table centre                          */
    u64 best; int mvx, mvy;             /* running best cost and MV                      */
} tz_ctx_t;

static u64 tz_cost(const tz_ctx_t *c, int mx, int my)
{
    u32 sad = orc_sad(16, 16, c->org, c->i_org, c->ref + my * c->i_ref + mx, c->i_ref);
    return ((u64)sad << 16) + (u64)((u32)(c->bits[mx] + c->bits[my]) * c->lambda);
}

static void tz_try(tz_ctx_t *c, int mx, int my, int *improved)
{
    u64 cost = tz_cost(c, mx, my);
    if (cost < c->best) { c->best = cost; c->mvx = mx; c->mvy = my; if (improved) *improved = 1; }
}

/* search_diamond with bi = 0 (src/me.c:199-334): the centre, the 5x5 core square (its edges
 * kept strictly inside the MV range, :240-243), then diamond rings of step 4, 8, 16 below
 * max_step (4 points at step 4, 8 at step 8, 16 at step 16, :307-331).  Returns the step of the
 * last ring point that improved the cost, else 2 if the core square moved the MV, else 0. */
static int tz_diamond(tz_ctx_t *c, int max_step)
{
    static const s8 RING_A[8][2] = { { -2, 0 }, { -1, 1 }, { 0, 2 }, { 1, 1 },
                                     { 2, 0 }, { 1, -1 }, { 0, -2 }, { -1, -1 } };
    static const s8 RING_B[16][2] = { { -4, 0 }, { -3, 1 }, { -2, 2 }, { -1, 3 }, { 0, 4 }, { 1, 3 },
                                      { 2, 2 }, { 3, 1 }, { 4, 0 }, { 3, -1 }, { 2, -2 }, { 1, -3 },
                                      { 0, -4 }, { -1, -3 }, { -2, -2 }, { -3, -1 } };
    const int cx = c->mvx, cy = c->mvy;
    int best_step = 0;
    tz_try(c, cx, cy, NULL);
    int x0 = MAX(cx - 2, c->minx + 1), x1 = MIN(cx + 2, c->maxx - 1);
    int y0 = MAX(cy - 2, c->miny + 1), y1 = MIN(cy + 2, c->maxy - 1);
    for (int my = y0; my <= y1; my++)
        for (int mx = x0; mx <= x1; mx++) tz_try(c, mx, my, NULL);
    if (c->mvx != cx || c->mvy != cy) best_step = 2;
    for (int step = 4, round = 0; step < max_step; step <<= 1, round++) {
        const s8(*ring)[2] = round < 2 ? RING_A : RING_B;
        int n = round < 2 ? 8 : 16, inc = round == 0 ? 2 : 1;
        int scale = round < 2 ? step >> 1 : step >> 2;
        for (int i = 0; i < n; i += inc) {
            int mx = cx + scale * ring[i][0], my = cy + scale * ring[i][1];
            if (mx < c->minx || mx > c->maxx || my < c->miny || my > c->maxy) continue;
            int imp = 0;
            tz_try(c, mx, my, &imp);
            if (imp) best_step = step;
        }
    }
    return best_step;
}

/* search_raster with adaptive_raster_range 0 (src/me.c:103-197, get_raster_range :65-100):
 * a grid of step 8 * (refi + 1) over [mv - range, mv + range] (clipped), then grids of the
 * halved step over [mv - step, mv + step] around the running best until the step is 1.
 * Each grid starts at its clipped lower corner. */
static void tz_raster(tz_ctx_t *c, int refi, int range)
{
    int step = MAX(5, 16 >> 1) * (refi + 1);
    int x0 = CLIP3(c->minx, c->maxx, c->mvx - range), x1 = CLIP3(c->minx, c->maxx, c->mvx + range);
    int y0 = CLIP3(c->miny, c->maxy, c->mvy - range), y1 = CLIP3(c->miny, c->maxy, c->mvy + range);
    for (int round = 0; step >= 1; round++, step >>= 1) {
        if (round) {
            x0 = MAX(c->mvx - step, c->minx); x1 = MIN(c->mvx + step, c->maxx);
            y0 = MAX(c->mvy - step, c->miny); y1 = MIN(c->mvy + step, c->maxy);
        }
        for (int my = y0; my <= y1; my += step)
            for (int mx = x0; mx <= x1; mx += step) tz_try(c, mx, my, NULL);
    }
}

/* get_ipred_neighbor, src/lookahead.c:40-80: neighbours of a w x h block taken from the
 * ORIGINAL picture -- 2w above and 2h to the left (cut at the picture edge, then the last
 * sample repeated up to 4 * max(w, h) + 4), the corner, 1 << (bd - 1) where unavailable */
static void loka_nbr(pel *nb, int x, int y, int w, int h, int W, int H, const pel *src, int s)
{
    pel *c = nb + ORC_NEIB_MID;
    int range = MAX(w, h) * 4 + 4, dflt = 128;
    if (y) {
        int n = MIN(2 * w, W - x);
        for (int i = 0; i < range; i++) c[1 + i] = src[-s + MIN(i, n - 1)];
    } else {
        for (int i = 0; i < range; i++) c[1 + i] = (pel)dflt;
    }
    if (x) {
        int n = MIN(2 * h, H - y);
        for (int i = 0; i < range; i++) c[-1 - i] = src[MIN(i, n - 1) * s - 1];
    } else {
        for (int i = 0; i < range; i++) c[-1 - i] = (pel)dflt;
    }
    c[0] = (x && y) ? src[-s - 1] : y ? src[-s] : x ? src[-1] : (pel)dflt;
}

/* cost_var (DEFINE_VAR, src/com_cost.c:139-151): sum of squares - (sum^2 >> 2 log2 n) */
static u64 loka_var(const pel *p, int s, int n)
{
    u64 sum = 0, sq = 0;
    for (int y = 0; y < n; y++, p += s)
        for (int x = 0; x < n; x++) { sum += p[x]; sq += (u64)(p[x] * p[x]); }
    return sq - ((sum * sum) >> (2 * ilog2(n)));
}

static void loka_unit(const orc_loka_cfg_t *cfg, const pel *org_y, int i_org, const pel *org_u, const pel *org_v,
                      int i_org_c, const pel *const *refs[2], int i_ref, const u8 *bits, u32 lambda,
                      int ux, int uy, orc_loka_unit_t *u)
{
    static const u8 IPM[11] = { 0, 1, 2, 4, 8, 12, 16, 20, 24, 28, 32 };   /* src/lookahead.c:213 */
    const int W = cfg->width, H = cfg->height, x = ux * 16, y = uy * 16;
    const int is_bi = cfg->num_ref[0] && cfg->num_ref[1];
    const pel *org = org_y + y * i_org + x;
    pel pred[256], best_pred[2][256];
    memset(u, 0, sizeof(*u));

    /* get_max_search_range (src/me.c:502-527) for mvp 0, mvr 2 */
    int mto = (MAX(W, H) << 2) + 3;
    tz_ctx_t c;
    c.org = org; c.i_org = i_org; c.i_ref = i_ref; c.lambda = lambda; c.bits = bits;
    if (cfg->is_padding) {
        c.minx = MAX(-128 + 1 - x, -mto + 4); c.miny = MAX(-128 + 1 - y, -mto + 4);
        c.maxx = MIN(W - 1 - x, mto - 4);     c.maxy = MIN(H - 1 - y, mto - 4);
    } else {
        c.minx = MAX(-x, -mto + 4);           c.miny = MAX(-y, -mto + 4);
        c.maxx = MIN(W - 1 - x - 16, mto - 4); c.maxy = MIN(H - 1 - y - 16, mto - 4);
    }
    int max_sr = cfg->max_search_range >> 1;

    u64 min_cost = ~(u64)0;
    for (int l = 0; l < 2; l++) {
        u64 min_dir = ~(u64)0;
        for (int r = 0; r < cfg->num_ref[l]; r++) {
            int dist = (int)(cfg->ptr - cfg->ref_ptr[l][r]);
            dist = ABSI(dist);
            int range = CLIP3(max_sr >> 2, max_sr, (max_sr * dist + (cfg->gop_size >> 1)) / cfg->gop_size);
            c.ref = refs[l][r] + y * i_ref + x;
            c.best = ~(u64)0;
            c.mvx = CLIP3(c.minx, c.maxx, 0); c.mvy = CLIP3(c.miny, c.maxy, 0);
            int bs = tz_diamond(&c, 32);
            if (c.mvx || c.mvy) {
                if (bs > 5) tz_raster(&c, r, range);
                tz_diamond(&c, 8);
            }
            u->mv[l][r][0] = (s16)c.mvx; u->mv[l][r][1] = (s16)c.mvy;
            /* com_mc_blk_luma at an integer MV inside [-MAX_CU_SIZE-4, max_coord]: a copy */
            const pel *blk = c.ref + c.mvy * i_ref + c.mvx;
            u32 cost = orc_had(16, 16, org, i_org, blk, i_ref, 8);
            u->satd[l][r] = cost;
            if (cost < min_dir) {
                min_dir = cost;
                if (cost < min_cost) min_cost = cost;
                if (is_bi) orc_ipcpy(blk, i_ref, best_pred[l], 16, 16, 16);
            }
        }
    }
    if (is_bi) {
        orc_pel_avrg(16, 16, pred, 16, best_pred[0], best_pred[1]);
        u->bi_satd = orc_had(16, 16, org, i_org, pred, 16, 8);
        if (u->bi_satd < min_cost) min_cost = u->bi_satd;
        const pel *z0 = refs[0][0] + y * i_ref + x, *z1 = refs[1][0] + y * i_ref + x;
        pel a[256], b[256];
        orc_ipcpy(z0, i_ref, a, 16, 16, 16);
        orc_ipcpy(z1, i_ref, b, 16, 16, 16);
        orc_pel_avrg(16, 16, pred, 16, a, b);
        u->zero_satd = orc_had(16, 16, org, i_org, pred, 16, 8);
        if (u->zero_satd < min_cost) min_cost = u->zero_satd;
    }

    /* intra: 11 modes predicted from the original picture's neighbours (:208-230) */
    pel nb[ORC_NEIB_SIZE];
    loka_nbr(nb, x, y, 16, 16, W, H, org, i_org);
    int avail = (x ? 2 : 0) | (y ? 1 : 0) | ((x && y) ? 4 : 0);
    u32 min_icost = 0xFFFFFFFFu;
    int best_mode = 0;
    for (int i = 0; i < 11; i++) {
        orc_intra_pred(nb, pred, IPM[i], 16, 16, 8, avail, 0);
        u32 cost = orc_had(16, 16, org, i_org, pred, 16, 8);
        if (cost < min_cost) min_cost = cost;
        if (cost < min_icost) { min_icost = cost; best_mode = IPM[i]; }
    }
    u->min_cost = (u32)min_cost;
    u->min_icost = min_icost;
    u->best_mode = (u8)best_mode;

    /* chroma with the best luma mode (:231-243) and the energy of the dQP map (:248-262) */
    int xc = x >> 1, yc = y >> 1;
    const pel *ou = org_u + yc * i_org_c + xc, *ov = org_v + yc * i_org_c + xc;
    loka_nbr(nb, xc, yc, 8, 8, W / 2, H / 2, ou, i_org_c);
    orc_intra_pred(nb, pred, best_mode, 8, 8, 8, avail, 0);
    u->icost_u = orc_had(8, 8, ou, i_org_c, pred, 8, 8);
    loka_nbr(nb, xc, yc, 8, 8, W / 2, H / 2, ov, i_org_c);
    orc_intra_pred(nb, pred, best_mode, 8, 8, 8, avail, 0);
    u->icost_v = orc_had(8, 8, ov, i_org_c, pred, 8, 8);
    u->energy = loka_var(org, i_org, 16) + loka_var(ou, i_org_c, 8) + loka_var(ov, i_org_c, 8);
}

/* lambda_mv of the estimation: base QP 32 (src/lookahead.c:85-106) */
static u32 loka_lambda(void)
{
    double base_lambda = 1.43631 * pow(2.0, (32 - 16.0) / 4.0);
    return (u32)floor(65536.0 * sqrt(base_lambda));
}

void orc_loka_units(const orc_loka_cfg_t *cfg, const pel *org_y, int i_org, const pel *org_u, const pel *org_v,
                    int i_org_c, const pel *const *ref_l0, const pel *const *ref_l1, int i_ref,
                    orc_loka_unit_t *units, int threads)
{
    int nux = cfg->width / 16, nuy = cfg->height / 16;
    int off = (MAX(cfg->width, cfg->height) << 2) + 3;
    u8 *tab = (u8 *)malloc((size_t)(2 * off + 1));
    orc_mvbits_table(tab, off);
    const pel *const *refs[2] = { ref_l0, ref_l1 };
    u32 lambda = loka_lambda();
#ifdef _OPENMP
    if (threads < 1) threads = 1;
    #pragma omp parallel for schedule(dynamic, 8) num_threads(threads)
#endif
    for (int i = 0; i < nux * nuy; i++)
        loka_unit(cfg, org_y, i_org, org_u, org_v, i_org_c, refs, i_ref, tab + off, lambda, i % nux, i / nux,
                  &units[i]);
    (void)threads;
    free(tab);
}

/* src/lookahead.c:201-292: totals accumulated in double in raster order, averages per sample,
 * the dQP map as 0.8 log2(energy) minus its mean */
double orc_loka_finish(const orc_loka_cfg_t *cfg, const orc_loka_unit_t *units, double *icost, double *icost_uv,
                       float *map_dqp)
{
    int n = (cfg->width / 16) * (cfg->height / 16);
    double tc = 0, ti = 0, tu = 0, tv = 0, tvar = 0;
    for (int i = 0; i < n; i++) {
        tc += units[i].min_cost;
        ti += units[i].min_icost;
        tu += units[i].icost_u;
        tv += units[i].icost_v;
        if (map_dqp) {
            u64 e = units[i].energy;
            map_dqp[i] = (float)(0.8 * log2((double)MAX(e, 1)));
            tvar += map_dqp[i];
        }
    }
    if (icost) *icost = ti / n / 16 / 16;
    if (icost_uv) { icost_uv[0] = tu / n / 8 / 8; icost_uv[1] = tv / n / 8 / 8; }
    if (map_dqp) {
        float avg = (float)(tvar / n);
        for (int i = 0; i < n; i++) map_dqp[i] -= avg;
    }
    return tc / n / 16 / 16;
}

/* ======================================================= per-call TZ motion search */

/* tbl_refi_bits (src/tables.c:52): truncated unary code of refi among num_refp references */
static int refi_bits(int num_refp, int refi)
{
    return num_refp <= 1 ? 0 : MIN(refi + 1, num_refp - 1);
}

/* the state of one me_search_tz call (inter_search_t fields it reads, src/me.c:529) */
typedef struct {
    const pel *org; int i_org;          /* block origin of org (or of 2 org - pred for bi)  */
    const pel *ref; int i_ref;          /* integer plane at the block origin                */
    const pel *const *planes;           /* the reference's 16 planes                        */
    int x, y, w, h;
    int minx, maxx, miny, maxy;         /* integer-sample MV range                          */
    int mvr;
    u32 lambda;
    const u8 *bx, *by;                  /* MV-bits tables offset by the predictor           */
    int shift;                          /* 16 - bi                                          */
    u64 best; int mvx, mvy;
} tzg_t;

static u64 tzg_cost(const tzg_t *c, int mx, int my)
{
    u32 sad = orc_sad(c->w, c->h, c->org, c->i_org, c->ref + my * c->i_ref + mx, c->i_ref);
    u32 bits = (u32)(c->bx[(mx * 4) >> c->mvr] + c->by[(my * 4) >> c->mvr]);
    return ((u64)sad << c->shift) + (u64)(bits * c->lambda);
}

static int tzg_try(tzg_t *c, int mx, int my)
{
    u64 cost = tzg_cost(c, mx, my);
    if (cost < c->best) { c->best = cost; c->mvx = mx; c->mvy = my; return 1; }
    return 0;
}

/* search_diamond (src/me.c:199-334) for any MV resolution, bi or not */
static int tzg_diamond(tzg_t *c, int max_step, int bi, const s16 *mvp)
{
    static const s8 RING_A[8][2] = { { -2, 0 }, { -1, 1 }, { 0, 2 }, { 1, 1 },
                                     { 2, 0 }, { 1, -1 }, { 0, -2 }, { -1, -1 } };
    static const s8 RING_B[16][2] = { { -4, 0 }, { -3, 1 }, { -2, 2 }, { -1, 3 }, { 0, 4 }, { 1, 3 },
                                      { 2, 2 }, { 3, 1 }, { 4, 0 }, { 3, -1 }, { 2, -2 }, { 1, -3 },
                                      { 0, -4 }, { -1, -3 }, { -2, -2 }, { -3, -1 } };
    const int cx = c->mvx, cy = c->mvy;
    int core = bi ? 5 : 2, cstep = 1, best_step = 0;
    if (bi) {
        if (c->mvr > 2) core++;
        int ix = (mvp[0] + 2) >> 2, iy = (mvp[1] + 2) >> 2;
        int diff = MAX(ABSI(ix - cx), ABSI(iy - cy)) >> MAX(0, c->mvr - 2);
        core = CLIP3(2, core, diff);
    }
    if (c->mvr > 2) { core <<= c->mvr - 2; cstep <<= c->mvr - 2; }
    int x0 = cx - core, y0 = cy - core, x1 = cx + core, y1 = cy + core;
    while (x0 <= c->minx) x0 += cstep;
    while (y0 <= c->miny) y0 += cstep;
    while (x1 >= c->maxx) x1 -= cstep;
    while (y1 >= c->maxy) y1 -= cstep;
    tzg_try(c, cx, cy);
    if (max_step)
        for (int my = y0; my <= y1; my += cstep)
            for (int mx = x0; mx <= x1; mx += cstep) tzg_try(c, mx, my);
    if (c->mvx != cx || c->mvy != cy) best_step = 2;
    if (bi) return best_step;
    int mvr_scale = MAX(c->mvr - 2, 0);
    for (int step = 4, round = 0; step < max_step; step <<= 1, round++) {
        int scale = (step << mvr_scale) >> 1;
        const s8(*ring)[2] = round < 2 ? RING_A : RING_B;
        int n = round < 2 ? 8 : 16, inc = round < 1 ? 2 : 1, sh = round < 2 ? 0 : 1;
        for (int i = 0; i < n; i += inc) {
            int mx = cx + (scale >> sh) * ring[i][0], my = cy + (scale >> sh) * ring[i][1];
            if (mx <= c->maxx && mx >= c->minx && my <= c->maxy && my >= c->miny && tzg_try(c, mx, my))
                best_step = step;
        }
    }
    return best_step;
}

/* search_raster with get_raster_range (src/me.c:65-197) for any MV resolution */
static void tzg_raster(tzg_t *c, const orc_tz_req_t *rq, const orc_tz_pic_t *pic)
{
    static const int BASE[5] = { 5, 5, 5, 6, 8 }, SMIN[5] = { 1, 1, 1, 2, 4 };
    const int mvr = c->mvr;
    int step = MAX(BASE[mvr], MIN(c->w >> 1, c->h >> 1)) * (rq->refi + 1);
    int max_sr = pic->max_search_range >> MAX(3 - mvr, 0);
    int rxy = CLIP3(max_sr >> 2, max_sr, (max_sr * rq->dist + (pic->gop_size >> 1)) / pic->gop_size);
    int rx = rxy, ry = rxy;
    if (mvr && (rq->flags & 2)) {
        rx = ABSI(rq->mv_ipel[0] - c->mvx) * 4;
        ry = ABSI(rq->mv_ipel[1] - c->mvy) * 2;
        rx = MIN(MAX(MAX(rx, max_sr >> 2), step * 8), rxy);
        ry = MIN(MAX(MAX(ry, max_sr >> 2), step * 4), rxy);
    }
    if (mvr > 2) { rx = (rx >> (mvr - 2)) << (mvr - 2); ry = (ry >> (mvr - 2)) << (mvr - 2); }
    int x0 = CLIP3(c->minx, c->maxx, c->mvx - rx), x1 = CLIP3(c->minx, c->maxx, c->mvx + rx);
    int y0 = CLIP3(c->miny, c->maxy, c->mvy - ry), y1 = CLIP3(c->miny, c->maxy, c->mvy + ry);
    for (int round = 0; step >= SMIN[mvr]; round++) {
        if (round) {
            x0 = MAX(c->mvx - step, c->minx); x1 = MIN(c->mvx + step, c->maxx);
            y0 = MAX(c->mvy - step, c->miny); y1 = MIN(c->mvy + step, c->maxy);
        }
        for (int my = y0; my <= y1; my += step)
            for (int mx = x0; mx <= x1; mx += step) tzg_try(c, mx, my);
        step >>= 1;
        if (mvr > 2) step = (step >> (mvr - 2)) << (mvr - 2);
    }
}

/* me_sub_pel_search (src/me.c:366-500): centre, 8 half-sample points, then (quarter-sample
 * resolution) 8 quarter-sample points; SATD cost, or SAD with the SATD recomputed at the end */
static u64 tzg_subpel(tzg_t *c, int *qx, int *qy, int bi, int cost_type, int W, int H)
{
    static const s8 HP[8][2] = { { -2, 0 }, { -2, 2 }, { 0, 2 }, { 2, 2 }, { 2, 0 }, { 2, -2 }, { 0, -2 }, { -2, -2 } };
    static const s8 QP[8][2] = { { -1, 0 }, { 0, 1 }, { 1, 0 }, { 0, -1 }, { -1, 1 }, { 1, 1 }, { -1, -1 }, { 1, -1 } };
    const int maxx = W + 4, maxy = H + 4, shift = 16 - bi, mvr = c->mvr;
    int cx = *qx, cy = *qy;
    const pel *p0 = c->ref + (cx >> 2) + (cy >> 2) * c->i_ref;
    u32 d = cost_type ? orc_sad(c->w, c->h, c->org, c->i_org, p0, c->i_ref)
                      : orc_had(c->w, c->h, c->org, c->i_org, p0, c->i_ref, 8);
    u64 best = (u64)(c->lambda * (u32)(c->bx[cx >> mvr] + c->by[cy >> mvr])) + ((u64)d << shift);
    for (int pass = 0; pass < (mvr == 0 ? 2 : 1); pass++) {
        const s8(*pat)[2] = pass ? QP : HP;
        cx = *qx; cy = *qy;
        for (int i = 0; i < 8; i++) {
            int vx = cx + pat[i][0], vy = cy + pat[i][1];
            const pel *p = mc_pointer(c->planes, c->i_ref, vx + (c->x << 2), vy + (c->y << 2), maxx, maxy);
            d = cost_type ? orc_sad(c->w, c->h, c->org, c->i_org, p, c->i_ref)
                          : orc_had(c->w, c->h, c->org, c->i_org, p, c->i_ref, 8);
            u64 cost = (u64)(c->lambda * (u32)(c->bx[vx >> mvr] + c->by[vy >> mvr])) + ((u64)d << shift);
            if (cost < best) { best = cost; *qx = vx; *qy = vy; }
        }
    }
    if (cost_type) {
        const pel *p = mc_pointer(c->planes, c->i_ref, *qx + (c->x << 2), *qy + (c->y << 2), maxx, maxy);
        d = orc_had(c->w, c->h, c->org, c->i_org, p, c->i_ref, 8);
        best = (u64)(c->lambda * (u32)(c->bx[*qx >> mvr] + c->by[*qy >> mvr])) + ((u64)d << (16 - bi));
    }
    return best;
}

static void tz_one(const orc_tz_pic_t *pic, const pel *org, int i_org, const pel *const *planes, int i_ref,
                   const u8 *bits, int mto, const orc_tz_req_t *rq, orc_tz_out_t *o)
{
    const int x = rq->x, y = rq->y, w = rq->w, h = rq->h, mvr = rq->mvr, bi = rq->bi;
    const int W = pic->width, H = pic->height;
    tzg_t c;
    pel org_bi[64 * 64];
    o->mv[0] = rq->mv[0]; o->mv[1] = rq->mv[1];
    o->mv_ipel[0] = rq->mv_ipel[0]; o->mv_ipel[1] = rq->mv_ipel[1];
    /* get_max_search_range (src/me.c:502-527) */
    int mt = (mto << mvr) >> 2, px = rq->mvp[0] >> 2, py = rq->mvp[1] >> 2;
    if (pic->is_padding) {
        c.minx = MAX(-128 + 1 - x, px - mt + 4); c.miny = MAX(-128 + 1 - y, py - mt + 4);
        c.maxx = MIN(W - 1 - x, px + mt - 4);     c.maxy = MIN(H - 1 - y, py + mt - 4);
    } else {
        c.minx = MAX(-x, px - mt + 4);             c.miny = MAX(-y, py - mt + 4);
        c.maxx = MIN(W - 1 - x - w, px + mt - 4);  c.maxy = MIN(H - 1 - y - h, py + mt - 4);
    }
    if (mvr > 2) {   /* com_ipel_range_rounding: towards zero to a multiple of 1 << (mvr - 2) */
        int s = mvr - 2;
        int *v[4] = { &c.minx, &c.miny, &c.maxx, &c.maxy };
        for (int i = 0; i < 4; i++) *v[i] = *v[i] >= 0 ? ((*v[i] >> s) << s) : -(((-*v[i]) >> s) << s);
    }
    if (c.minx > c.maxx || c.miny > c.maxy) { o->cost = ~(u64)0; return; }
    const pel *const *pl = planes + rq->ref_slot * 16;
    c.planes = pl; c.i_ref = i_ref; c.ref = pl[0] + y * i_ref + x;
    c.x = x; c.y = y; c.w = w; c.h = h; c.mvr = mvr; c.lambda = rq->lambda_mv; c.shift = 16 - bi;
    c.bx = bits - (rq->mvp[0] >> mvr); c.by = bits - (rq->mvp[1] >> mvr);
    if (bi) {
        /* create_bi_org (src/inter.c:55) against com_mc_cu's prediction of the other list */
        const pel *pr = mc_pointer(planes + rq->other_slot * 16, i_ref, (x << 2) + rq->other_mv[0],
                                   (y << 2) + rq->other_mv[1], W + 4, H + 4);
        const pel *og = org + y * i_org + x;
        for (int j = 0; j < h; j++)
            for (int i = 0; i < w; i++) org_bi[j * w + i] = (pel)CLIP3(0, 255, 2 * og[j * i_org + i] - pr[j * i_ref + i]);
        c.org = org_bi; c.i_org = w;
    } else {
        c.org = org + y * i_org + x; c.i_org = i_org;
    }
    int mvx = bi ? rq->mv[0] : rq->mvp[0], mvy = bi ? rq->mv[1] : rq->mvp[1];
    c.mvx = CLIP3(c.minx, c.maxx, (mvx + 2) >> 2);
    c.mvy = CLIP3(c.miny, c.maxy, (mvy + 2) >> 2);
    c.best = ~(u64)0;
    int bs = tzg_diamond(&c, 32, bi, rq->mvp);
    if (!bi && (ABSI(rq->mvp[0] - (c.mvx << 2)) > 2 || ABSI(rq->mvp[1] - (c.mvy << 2)) > 2)) {
        if (bs > 5) tzg_raster(&c, rq, pic);
        tzg_diamond(&c, 8, bi, rq->mvp);
    }
    if (!bi) { o->mv_ipel[0] = (s16)c.mvx; o->mv_ipel[1] = (s16)c.mvy; }
    int qx = c.mvx << 2, qy = c.mvy << 2;
    u64 cost = c.best;
    if (mvr < 2) cost = tzg_subpel(&c, &qx, &qy, bi, rq->flags & 1, W, H);
    int extra = refi_bits(rq->num_refp, rq->refi) + mvr + (mvr < 4) + (bi ? rq->mot_bits_other + 1 : 2);
    cost += (u64)(rq->lambda_mv * (u32)extra);
    o->mv[0] = (s16)qx; o->mv[1] = (s16)qy;
    o->cost = (u32)((cost + (1 << 15)) >> 16);
}

void orc_me_tz(const orc_tz_pic_t *pic, const pel *org, int i_org, const pel *const *planes, int i_ref,
               const orc_tz_req_t *reqs, int n, orc_tz_out_t *out, int threads)
{
    int off = (MAX(pic->width, pic->height) << 2) + 3;
    u8 *tab = (u8 *)malloc((size_t)(2 * off + 1));
    orc_mvbits_table(tab, off);
#ifdef _OPENMP
    if (threads < 1) threads = 1;
    #pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
#endif
    for (int i = 0; i < n; i++) tz_one(pic, org, i_org, planes, i_ref, tab + off, off, &reqs[i], &out[i]);
    (void)threads;
    free(tab);
}

/* ============================================================ CU motion compensation */

/* com_mc_blk_chroma with hp_flag 0 (src/com_mc.c:103-138): 1/8-sample position, clipped to
 * [-(MAX_CU_SIZE/2) - 2, max_pos], copy or 4-tap filters (ipflt H_4 / V_4, ipflt_ext EXT_4) */
static void mc_chroma_blk(const pel *plane, int i_c, pel *dst, int qx, int qy, int w, int h, int maxx, int maxy)
{
    const s8(*coef)[4] = (const s8(*)[4])orc_mc_chroma_coef();
    int dx = qx & 7, dy = qy & 7;
    int x = CLIP3(-64 - 2, maxx, qx >> 3), y = CLIP3(-64 - 2, maxy, qy >> 3);
    const pel *src = plane + y * i_c + x;
    if (!dx && !dy) orc_ipcpy(src, i_c, dst, w, w, h);
    else if (!dy) orc_ipflt(1, src, i_c, dst, w, w, h, coef[dx], 255);
    else if (!dx) orc_ipflt(3, src, i_c, dst, w, w, h, coef[dy], 255);
    else orc_ipflt_ext(1, src, i_c, dst, w, w, h, coef[dx], coef[dy], 255);
}

/* com_mc_cu (src/com_mc.c:140-200): each used list's prediction, the two averaged (pel_avrg);
 * identical motion on the same picture keeps the first, which the average equals */
void orc_mc_cu(int width, int height, const pel *const *planes, int i_ref, const pel *const *chroma, int i_c,
               const orc_mc_req_t *reqs, int n, pel *out)
{
    for (int i = 0; i < n; i++) {
        const orc_mc_req_t *r = &reqs[i];
        const int w = r->w, h = r->h, wc = w >> 1, hc = h >> 1;
        pel pred[2][3][64 * 64];
        int np = 0;
        for (int l = 0; l < 2; l++) {
            if (r->slot[l] < 0) continue;
            int qx = (r->x << 2) + r->mv[l][0], qy = (r->y << 2) + r->mv[l][1];
            if (r->channel != 2) {
                const pel *p = mc_pointer(planes + r->slot[l] * 16, i_ref, qx, qy, width + 4, height + 4);
                orc_ipcpy(p, i_ref, pred[np][0], w, w, h);
            }
            if (r->channel != 1)
                for (int c = 0; c < 2; c++)
                    mc_chroma_blk(chroma[r->slot[l] * 2 + c], i_c, pred[np][1 + c], qx, qy, wc, hc, (width + 4) >> 1,
                                  (height + 4) >> 1);
            np++;
        }
        pel *o = out + r->out_offset;
        if (r->channel != 2) {
            if (np == 2) orc_pel_avrg(w, h, o, w, pred[0][0], pred[1][0]);
            else memcpy(o, pred[0][0], (size_t)w * h);
            o += w * h;
        }
        if (r->channel != 1)
            for (int c = 0; c < 2; c++, o += wc * hc) {
                if (np == 2) orc_pel_avrg(wc, hc, o, wc, pred[0][1 + c], pred[1][1 + c]);
                else memcpy(o, pred[0][1 + c], (size_t)wc * hc);
            }
    }
}

/* ============================================================ affine motion compensation */

/* 1/16-sample luma and 1/32-sample chroma filters of affine prediction (com_tbl_mc_l_coeff_hp,
 * com_tbl_mc_c_coeff_hp, src/com_tables.c:130-189) */
static const s8 MC_L_HP[16][8] = {
    { 0, 0, 0, 64, 0, 0, 0, 0 },      { 0, 1, -3, 63, 4, -2, 1, 0 },     { -1, 2, -5, 62, 8, -3, 1, 0 },
    { -1, 3, -8, 60, 13, -4, 1, 0 },   { -1, 4, -10, 58, 17, -5, 1, 0 },  { -1, 4, -11, 52, 26, -8, 3, -1 },
    { -1, 3, -9, 47, 31, -10, 4, -1 }, { -1, 4, -11, 45, 34, -10, 4, -1 }, { -1, 4, -11, 40, 40, -11, 4, -1 },
    { -1, 4, -10, 34, 45, -11, 4, -1 }, { -1, 4, -10, 31, 47, -9, 3, -1 }, { -1, 3, -8, 26, 52, -11, 4, -1 },
    { 0, 1, -5, 17, 58, -10, 4, -1 },  { 0, 1, -4, 13, 60, -8, 3, -1 },   { 0, 1, -3, 8, 62, -5, 2, -1 },
    { 0, 1, -2, 4, 63, -3, 1, 0 },
};
static const s8 MC_C_HP[32][4] = {
    { 0, 64, 0, 0 },    { -1, 63, 2, 0 },   { -2, 62, 4, 0 },   { -2, 60, 7, -1 },  { -2, 58, 10, -2 },
    { -3, 57, 12, -2 }, { -4, 56, 14, -2 }, { -4, 55, 15, -2 }, { -4, 54, 16, -2 }, { -5, 53, 18, -2 },
    { -6, 52, 20, -2 }, { -6, 49, 24, -3 }, { -6, 46, 28, -4 }, { -5, 44, 29, -4 }, { -4, 42, 30, -4 },
    { -4, 39, 33, -4 }, { -4, 36, 36, -4 }, { -4, 33, 39, -4 }, { -4, 30, 42, -4 }, { -4, 29, 44, -5 },
    { -4, 28, 46, -6 }, { -3, 24, 49, -6 }, { -2, 20, 52, -6 }, { -2, 18, 53, -5 }, { -2, 16, 54, -4 },
    { -2, 15, 55, -4 }, { -2, 14, 56, -4 }, { -2, 12, 57, -3 }, { -2, 10, 58, -2 }, { -1, 7, 60, -2 },
    { 0, 4, 62, -2 },   { 0, 2, 63, -1 },
};

/* com_mv_rounding_s32 (inc/com_util.h:189) with right shift 7, left shift 0: magnitude rounded */
static s32 affine_round7(s32 v) { return v >= 0 ? (v + 64) >> 7 : -((-v + 64) >> 7); }

/* com_mc_blk_luma with hp_flag 1 (src/com_mc.c:41-87): its plane shortcut never applies (its
 * vertical test needs dy == 0 and dy == 8 at once), so every block is filtered from the integer
 * plane with the 16-phase filters */
static void affine_luma_blk(const pel *plane, int i_ref, pel *dst, int id, int qx, int qy, int w, int h, int maxx,
                            int maxy)
{
    int dx = qx & 15, dy = qy & 15;
    int x = CLIP3(-128 - 4, maxx, qx >> 4), y = CLIP3(-128 - 4, maxy, qy >> 4);
    const pel *src = plane + y * i_ref + x;
    if (!dx && !dy) orc_ipcpy(src, i_ref, dst, id, w, h);
    else if (!dy) orc_ipflt(0, src, i_ref, dst, id, w, h, MC_L_HP[dx], 255);
    else if (!dx) orc_ipflt(2, src, i_ref, dst, id, w, h, MC_L_HP[dy], 255);
    else orc_ipflt_ext(0, src, i_ref, dst, id, w, h, MC_L_HP[dx], MC_L_HP[dy], 255);
}

/* com_mc_blk_chroma with hp_flag 1 (src/com_mc.c:103-138): 1/32-sample positions */
static void affine_chroma_blk(const pel *plane, int i_c, pel *dst, int id, int qx, int qy, int w, int h, int maxx,
                              int maxy)
{
    int dx = qx & 31, dy = qy & 31;
    int x = CLIP3(-64 - 2, maxx, qx >> 5), y = CLIP3(-64 - 2, maxy, qy >> 5);
    const pel *src = plane + y * i_c + x;
    if (!dx && !dy) orc_ipcpy(src, i_c, dst, id, w, h);
    else if (!dy) orc_ipflt(1, src, i_c, dst, id, w, h, MC_C_HP[dx], 255);
    else if (!dx) orc_ipflt(3, src, i_c, dst, id, w, h, MC_C_HP[dy], 255);
    else orc_ipflt_ext(1, src, i_c, dst, id, w, h, MC_C_HP[dx], MC_C_HP[dy], 255);
}

/* com_mc_blk_affine (src/com_mc.c:256-359): sub-block MVs from the control points at the
 * sub-block centres (corner sub-blocks at the control points), rounded to 1/16 and clipped to
 * 18 bits; chroma 4x4 blocks take the rounded mean of their four 4x4 luma MVs */
static void affine_blk(int W, int H, int x, int y, int cw, int ch, const s32 (*ac)[2], int cp_num, int sub,
                       const pel *plane, int i_ref, const pel *pu, const pel *pv, int i_c, pel *py, pel *ou, pel *ov)
{
    static s32 mvs[16][16][2];
    const int lw = ilog2(cw), lh = ilog2(ch), half = sub >> 1;
    const s32 dhx = ((ac[1][0] - ac[0][0]) * 128) >> lw, dhy = ((ac[1][1] - ac[0][1]) * 128) >> lw;
    s32 dvx = -dhy, dvy = dhx;
    if (cp_num == 3) { dvx = ((ac[2][0] - ac[0][0]) * 128) >> lh; dvy = ((ac[2][1] - ac[0][1]) * 128) >> lh; }
    for (int h = 0; h < ch; h += sub)
        for (int w = 0; w < cw; w += sub) {
            int px = w + half, pyy = h + half;
            if (w == 0 && h == 0) { px = 0; pyy = 0; }
            else if (w + sub == cw && h == 0) { px = cw; pyy = 0; }
            else if (w == 0 && h + sub == ch && cp_num == 3) { px = 0; pyy = ch; }
            s32 mx = ac[0][0] * 128 + dhx * px + dvx * pyy, my = ac[0][1] * 128 + dhy * px + dvy * pyy;
            mx = CLIP3(-131072, 131071, affine_round7(mx));
            my = CLIP3(-131072, 131071, affine_round7(my));
            for (int j = 0; j < sub / 4; j++)
                for (int i = 0; i < sub / 4; i++) { mvs[(w >> 2) + i][(h >> 2) + j][0] = mx; mvs[(w >> 2) + i][(h >> 2) + j][1] = my; }
            affine_luma_blk(plane, i_ref, py + h * cw + w, cw, ((x + w) << 4) + mx, ((y + h) << 4) + my, sub, sub,
                            W + 4, H + 4);
        }
    for (int h = 0; h < ch; h += 8)
        for (int w = 0; w < cw; w += 8) {
            int ws = w >> 2, hs = h >> 2;
            s32 mx = (mvs[ws][hs][0] + mvs[ws + 1][hs][0] + mvs[ws][hs + 1][0] + mvs[ws + 1][hs + 1][0] + 2) >> 2;
            s32 my = (mvs[ws][hs][1] + mvs[ws + 1][hs][1] + mvs[ws][hs + 1][1] + mvs[ws + 1][hs + 1][1] + 2) >> 2;
            int qx = ((x + w) << 4) + mx, qy = ((y + h) << 4) + my;
            affine_chroma_blk(pu, i_c, ou + (h >> 1) * (cw >> 1) + (w >> 1), cw >> 1, qx, qy, 4, 4, (W + 4) >> 1,
                              (H + 4) >> 1);
            affine_chroma_blk(pv, i_c, ov + (h >> 1) * (cw >> 1) + (w >> 1), cw >> 1, qx, qy, 4, 4, (W + 4) >> 1,
                              (H + 4) >> 1);
        }
}

/* com_mc_cu_affine (src/com_mc.c:361-422): 4x4 sub-blocks, 8x8 with affine_subblk_size_idx 1 or
 * with both lists; the two lists averaged */
void orc_mc_affine(int width, int height, const pel *const *planes, int i_ref, const pel *const *chroma, int i_c,
                   const orc_affine_req_t *reqs, int n, pel *out)
{
    static pel pr[2][3][64 * 64];
    for (int i = 0; i < n; i++) {
        const orc_affine_req_t *r = &reqs[i];
        const int w = r->w, h = r->h, bi = r->slot[0] >= 0 && r->slot[1] >= 0;
        const int sub = (r->sub8 == 1 || bi) ? 8 : 4;
        int np = 0;
        for (int l = 0; l < 2; l++) {
            if (r->slot[l] < 0) continue;
            int s = r->slot[l];
            affine_blk(width, height, r->x, r->y, w, h, r->cpmv[l], r->cp_num, sub, planes[s * 16], i_ref,
                       chroma[s * 2], chroma[s * 2 + 1], i_c, pr[np][0], pr[np][1], pr[np][2]);
            np++;
        }
        pel *o = out + r->out_offset;
        const int sizes[3] = { w * h, w * h / 4, w * h / 4 };
        for (int c = 0; c < 3; c++, o += sizes[c - 1]) {
            for (int k = 0; k < sizes[c]; k++)
                o[k] = np == 2 ? (pel)((pr[0][c][k] + pr[1][c][k] + 1) >> 1) : pr[0][c][k];
        }
    }
}

/* ============================================================ coefficient rate */

/* The context-model update the reference tabulates in tbl_plps / tbl_plps_ext (src/entropy.c:41,
 * 16,384 entries): a model is (window state c in bits 11-12) | (LPS probability p, 10 bits, in
 * bits 1-10) | MPS.  The window is 3, 3, 4, 5 for states 0..3.  After an MPS p loses
 * p >> w + p >> (w + 2) and state 0 becomes 1; after an LPS p gains 197, 95 or 46 (w = 3, 4, 5),
 * reflected about 1023 with the MPS flipped when it passes it, and the state steps up to 3.
 * (The rule reproduces all 16,384 entries of the reference's table.) */
int orc_lbac_next(int model, int mps)
{
    const int c = (model >> 11) & 3, w = c < 2 ? 3 : c + 2;
    int p = (model >> 1) & 1023, m = model & 1;
    if (mps) {
        p -= (p >> w) + (p >> (w + 2));
        return ((c == 0 ? 1 : c) << 11) | (p << 1) | m;
    }
    p += w == 3 ? 197 : (w == 4 ? 95 : 46);
    if (p > 1023) { p = 2047 - p; m ^= 1; }
    return (MIN(c + 1, 3) << 11) | (p << 1) | m;
}

/* counting-mode coding of one bin with model *mdl: range, bits, model updated */
static void crate_bin(u32 *range, u32 *bits, s16 *mdl, int bin)
{
    const u32 lps = (u32)(*mdl & 2047) >> 3;
    u32 mps = *range - lps;
    const int s = mps < 256;
    mps |= 0x100;
    if (bin == (*mdl & 1)) {
        *bits += s;
        *range = mps;
        *mdl = (s16)orc_lbac_next(*mdl, 1);
    } else {
        const u32 l = (*range << s) - mps;
        const int sh = 8 - ilog2((int)l);
        *range = l << sh;
        *bits += sh + s;
        *mdl = (s16)orc_lbac_next(*mdl, 0);
    }
}

/* a truncated unary symbol of the run / level coding: the first bin on m[0] ('1' for 0), the
 * rest on m[1] ('0' per unit, the closing '1' omitted at the cap), as the reference's
 * counting-mode run and level coders do (src/entropy.c:1715-1782, :1800-1866) */
static void crate_unary(u32 *range, u32 *bits, s16 *m, int sym, int cap)
{
    crate_bin(range, bits, &m[0], sym == 0);
    if (sym == 0) return;
    for (int k = 1; k <= sym && k < cap; k++) crate_bin(range, bits, &m[1], k == sym);
}

/* bits of the exp-Golomb escape of value v (order 0 code of v, with the reference's loop) */
static u32 crate_egk(int v)
{
    int order = 1;
    for (int s = v; s >= 0; order++) s -= 1 << order;
    return (u32)((order << 1) - 1);
}

/* lbac_enc_run_length_cc_rdo (src/entropy.c:1688-1950): for each non-zero level in scan order,
 * its run of zeros (truncated unary capped at 16 + escape; the run_rdoq models follow the same
 * run without the cap), its level - 1 (capped at 8 + escape), the sign, and the last flag on the
 * averaged pair (last1 by the previous level, last2 by log2 of the scan position) */
static void crate_one(const s16 *coef, const orc_coef_rate_req_t *r, orc_coef_rate_out_t *o)
{
    o->ctx = r->ctx;
    orc_coef_ctx_t *c = &o->ctx;
    const u16 *scan = orc_scan(r->log2w, r->log2h);
    const int n = 1 << (r->log2w + r->log2h);
    u32 range = r->range, bits = 0;
    int t0 = 10, num_sig = r->num_sig, last = -1, pos = 0;
    do {
        while (!coef[scan[pos]]) pos++;
        const int run = pos - last - 1;
        last = pos;
        crate_unary(&range, &bits, &c->run[t0], MIN(run, 16), 16);
        if (run >= 16) bits += crate_egk(run - 17);
        /* run_rdoq: the uncapped unary run's model updates, no bits */
        c->run_rdoq[t0] = (s16)orc_lbac_next(c->run_rdoq[t0], (run == 0) == (c->run_rdoq[t0] & 1));
        for (int k = 1; k <= run; k++)
            c->run_rdoq[t0 + 1] = (s16)orc_lbac_next(c->run_rdoq[t0 + 1], (k == run) == (c->run_rdoq[t0 + 1] & 1));
        const int level = ABSI(coef[scan[pos]]);
        crate_unary(&range, &bits, &c->level[t0], MIN(level - 1, 8), 8);
        if (level >= 9) bits += crate_egk(level - 10);
        bits++;                                                   /* sign */
        if (pos == n - 1) break;
        num_sig--;
        /* last flag on the pair (lbac_encode_binW): the common MPS, or the likelier one */
        s16 *m1 = &c->last1[t0 >> 1], *m2 = &c->last2[ilog2(pos + 1)];
        t0 = MIN(level - 1, 5) << 1;
        const int p1 = (*m1 & 2047) >> 1, p2 = (*m2 & 2047) >> 1, c1 = *m1 & 1, c2 = *m2 & 1;
        int cm, pl;
        if (c1 == c2) { cm = c1; pl = (p1 + p2) >> 1; }
        else if (p1 < p2) { cm = c1; pl = (256 << 2) - 1 - ((p2 - p1) >> 1); }
        else { cm = c2; pl = (256 << 2) - 1 - ((p1 - p2) >> 1); }
        const int flag = num_sig == 0;
        u32 mps = range - ((u32)pl >> 2);
        const int s = mps < 256;
        mps |= 0x100;
        if (flag == cm) { bits += s; range = mps; }
        else {
            const u32 l = (range << s) - mps;
            const int sh = 8 - ilog2((int)l);
            range = l << sh;
            bits += sh + s;
        }
        *m1 = (s16)orc_lbac_next(*m1, flag == c1);
        *m2 = (s16)orc_lbac_next(*m2, flag == c2);
        pos++;
    } while (num_sig);
    o->bits = bits;
    o->range = (u16)range;
    o->pad = 0;
}

void orc_coef_rate(const s16 *levels, const orc_coef_rate_req_t *reqs, int n, orc_coef_rate_out_t *out)
{
    orc_init();
    for (int i = 0; i < n; i++) crate_one(levels + reqs[i].coef_offset, &reqs[i], &out[i]);
}

/* ============================================================ intra mode candidates */

/* one bin of lbac_encode_bin in counting mode (src/entropy.c:1168-1187): the range after it and
 * the bits it adds.  Each intra_dir context model is used once per syntax element, so its
 * update does not change the count. */
static void rmd_bin(u32 *range, int *bits, int bin, int model)
{
    const u32 lps = (u32)(model & 2047) >> 3;
    u32 mps = *range - lps;
    const int s = mps < 256;
    mps |= 0x100;
    if (bin == (model & 1)) {
        *bits += s;
        *range = mps;
    } else {
        const u32 l = (*range << s) - mps;          /* 1..510 */
        const int sh = 8 - ilog2((int)l);            /* get_shift */
        *range = l << sh;
        *bits += sh + s;
    }
}

/* lbac_enc_intra_dir (src/entropy.c:2118-2130): an MPM as flag 1 + its index, any other mode as
 * flag 0 + its 5-bit rank among the non-MPM modes (msb first, contexts 1..5) */
int orc_intra_dir_bits(int range, const s16 *ctx, int ipm, const u8 *mpm)
{
    const int code = ipm == mpm[0] ? -2 : (ipm == mpm[1] ? -1 : (ipm < mpm[0] ? ipm : (ipm < mpm[1] ? ipm - 1 : ipm - 2)));
    u32 r = (u32)range;
    int bits = 0;
    if (code < 0) {
        rmd_bin(&r, &bits, 1, ctx[0]);
        rmd_bin(&r, &bits, code + 2, ctx[6]);
    } else {
        rmd_bin(&r, &bits, 0, ctx[0]);
        for (int i = 4; i >= 0; i--) rmd_bin(&r, &bits, (code >> i) & 1, ctx[1 + (4 - i)]);
    }
    return bits;
}

/* com_update_cand_list (src/intra.c:187-207): the mode's cost is recorded, and the mode enters
 * the first len entries of the cost-ordered list before the first entry it does not beat
 * strictly (empty entries count as beaten), the entries below it moving down one */
static void rmd_update(int ipm, double cost, int len, int *list, double *cost_of)
{
    cost_of[ipm] = cost;
    int shift = 0, p = len - 1;
    while (shift < len && (list[p] < 0 || cost < cost_of[list[p]])) { p--; shift++; }
    if (shift) {
        int q = len - 1;
        for (shift--; shift; shift--, q--) list[q] = list[q - 1];
        list[q] = ipm;
    }
}

typedef struct {
    const u32 *satd;
    const orc_rmd_req_t *r;
    int *list;
    double *cost_of;
} rmd_ctx_t;

/* check_one_mode (src/intra.c:209-224) with the mode's SATD given: cost = SATD + bits x
 * sqrt_lambda in double, then the list update */
static void rmd_check(const rmd_ctx_t *c, int ipm, int len)
{
    const int bits = orc_intra_dir_bits(c->r->range, c->r->ctx, ipm, c->r->mpm);
    const double cost = (double)c->satd[ipm] + (double)bits * c->r->sqrt_lambda;
    rmd_update(ipm, cost, len, c->list, c->cost_of);
}

/* make_ipred_list (src/intra.c:226-367): with intra_fast_rmd the 10 coarse modes, then +-2 of the
 * best 7, +-1 of the first 3 angular entries, and the MPMs not yet tried; otherwise every mode.
 * Then the MPMs the list lacks replace its last entries, and entries costlier than the inter
 * SATD x threshold are cut from the end.  Reproduces the reference's stale entries: the list
 * keeps 10 positions from the coarse stage while later stages insert into 4 or 5. */
static int rmd_one(const u32 *satd, const orc_rmd_req_t *r, int *list)
{
    const int w = r->pb_w, h = r->pb_h;
    int cnt = (w >= h * 4 || h >= w * 4) ? 4 : 5;
    double cost_of[33];
    for (int i = 0; i < 33; i++) { list[i] = -1; cost_of[i] = 1.7e+308; }
    rmd_ctx_t c = { satd, r, list, cost_of };
    if (r->fast) {
        static const int r4[10] = { 0, 1, 2, 6, 10, 14, 18, 22, 26, 30 };
        int map[35] = { 0 };
        for (int i = 0; i < 10; i++) map[r4[i]] = 1;
        for (int i = r->skip_ipd ? 3 : 0; i < 10; i++) rmd_check(&c, r4[i], i + 1);
        int r2[12], n2 = 0;
        for (int k = 0; k < 7; k++) {
            const int ipm = list[k];
            if (ipm >= 6) {
                if (!map[ipm - 2]) { r2[n2++] = ipm - 2; map[ipm - 2] = 1; }
                if (!map[ipm + 2]) { r2[n2++] = ipm + 2; map[ipm + 2] = 1; }
            }
        }
        for (int i = 0; i < n2; i++) rmd_check(&c, r2[i], MAX(cnt, 3));
        int r1[8], n1 = 0;
        for (int k = 0, i = 0; k < 3 && i < 10;) {
            const int ipm = list[i++];
            if (ipm >= 4) {
                k++;
                if (!map[ipm - 1]) { r1[n1++] = ipm - 1; map[ipm - 1] = 1; }
                if (ipm + 1 < 33 && !map[ipm + 1]) { r1[n1++] = ipm + 1; map[ipm + 1] = 1; }
            }
        }
        for (int i = 0; i < n1; i++) rmd_check(&c, r1[i], MIN(cnt, 5));
        for (int k = 0; k < 2; k++) {
            const int m = r->mpm[k];
            if (m < 33) {
                if (r->skip_ipd && m <= 2) continue;
                if (!map[m]) rmd_check(&c, m, MIN(cnt, 5));
            }
        }
    } else {
        for (int i = r->skip_ipd ? 3 : 0; i < 33; i++) rmd_check(&c, i, cnt);
    }
    int need[2] = { 0, 0 };
    for (int k = 0; k < 2; k++)
        if (r->mpm[k] != 33 && !(r->skip_ipd && r->mpm[k] <= 2)) need[k] = 1;
    for (int i = 0; i < cnt; i++) {
        if (need[0] && list[i] == r->mpm[0]) need[0] = 0;
        if (need[1] && list[i] == r->mpm[1]) need[1] = 0;
    }
    if (need[0] + need[1] == 2) {
        const int first = cost_of[r->mpm[0]] <= cost_of[r->mpm[1]];
        list[cnt - 2] = first ? r->mpm[0] : r->mpm[1];
        list[cnt - 1] = first ? r->mpm[1] : r->mpm[0];
    } else if (need[0] + need[1]) {
        const int add = need[0] ? 0 : 1;
        if (list[cnt - 1] == r->mpm[1 - add]) list[cnt - 2] = list[cnt - 1];
        list[cnt - 1] = r->mpm[add];
    }
    for (int i = cnt - 1; i >= 0; i--) {
        if (r->inter_satd != ~0ull && cost_of[list[i]] > (double)r->inter_satd * r->satd_threshold) cnt--;
        else break;
    }
    return cnt;
}

void orc_intra_rmd(const u32 *satd, const orc_rmd_req_t *reqs, int n, orc_rmd_out_t *out)
{
    for (int i = 0; i < n; i++) {
        int list[33];
        const int cnt = rmd_one(satd + (size_t)reqs[i].satd_row * 33, &reqs[i], list);
        for (int k = 0; k < 5; k++) out[i].list[k] = (s8)list[k];
        out[i].count = (u8)cnt;
        out[i].pad[0] = out[i].pad[1] = 0;
    }
}

/* ============================================================ weighted quantisation */

/* quant_non_zero's pic_wq_enable branch (src/quant.c:335-380): each level is
 * (s16)((|c| scale ns_scale 64 / weight + offset) >> shift) in 64-bit arithmetic, shift = 14 +
 * 7 - (log2_size - ns_shift) with ns_shift 7 (and ns_scale 181) for blocks whose log2 w + log2 h
 * is odd, offset (171 intra slice / 85) << (shift - 9); the weight of sample (i, j) is
 * wq[(i / step) * width + (j >> idx_shift)] of the 4x4 matrix for 4x4 blocks, else of the 8x8
 * one with idx_shift = max(log2 w, log2 h) - 3 and step = 1 << idx_shift */
static int quant_wq_block(const orc_rdoq_req_t *r, const u8 *wq4, const u8 *wq8, s16 *coef)
{
    const int lw = r->log2w, lh = r->log2h, w = 1 << lw, h = 1 << lh;
    if (w > 32)
        for (int i = 0; i < h; i++) memset(coef + i * w + 32, 0, sizeof(s16) * (w - 32));
    if (h > 32) memset(coef + w * h / 2, 0, sizeof(s16) * (w * h / 2));
    const int scale = Q_SCALE[r->qp];
    const int log2_size = (lw + lh) >> 1, odd = (lw + lh) & 1;
    const int ns_shift = odd ? 7 : 0, ns_scale = odd ? 181 : 1;
    const int tr_shift = 15 - 8 - (log2_size - ns_shift);
    const int shift = 14 + tr_shift;
    const s64 offset = (s64)(r->slice_type == 1 ? 171 : 85) << (shift - 9);
    const u8 *wq = (lw == 2 && lh == 2) ? wq4 : wq8;
    const int idx_shift = (lw == 2 && lh == 2) ? 0 : MAX(lw, lh) - 3;
    const int width = (lw == 2 && lh == 2) ? 4 : 8;
    int nz = 0;
    for (int i = 0; i < h; i++)
        for (int j = 0; j < w; j++) {
            const int c = coef[i * w + j];
            const int weight = wq[(i >> idx_shift) * width + (j >> idx_shift)];
            const int lev = (s16)(((s64)ABSI(c) * scale * ns_scale * 64 / weight + offset) >> shift);
            coef[i * w + j] = (s16)(c < 0 ? -lev : lev);
            nz += coef[i * w + j] != 0;
        }
    return nz;
}

void orc_quant_wq(const orc_rdoq_req_t *reqs, int n, const u8 *wq4, const u8 *wq8, s16 *coefs, s32 *num_nz)
{
    orc_init();
    for (int i = 0; i < n; i++) num_nz[i] = quant_wq_block(&reqs[i], wq4, wq8, coefs + reqs[i].coef_offset);
}

/* ============================================================ affine motion search */

#define CPMV_MIN (-131072)
#define CPMV_MAX 131071

/* Tab_Affine_AMVR (inc/com_define.h:203): CPMV step of the affine AMVR index */
static int affme_shift(int mvr) { return mvr == 0 ? 2 : (mvr == 1 ? 4 : 0); }

/* MV_COST (src/inter.c:41): unsigned 32-bit product, rounded */
static u32 affme_mv_cost(u32 lambda_mv, int bits) { return (u32)(lambda_mv * (u32)bits + 32768u) >> 16; }

/* affine_mv_bits (src/inter.c:1317-1337) */
static int affme_bits(const s32 (*mv)[2], const s32 (*mvp)[2], int num_refp, int refi, int mvr)
{
    int bits = num_refp <= 1 ? 0 : MIN(refi + 1, num_refp - 1);     /* tbl_refi_bits, src/tables.c:52 */
    const int sh = affme_shift(mvr);
    for (int v = 0; v < 2; v++) {
        int dx = ABSI((mv[v][0] - mvp[v][0]) >> sh), dy = ABSI((mv[v][1] - mvp[v][1]) >> sh);
        bits += ((ilog2(dx + 1) + ilog2(dy + 1)) << 1) + 2 + !!dx + !!dy;
    }
    return bits;
}

/* com_mc_blk_affine_luma (src/com_mc.c:202-250): two control points, sub x sub blocks, each
 * filtered from the integer plane at its 1/16-sample MV */
static void affme_pred(int W, int H, int x, int y, int cw, int ch, const s32 (*ac)[2], int sub, const pel *plane,
                       int i_ref, pel *pred)
{
    const int lw = ilog2(cw), half = sub >> 1;
    const s32 dhx = ((ac[1][0] - ac[0][0]) * 128) >> lw, dhy = ((ac[1][1] - ac[0][1]) * 128) >> lw;
    const s32 dvx = -dhy, dvy = dhx;
    for (int h = 0; h < ch; h += sub)
        for (int w = 0; w < cw; w += sub) {
            int px = w + half, py = h + half;
            if (w == 0 && h == 0) { px = 0; py = 0; }
            else if (w + sub == cw && h == 0) { px = cw; py = 0; }
            s32 mx = CLIP3(CPMV_MIN, CPMV_MAX, affine_round7(ac[0][0] * 128 + dhx * px + dvx * py));
            s32 my = CLIP3(CPMV_MIN, CPMV_MAX, affine_round7(ac[0][1] * 128 + dhy * px + dvy * py));
            affine_luma_blk(plane, i_ref, pred + h * cw + w, cw, ((x + w) << 4) + mx, ((y + h) << 4) + my, sub, sub,
                            W + 4, H + 4);
        }
}

/* (s16) of a double the way x86-64 code converts it (cvttsd2si to 32 bits, then the low 16
 * bits): NaN and values outside the 32-bit range become INT_MIN, whose low half is 0 */
static s16 affme_to_s16(double v)
{
    int i = (v > -2147483649.0 && v < 2147483648.0) ? (int)v : (int)0x80000000u;
    return (s16)i;
}

/* solve_equal (src/inter.c:1280-1315): Gaussian elimination with partial pivoting over the
 * rows 1..order of a (row 0 is the swap buffer), then back substitution.  Bit-exact doubles
 * need the reference's operation order, which this follows term by term. */
static void affme_solve(double (*a)[5], int order, double *x)
{
    for (int i = 1; i < order; i++) {
        double best = fabs(a[i][i - 1]);
        int bi = i;
        for (int j = i + 1; j < order + 1; j++)
            if (fabs(a[j][i - 1]) > best) { best = fabs(a[j][i - 1]); bi = j; }
        if (bi != i)
            for (int j = 0; j < order + 1; j++) { a[0][j] = a[i][j]; a[i][j] = a[bi][j]; a[bi][j] = a[0][j]; }
        for (int j = i + 1; j < order + 1; j++)
            for (int k = i; k < order + 1; k++) {
                double t = a[i][k] * a[j][i - 1];
                t = t / a[i][i - 1];
                a[j][k] = a[j][k] - t;
            }
    }
    x[order - 1] = a[order][order] / a[order][order - 1];
    for (int i = order - 2; i >= 0; i--) {
        double t = 0;
        for (int j = i + 1; j < order; j++) {
            double m = a[i + 1][j] * x[j];
            t = t + m;
        }
        x[i] = (a[i + 1][order] - t) / a[i + 1][i];
    }
}

/* the normal equations of one gradient step: residual, Sobel gradients of the prediction
 * (affine_sobel_flt_hor / _ver, src/com_util.c:2966-3018: interior 3x3 Sobel, border samples
 * copy their nearest interior neighbour) and their products (affine_coef_computer, :3020) */
static void affme_equations(const pel *org, int i_org, const pel *pred, int w, int h, s64 (*coef)[5])
{
    memset(coef, 0, sizeof(s64) * 25);
    for (int j = 0; j < h; j++)
        for (int k = 0; k < w; k++) {
            const int jj = CLIP3(1, h - 2, j), kk = CLIP3(1, w - 2, k);
            const pel *p = pred + jj * w + kk;
            const int gx = p[1 - w] - p[-1 - w] + 2 * p[1] - 2 * p[-1] + p[1 + w] - p[-1 + w];
            const int gy = p[w - 1] - p[-w - 1] + 2 * p[w] - 2 * p[-w] + p[w + 1] - p[-w + 1];
            const int resi = org[j * i_org + k] - pred[j * w + k];
            const int c[4] = { gx, k * gx + j * gy, gy, j * gx - k * gy };
            for (int col = 0; col < 4; col++) {
                for (int row = 0; row < 4; row++) coef[col + 1][row] += (s64)c[col] * c[row];
                coef[col + 1][4] += (s64)c[col] * resi * 8;
            }
        }
}

typedef struct {
    int W, H, x, y, w, h, sub, bi, mvr, num_refp, refi, other_bits;
    u32 lambda;
    const pel *org, *plane;
    int i_org, i_ref;
} affme_ctx_t;

static u64 affme_cost(const affme_ctx_t *c, const s32 (*mv)[2], const s32 (*mvp)[2], pel *pred, int *bits)
{
    affme_pred(c->W, c->H, c->x, c->y, c->w, c->h, mv, c->sub, c->plane, c->i_ref, pred);
    *bits = affme_bits(mv, mvp, c->num_refp, c->refi, c->mvr) + (c->bi ? c->other_bits : 0);
    return (u64)affme_mv_cost(c->lambda, *bits) + (orc_had(c->w, c->h, c->org, c->i_org, pred, c->w, 8) >> c->bi);
}

/* affine_me_gradient (src/inter.c:1339-1470): up to 7 (uni) / 5 (bi) Gauss-Newton steps on the
 * 4-parameter model; each step's CPMV change rounded to the AMVR step, kept only when the
 * SATD + MV cost drops.  mv in/out; returns the SATD part of the best cost. */
static u64 affme_gradient(const affme_ctx_t *c, const s32 (*mvp)[2], s32 (*mv)[2], int *best_bits_out)
{
    pel pred[64 * 64];
    s32 mvt[2][2] = { { mv[0][0], mv[0][1] }, { mv[1][0], mv[1][1] } };
    int best_bits, bits;
    u64 best = affme_cost(c, (const s32 (*)[2])mvt, mvp, pred, &best_bits);
    const int sh = affme_shift(c->mvr);
    for (int iter = 0; iter < (c->bi ? 5 : 7); iter++) {
        s64 coef[5][5];
        double a[5][5], para[4], d[4];
        affme_equations(c->org, c->i_org, pred, c->w, c->h, coef);
        for (int r = 0; r < 5; r++)
            for (int k = 0; k < 5; k++) a[r][k] = (double)coef[r][k];
        affme_solve(a, 4, para);
        d[0] = para[0];
        d[2] = para[2];
        d[1] = para[1] * c->w + para[0];
        d[3] = -para[3] * c->w + para[2];
        s16 mvd[4];                        /* x0, y0, x1, y1 */
        const int order[4] = { 0, 2, 1, 3 };
        for (int v = 0; v < 4; v++) {
            const double dv = d[order[v]];
            if (sh == 0) mvd[v] = affme_to_s16(dv * 16 + (dv >= 0 ? 0.5 : -0.5));
            else {
                mvd[v] = affme_to_s16(dv * 4 + (dv >= 0 ? 0.5 : -0.5));
                mvd[v] = (s16)(mvd[v] << 2);
                mvd[v] = (s16)(((mvd[v] + (1 << (sh - 1))) >> sh) << sh);   /* com_mv_rounding_s16 */
            }
        }
        if (!mvd[0] && !mvd[1] && !mvd[2] && !mvd[3]) break;
        for (int v = 0; v < 2; v++)
            for (int k = 0; k < 2; k++) {
                s32 m = CLIP3(CPMV_MIN, CPMV_MAX, mvt[v][k] + mvd[v * 2 + k]);
                if (m == CPMV_MAX) m = m >> sh << sh;
                mvt[v][k] = m;
            }
        u64 cost = affme_cost(c, (const s32 (*)[2])mvt, mvp, pred, &bits);
        if (cost < best) {
            best = cost;
            best_bits = bits;
            memcpy(mv, mvt, sizeof(mvt));
        }
    }
    *best_bits_out = best_bits;
    return best - affme_mv_cost(c->lambda, best_bits);
}

/* the start CPMVs of analyze_affine_uni (src/inter.c:1607-1647): the better (SATD + MV cost) of
 * the MVP and the uni-prediction MV clipped as mv_clip does (:1472), scaled to 1/16 samples and,
 * at AMVR index 1, rounded to whole samples */
static void affme_uni_start(const affme_ctx_t *c, const s32 (*mvp)[2], s32 um_x, s32 um_y, s32 (*start)[2])
{
    pel pred[64 * 64];
    int bits;
    const u64 c_mvp = affme_cost(c, mvp, mvp, pred, &bits);
    const int x = c->x << 2, y = c->y << 2, w = c->w << 2, h = c->h << 2;
    const int min_x = (-128 - 4) << 2, min_y = (-128 - 4) << 2;
    const int max_x = (c->W - 1 + 128 + 4) << 2, max_y = (c->H - 1 + 128 + 4) << 2;
    s16 mx = (s16)um_x, my = (s16)um_y;
    if (x + mx < min_x) mx = (s16)(min_x - x);
    if (y + my < min_y) my = (s16)(min_y - y);
    if (x + mx + w - 4 > max_x) mx = (s16)(max_x - x - w + 4);
    if (y + my + h - 4 > max_y) my = (s16)(max_y - y - h + 4);
    s32 tx = (s32)mx << 2, ty = (s32)my << 2;
    if (c->mvr == 1) {
        tx = tx >= 0 ? ((tx + 8) >> 4) << 4 : -(((-tx + 8) >> 4) << 4);
        ty = ty >= 0 ? ((ty + 8) >> 4) << 4 : -(((-ty + 8) >> 4) << 4);
    }
    tx = CLIP3(CPMV_MIN, CPMV_MAX, tx);
    ty = CLIP3(CPMV_MIN, CPMV_MAX, ty);
    const s32 tmp[2][2] = { { tx, ty }, { tx, ty } };
    const u64 c_tmp = affme_cost(c, tmp, mvp, pred, &bits);
    memcpy(start, c_tmp < c_mvp ? tmp : mvp, sizeof(tmp));
}

static void affme_one(int W, int H, const pel *org, int i_org, const pel *const *planes, int i_ref,
                      const orc_affme_req_t *r, orc_affme_out_t *o)
{
    pel org_bi[64 * 64];
    affme_ctx_t c;
    c.W = W; c.H = H; c.x = r->x; c.y = r->y; c.w = r->w; c.h = r->h;
    c.bi = r->flags & ORC_AFFME_BI;
    c.sub = (c.bi || (r->flags & ORC_AFFME_SUB8)) ? 8 : 4;
    c.mvr = r->mvr; c.num_refp = r->num_refp; c.refi = r->refi; c.other_bits = r->mot_bits_other;
    c.lambda = r->lambda_mv;
    c.plane = planes[r->ref_slot * 16];
    c.i_ref = i_ref;
    c.org = org + r->y * i_org + r->x;
    c.i_org = i_org;
    if (c.bi) {                           /* create_bi_org (src/inter.c:55) over an 8x8 prediction */
        pel pred[64 * 64];
        affme_pred(W, H, r->x, r->y, r->w, r->h, r->other_mv, 8, planes[r->other_slot * 16], i_ref, pred);
        for (int j = 0; j < r->h; j++)
            for (int i = 0; i < r->w; i++)
                org_bi[j * r->w + i] = (pel)CLIP3(0, 255, (c.org[j * i_org + i] << 1) - pred[j * r->w + i]);
        c.org = org_bi;
        c.i_org = r->w;
    }
    s32 mv[2][2];
    if (!c.bi && (r->flags & ORC_AFFME_UNI_START)) affme_uni_start(&c, r->mvp, r->mv[0][0], r->mv[0][1], mv);
    else memcpy(mv, r->mv, sizeof(mv));
    int bits;
    const u64 satd = affme_gradient(&c, r->mvp, mv, &bits);
    memcpy(o->mv, mv, sizeof(mv));
    o->satd = (u32)satd;
    o->bits = bits;
    o->cost = satd + affme_mv_cost(c.lambda, bits);
}

static int affme_valid(int W, int H, const orc_affme_req_t *r)
{
    const int w = r->w, h = r->h;
    if ((w != 16 && w != 32 && w != 64) || (h != 16 && h != 32 && h != 64)) return 0;
    if (r->x < 0 || r->y < 0 || r->x + w > W || r->y + h > H || r->mvr > 2 || r->refi < 0 || r->refi >= r->num_refp)
        return 0;
    for (int v = 0; v < 2; v++)
        for (int k = 0; k < 2; k++) {
            if (r->mvp[v][k] < CPMV_MIN || r->mvp[v][k] > CPMV_MAX) return 0;
            if (!(r->flags & ORC_AFFME_UNI_START) && (r->mv[v][k] < CPMV_MIN || r->mv[v][k] > CPMV_MAX)) return 0;
            if ((r->flags & ORC_AFFME_BI) && (r->other_mv[v][k] < CPMV_MIN || r->other_mv[v][k] > CPMV_MAX)) return 0;
        }
    return 1;
}

void orc_me_affine(int width, int height, const pel *org, int i_org, const pel *const *planes, int i_ref,
                   const orc_affme_req_t *reqs, int n, orc_affme_out_t *out, int threads)
{
    orc_init();
#ifdef _OPENMP
    if (threads < 1) threads = 1;
    #pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
#endif
    for (int i = 0; i < n; i++) {
        if (affme_valid(width, height, &reqs[i])) affme_one(width, height, org, i_org, planes, i_ref, &reqs[i], &out[i]);
        else {
            memcpy(out[i].mv, reqs[i].mv, sizeof(out[i].mv));
            out[i].satd = 0;
            out[i].bits = 0;
            out[i].cost = ~0ull;
        }
    }
    (void)threads;
}

/* ============================================================ RDOQ of a transform block */

/* rdoq_one_coef (src/quant.c:158-194): the cheaper of keeping the coefficient at its level, one
 * below, or (implicitly) zero; u32 arithmetic of the level difference as in the reference */
static u32 rdoq_coef(s64 uncoded, s64 *coded, u32 level_double, u32 abs_level, const s32 *est_run,
                     const s32 (*est_level)[2], int q_bits, s32 err_scale, s64 lambda, int last_pos)
{
    u32 best = 0;
    *coded = uncoded + (s64)est_run[0] * lambda;
    for (int checks = 2; abs_level && checks; checks--, abs_level--) {
        s32 diff = (s32)(level_double - (abs_level << q_bits));
        s64 err = ((s64)diff * err_scale) >> 20;
        s32 rate = 32768;
        if (!last_pos) rate += est_run[1];
        if (abs_level == 1) rate += est_level[0][1];
        else if (abs_level < 9) rate += est_level[0][0] + est_level[1][0] * (s32)(abs_level - 2) + est_level[1][1];
        else rate += est_level[0][0] + est_level[1][0] * 7 + ((ilog2((int)abs_level - 8) << 1) + 1) * 32768;
        s64 cost = err * err + (s64)rate * lambda;
        if (cost < *coded) { best = abs_level; *coded = cost; }
    }
    return best;
}

static int rdoq_block(const orc_rdoq_req_t *r, const orc_rdoq_est_t *E, s16 *coef)
{
    const int lw = r->log2w, lh = r->log2h, w = 1 << lw, h = 1 << lh, qp = r->qp, ch = r->ch_type;
    /* quant_non_zero (src/quant.c:315-336): coefficients past 32 columns / rows are zeroed */
    if (w > 32)
        for (int y = 0; y < h; y++) memset(coef + y * w + 32, 0, 32 * sizeof(s16));
    if (h > 32) memset(coef + w * h / 2, 0, (size_t)w * h / 2 * sizeof(s16));
    /* rdoq_quant_block (src/quant.c:196-313) */
    const int odd = (lw + lh) & 1, log2_size = (lw + lh) >> 1;
    const int q_bits = 14 + (15 - 8 - log2_size);
    const int q_value = odd ? (Q_SCALE[qp] * 181 + 64) >> 7 : Q_SCALE[qp];
    const int max_num = 1 << (lw + lh), max_used = 1 << (lw + MIN(5, lh));
    const int offset = (r->slice_type == 1 ? 201 : 153) << (q_bits - 9);
    const int nz_thr = ((((1 << q_bits) - offset) << 10) / q_value - 1) >> 10;
    if (orc_quant_check(coef, max_used, nz_thr)) return 0;
    static s16 c1[64 * 64], lev[64 * 64];
    static u32 absc[64 * 64];
    static s64 zerr[64 * 64];
    const s32 err_scale = RDOQ_ERR_SCALE[qp][log2_size - 1];
    const u16 *scan = SCAN[lw][lh];
    for (int i = 0; i < max_num; i++) c1[i] = coef[scan[i]];
    const int last_nz = orc_quant_rdoq(c1, max_num, q_value, q_bits, err_scale, 20, absc, lev, zerr);
    const s64 lambda = r->lambda;
    s64 best_delta, curr_delta;
    if (!r->is_intra && ch == 0) { best_delta = (s64)E->ctp[1] * lambda; curr_delta = (s64)E->ctp[0] * lambda; }
    else { best_delta = (s64)E->cbf[ch][0] * lambda; curr_delta = (s64)E->cbf[ch][1] * lambda; }
    const int base = ch == 0 ? 0 : 12;
    const s32 (*lst)[2] = E->lst[ch != 0][5];
    const s32 (*est_run)[2] = E->run + 10 + base, (*est_lvl)[2] = E->lvl + 10 + base;
    u32 last_b_zero = 0, end_pos = 0;
    int last_checked = 0, tmp_nz = 0, num_nz = 0, zero_bins = 0;
    memset(coef, 0, (size_t)max_num * sizeof(s16));
    for (int i = 0; i <= last_nz; i++) {
        if (!lev[i]) { zero_bins += est_run[last_b_zero][0]; last_b_zero = 1; continue; }
        if (zero_bins) { curr_delta += (s64)zero_bins * lambda; zero_bins = 0; }
        s64 cc;
        u32 level = rdoq_coef(zerr[i], &cc, absc[i], (u32)lev[i], est_run[last_b_zero], est_lvl, q_bits, err_scale,
                              lambda, i == max_num - 1);
        curr_delta += cc - zerr[i];
        if (level) {
            last_checked = i;
            coef[scan[i]] = (s16)(c1[i] < 0 ? -(int)level : (int)level);
            s64 f0 = (s64)lst[ilog2(i + 1)][0] * lambda, f1 = (s64)lst[ilog2(i + 1)][1] * lambda;
            s64 end_cost = curr_delta + f1;
            curr_delta += f0;
            tmp_nz++;
            if (end_cost < best_delta) { best_delta = end_cost; end_pos = (u32)i; num_nz += tmp_nz; tmp_nz = 0; }
            last_b_zero = 0;
            int off = (MIN((int)level - 1, 5) << 1) + base;
            est_lvl = E->lvl + off;
            est_run = E->run + off;
            lst = E->lst[ch != 0][MIN((int)level - 1, 5)];
        } else {
            last_b_zero = 1;
        }
    }
    if (num_nz)
        for (int i = (int)end_pos + 1; i <= last_checked; i++) coef[scan[i]] = 0;
    return num_nz;
}

void orc_rdoq(const orc_rdoq_req_t *reqs, int n, const orc_rdoq_est_t *ests, s16 *coefs, s32 *num_nz)
{
    orc_init();
    for (int i = 0; i < n; i++) num_nz[i] = rdoq_block(&reqs[i], &ests[reqs[i].est], coefs + reqs[i].coef_offset);
}

/* ======================================================================================
 * Affine control-point MVP -- com_get_affine_mvp_scaling, src/com_util.c:1983-2058, with
 * scaling_mv1 (src/com_util.c:322-341) and com_mv_rounding_s32 (inc/com_util.h:189-194)
 * ====================================================================================== */

/* the neighbour's MV scaled by the ratio of POC distances (both from the current picture):
 * ratio = (2^14 / t_neb) * t_cur with C's truncating division first, then a symmetric rounding
 * shift and an s16 clip */
static s16 affmvp_scale(s16 mv, int ratio)
{
    const s64 t = (s64)mv * ratio;
    s64 r = t == 0 ? 0 : t > 0 ? (t + 8192) >> 14 : -((-t + 8192) >> 14);
    if (r < -32768) r = -32768;
    if (r > 32767) r = 32767;
    return (s16)r;
}

/* 1/4 -> 1/16 sample, rounded to the AMVR resolution (the magnitude rounded, the sign kept),
 * clipped to the 18-bit CPMV range */
static s32 affmvp_round(s16 v, int shift)
{
    const s32 x = (s32)v * 4;
    const s32 add = shift > 0 ? 1 << (shift - 1) : 0;
    s32 r = x >= 0 ? ((x + add) >> shift) << shift : -(((-x + add) >> shift) << shift);
    if (r < -131072) r = -131072;
    if (r > 131071) r = 131071;
    return r;
}

static int affmvp_one(s64 ptr, const s64 *ref_ptr, int n_ref, const s16 *map_mv, const s8 *map_refi,
                      long long n_field, int i_scu, const orc_affmvp_req_t *q, orc_affmvp_out_t *o)
{
    const int lidx = q->lidx;
    if (lidx < 0 || lidx > 1 || q->cur_refi < 0 || q->cur_refi >= n_ref || q->mvr < 0 || q->mvr > 2 ||
        q->cu_width < 4)
        return 1;
    const int t_cur = (int)(ptr * 2 - ref_ptr[q->cur_refi * 2 + lidx] * 2);
    if (t_cur == 0) return 1;
    const long long origin = i_scu + 1;
    const int wsc = q->cu_width >> 2;
    /* top-left: A (left), B (above), D (above-left); top-right: G (above the last column), C
     * (above-right); the first neighbour with a valid reference index in list lidx */
    const long long nb[5] = { q->scup - 1, q->scup - i_scu, q->scup - i_scu - 1,
                              q->scup - i_scu + wsc - 1, q->scup - i_scu + wsc };
    s16 mv[2][2] = { { 0, 0 }, { 0, 0 } };
    for (int g = 0; g < 2; g++) {
        const int k0 = g == 0 ? 0 : 3, k1 = g == 0 ? 3 : 5;
        for (int k = k0; k < k1; k++) {
            const long long a = origin + nb[k];
            if (a < 0 || a >= n_field) return 1;
            const int refi = map_refi[a * 2 + lidx];
            if (refi < 0) continue;
            if (refi >= n_ref) return 1;
            const int t_neb = (int)(ptr * 2 - ref_ptr[refi * 2 + lidx] * 2);
            if (t_neb == 0) return 1;
            const int ratio = (1 << 14) / t_neb * t_cur;
            mv[g][0] = affmvp_scale(map_mv[(a * 2 + lidx) * 2 + 0], ratio);
            mv[g][1] = affmvp_scale(map_mv[(a * 2 + lidx) * 2 + 1], ratio);
            break;
        }
    }
    const int shift = q->mvr == 0 ? 2 : q->mvr == 1 ? 4 : 0;
    for (int g = 0; g < 2; g++)
        for (int d = 0; d < 2; d++) o->mvp[g][d] = affmvp_round(mv[g][d], shift);
    return 0;
}

int orc_affine_mvp(s64 ptr, const s64 *ref_ptr, int n_ref, const s16 *map_mv, const s8 *map_refi, int i_scu,
                   int rows, const orc_affmvp_req_t *reqs, int n, orc_affmvp_out_t *out)
{
    int bad = 0;
    for (int i = 0; i < n; i++) {
        memset(&out[i], 0, sizeof(out[i]));
        if (affmvp_one(ptr, ref_ptr, n_ref, map_mv, map_refi, (long long)rows * i_scu, i_scu, &reqs[i], &out[i])) {
            memset(&out[i], 0, sizeof(out[i]));
            bad++;
        }
    }
    return bad;
}

/* ======================================================================================
 * Affine merge candidates -- com_get_affine_merge_candidate, src/com_util.c:1761-1981
 * ====================================================================================== */

/* com_mv_rounding_s32 with right shift 7, no left shift: the magnitude rounded, the sign kept */
static s32 affmrg_round7(s32 v)
{
    return v >= 0 ? (s32)(((u32)v + 64u) >> 7) : -(s32)(((u32)(-(s64)v) + 64u) >> 7);
}

static s32 affmrg_clip18(s32 v)
{
    return v < -131072 ? -131072 : v > 131071 ? 131071 : v;
}

/* scaling_mv1: the MV scaled by (2^14 / t_neb) * t_cur with symmetric rounding and an s16 clip */
static int affmrg_scale(s64 ptr_cur, s64 ptr_cur_ref, s64 ptr_neb, s64 ptr_neb_ref, const s16 mv[2], s16 out[2])
{
    const int t0 = (int)(ptr_neb * 2 - ptr_neb_ref * 2), t1 = (int)(ptr_cur * 2 - ptr_cur_ref * 2);
    if (t0 == 0 || t1 == 0) return 1;
    const int ratio = (1 << 14) / t0 * t1;
    for (int d = 0; d < 2; d++) {
        const s64 t = (s64)mv[d] * ratio;
        s64 r = t == 0 ? 0 : t > 0 ? (t + 8192) >> 14 : -((-t + 8192) >> 14);
        if (r < -32768) r = -32768;
        if (r > 32767) r = 32767;
        out[d] = (s16)r;
    }
    return 0;
}

/* the fields of one request, with bounds-checked reads (relative to SCU (0, 0)) */
typedef struct {
    const orc_affmrg_pic_t *P;
    const s16 *mv; const s8 *refi; const u8 *scu; const u32 *pos; const s16 *col_mv; const s8 *col_refi;
    long long origin, nf;
    int bad;
} affmrg_ctx_t;

static int affmrg_in(affmrg_ctx_t *c, long long a)
{
    if (a + c->origin < 0 || a + c->origin >= c->nf) { c->bad = 1; return 0; }
    return 1;
}
#define AM_SCU(c, a) (affmrg_in(c, a) ? (c)->scu[(a) + (c)->origin] : 0)
#define AM_POS(c, a) (affmrg_in(c, a) ? (c)->pos[(a) + (c)->origin] : 0u)
#define AM_REFI(c, a, l) (affmrg_in(c, a) ? (c)->refi[((a) + (c)->origin) * 2 + (l)] : -1)
#define AM_MV(c, a, l, d) (affmrg_in(c, a) ? (c)->mv[(((a) + (c)->origin) * 2 + (l)) * 2 + (d)] : 0)

/* com_derive_affine_model_mv: the CU's control points from the affine neighbour covering scun */
static void affmrg_model_mv(affmrg_ctx_t *c, int scup, int scun, int lidx, int cw, int ch, s32 mvp[3][2], int *vn)
{
    const int i_scu = c->P->i_scu;
    const u32 pos = AM_POS(c, scun);
    const int lw = (int)(pos & 7), lh = (int)((pos >> 3) & 7), nw = 1 << lw, nh = 1 << lh;
    const int diff_w = 7 - lw, diff_h = 7 - lh;
    const int a0 = (int)(pos >> 6), a1 = a0 + ((nw >> 2) - 1), a2 = a0 + ((nh >> 2) - 1) * i_scu, a3 = a2 + ((nw >> 2) - 1);
    int neb_x = (a0 % i_scu) << 2, neb_y = (a0 / i_scu) << 2;
    const int cur_x = (scup % i_scu) << 2, cur_y = (scup / i_scu) << 2;
    const int ad[4] = { a0, a1, a2, a3 };
    s32 nm[4][2];
    for (int i = 0; i < 4; i++)
        for (int d = 0; d < 2; d++) nm[i][d] = AM_MV(c, ad[i], lidx, d);
    int top = 0;
    if ((neb_y + nh) % (1 << c->P->log2_max_cuwh) == 0 && neb_y + nh == cur_y) {
        top = 1;
        neb_y += nh;
        nm[0][0] = nm[2][0]; nm[0][1] = nm[2][1];
        nm[1][0] = nm[3][0]; nm[1][1] = nm[3][1];
    }
    const s32 dhx = (s32)((u32)(nm[1][0] - nm[0][0]) << diff_w), dhy = (s32)((u32)(nm[1][1] - nm[0][1]) << diff_w);
    s32 dvx, dvy;
    if (*vn == 3 && !top) {
        dvx = (s32)((u32)(nm[2][0] - nm[0][0]) << diff_h);
        dvy = (s32)((u32)(nm[2][1] - nm[0][1]) << diff_h);
    } else {
        dvx = -dhy;
        dvy = dhx;
        *vn = 2;
    }
    const s32 hb = (s32)((u32)nm[0][0] << 7), vb = (s32)((u32)nm[0][1] << 7);
    for (int k = 0; k < *vn; k++) {
        const int ox = cur_x - neb_x + (k == 1 ? cw : 0), oy = cur_y - neb_y + (k == 2 ? ch : 0);
        const s32 th = (s32)((u32)dhx * (u32)ox + (u32)dvx * (u32)oy + (u32)hb);
        const s32 tv = (s32)((u32)dhy * (u32)ox + (u32)dvy * (u32)oy + (u32)vb);
        mvp[k][0] = affmrg_clip18((s32)((u32)affmrg_round7(th) << 2));
        mvp[k][1] = affmrg_clip18((s32)((u32)affmrg_round7(tv) << 2));
    }
}

/* com_derive_affine_constructed_candidate for one model (cp_idx[0..ver-1]) */
static void affmrg_constructed(orc_affmrg_out_t *o, int *cnt, int cw, int ch, const int valid[4], const s16 cmv[2][4][2],
                               const int crefi[2][4], const int *cp_idx, int model, int ver)
{
    if (*cnt >= 5) return;
    for (int i = 0; i < ver; i++)
        if (!valid[cp_idx[i]]) return;
    int vm[2] = { 0, 0 };
    for (int l = 0; l < 2; l++) {
        int ok = 1;
        for (int i = 0; i < ver; i++)
            if (crefi[l][cp_idx[i]] < 0 || crefi[l][cp_idx[i]] != crefi[l][cp_idx[0]]) ok = 0;
        vm[l] = ok;
    }
    if (!vm[0] && !vm[1]) return;
    const int k = *cnt;
    o->cp_num[k] = (s8)ver;
    const int lw = cw == 16 ? 4 : cw == 32 ? 5 : cw == 64 ? 6 : 7, lh = ch == 16 ? 4 : ch == 32 ? 5 : ch == 64 ? 6 : 7;
    const int sh = 7 + lw - lh;
    for (int l = 0; l < 2; l++) {
        if (!vm[l]) {
            o->refi[k][l] = -1;
            for (int i = 0; i < ver; i++) o->cpmv[k][l][i][0] = o->cpmv[k][l][i][1] = 0;
            continue;
        }
        s32 t[4][2] = { { 0, 0 }, { 0, 0 }, { 0, 0 }, { 0, 0 } };
        for (int i = 0; i < ver; i++) { t[cp_idx[i]][0] = cmv[l][cp_idx[i]][0]; t[cp_idx[i]][1] = cmv[l][cp_idx[i]][1]; }
        for (int d = 0; d < 2; d++) {
            if (model == 1) t[2][d] = t[3][d] + t[0][d] - t[1][d];
            if (model == 2) t[1][d] = t[3][d] + t[0][d] - t[2][d];
            if (model == 3) t[0][d] = t[1][d] + t[2][d] - t[3][d];
        }
        if (model == 5) {
            const s32 th = (s32)(((u32)(t[2][1] - t[0][1]) << sh) + ((u32)t[0][0] << 7));
            const s32 tv = (s32)((u32)(-(s32)((u32)(t[2][0] - t[0][0]) << sh)) + ((u32)t[0][1] << 7));
            t[1][0] = affmrg_round7(th);
            t[1][1] = affmrg_round7(tv);
        }
        o->refi[k][l] = (s8)crefi[l][cp_idx[0]];
        for (int i = 0; i < ver; i++)
            for (int d = 0; d < 2; d++) o->cpmv[k][l][i][d] = affmrg_clip18((s32)((u32)t[i][d] << 2));
    }
    (*cnt)++;
}

static int affmrg_one(const orc_affmrg_pic_t *P, affmrg_ctx_t *c, const orc_affmrg_req_t *q, orc_affmrg_out_t *o)
{
    const int cw = q->cu_width, ch = q->cu_height;
    if ((cw != 16 && cw != 32 && cw != 64 && cw != 128) || (ch != 16 && ch != 32 && ch != 64 && ch != 128)) return 1;
    const int i_scu = P->i_scu, scup = q->scup, wsc = cw >> 2, hsc = ch >> 2;
    c->bad = 0;
    int cnt = 0;
    /* model-based: F, G, C, A, D; the first two affine neighbours of distinct CUs */
    {
        const int nb[5] = { scup + i_scu * (hsc - 1) - 1, scup - i_scu + wsc - 1, scup - i_scu + wsc, scup - 1,
                            scup - i_scu - 1 };
        int valid[5], tl[5] = { 0, 0, 0, 0, 0 };
        for (int k = 0; k < 5; k++) {
            valid[k] = (AM_SCU(c, nb[k]) >> 4) & 3;
            if (valid[k]) tl[k] = (int)(AM_POS(c, nb[k]) >> 6);
        }
        if (valid[2] && valid[1] && tl[1] == tl[2]) valid[2] = 0;
        const int v3 = valid[3];
        if (valid[3] && valid[0] && tl[0] == tl[3]) valid[3] = 0;
        if ((valid[4] && v3 && tl[4] == tl[3]) || (valid[4] && valid[1] && tl[4] == tl[1])) valid[4] = 0;
        for (int k = 0; k < 5; k++) {
            if (valid[k]) {
                int vn = ((AM_SCU(c, nb[k]) >> 4) & 3) == 1 ? 2 : 3;
                for (int l = 0; l < 2; l++) {
                    const int r = AM_REFI(c, nb[k], l);
                    if (r >= 0) {
                        o->refi[cnt][l] = (s8)r;
                        affmrg_model_mv(c, scup, nb[k], l, cw, ch, o->cpmv[cnt][l], &vn);
                    } else {
                        o->refi[cnt][l] = -1;
                        memset(o->cpmv[cnt][l], 0, sizeof(o->cpmv[cnt][l]));
                    }
                }
                o->cp_num[cnt] = (s8)vn;
                cnt++;
            }
            if (cnt >= 2) break;
        }
    }
    /* control points: LT from A, B, D; RT from G, C; LB from F (the first inter SCU); RB from
     * the colocated picture at the bottom-right SCU's colocated position, scaled */
    {
        s16 cmv[2][4][2];
        int crefi[2][4], valid[4] = { 0, 0, 0, 0 };
        memset(cmv, 0, sizeof(cmv));
        for (int l = 0; l < 2; l++)
            for (int i = 0; i < 4; i++) crefi[l][i] = -1;
        const int lt[3] = { scup - 1, scup - i_scu, scup - i_scu - 1 }, rt[2] = { scup - i_scu + wsc - 1, scup - i_scu + wsc };
        const int lb = scup + i_scu * (hsc - 1) - 1;
        for (int g = 0; g < 3; g++) {
            const int n = g == 0 ? 3 : g == 1 ? 2 : 1;
            for (int k = 0; k < n; k++) {
                const int a = g == 0 ? lt[k] : g == 1 ? rt[k] : lb;
                if ((AM_SCU(c, a) & 3) != 1) continue;
                for (int l = 0; l < 2; l++) {
                    crefi[l][g] = AM_REFI(c, a, l);
                    cmv[l][g][0] = (s16)AM_MV(c, a, l, 0);
                    cmv[l][g][1] = (s16)AM_MV(c, a, l, 1);
                }
                valid[g] = 1;
                break;
            }
        }
        const int rb = scup + i_scu * (hsc - 1) + (wsc - 1);
        /* get_colocal_scup */
        const int bx = rb % i_scu, by = rb / i_scu;
        int xpos = (bx & ~3) + 2, ypos = (by & ~3) + 2;
        if (ypos >= P->pic_height_in_scu) ypos = ((by & ~3) + P->pic_height_in_scu) >> 1;
        if (xpos >= P->pic_width_in_scu) xpos = ((bx & ~3) + P->pic_width_in_scu) >> 1;
        const long long co = (long long)ypos * i_scu + xpos;
        if (co + c->origin < 0 || co + c->origin >= c->nf) return 1;
        const int cr = c->col_refi[(co + c->origin) * 2 + 0];
        const s16 cm[2] = { c->col_mv[((co + c->origin) * 2 + 0) * 2 + 0], c->col_mv[((co + c->origin) * 2 + 0) * 2 + 1] };
        if (cr >= 17) return 1;
        if (P->slice_type == 3) {
            if (cr >= 0) {
                s16 m[2];
                for (int l = 0; l < 2; l++) {
                    if (affmrg_scale(P->ptr, P->ref0_ptr[l], P->ref0_ptr[1], P->col_list_ptr[cr], cm, m)) return 1;
                    crefi[l][3] = 0;
                    cmv[l][3][0] = m[0]; cmv[l][3][1] = m[1];
                }
                valid[3] = 1;
            }
        } else if (cr >= 0) {
            s16 m[2];
            if (affmrg_scale(P->ptr, P->ref0_ptr[0], P->ref0_ptr[0], P->col_list_ptr[cr], cm, m)) return 1;
            crefi[0][3] = 0;
            cmv[0][3][0] = m[0]; cmv[0][3][1] = m[1];
            crefi[1][3] = -1;
            cmv[1][3][0] = cmv[1][3][1] = 0;
            valid[3] = 1;
        }
        static const int models[6][3] = { { 0, 1, 2 }, { 0, 1, 3 }, { 0, 2, 3 }, { 1, 2, 3 }, { 0, 1, 0 }, { 0, 2, 0 } };
        static const int vers[6] = { 3, 3, 3, 3, 2, 2 };
        for (int m = 0; m < 6; m++) affmrg_constructed(o, &cnt, cw, ch, valid, cmv, crefi, models[m], m, vers[m]);
    }
    o->num = cnt;
    for (int k = cnt; k < 5; k++) {
        o->cp_num[k] = 2;
        memset(o->cpmv[k], 0, sizeof(o->cpmv[k]));
        o->refi[k][0] = 0;
        o->refi[k][1] = -1;
    }
    /* vertices past a candidate's control-point count carry nothing */
    for (int k = 0; k < 5; k++)
        for (int l = 0; l < 2; l++)
            for (int i = o->cp_num[k]; i < 3; i++) o->cpmv[k][l][i][0] = o->cpmv[k][l][i][1] = 0;
    return c->bad;
}

int orc_affine_merge(const orc_affmrg_pic_t *pic, const s16 *map_mv, const s8 *map_refi, const u8 *map_scu,
                     const u32 *map_pos, const s16 *col_mv, const s8 *col_refi, const orc_affmrg_req_t *reqs, int n,
                     orc_affmrg_out_t *out)
{
    affmrg_ctx_t c;
    c.P = pic; c.mv = map_mv; c.refi = map_refi; c.scu = map_scu; c.pos = map_pos; c.col_mv = col_mv; c.col_refi = col_refi;
    c.origin = pic->i_scu + 1;
    c.nf = (long long)pic->rows * pic->i_scu;
    int bad = 0;
    for (int i = 0; i < n; i++) {
        memset(&out[i], 0, sizeof(out[i]));
        if (affmrg_one(pic, &c, &reqs[i], &out[i])) {
            memset(&out[i], 0, sizeof(out[i]));
            bad++;
        }
    }
    return bad;
}
