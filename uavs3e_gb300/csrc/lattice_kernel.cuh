// Device side of the batched intra lattice: the tile body of every CU shape class; the
// persistent kernel, the device work queue, the layout tuner and the C ABI are in lattice.cu.
#pragma once
#include "common.cuh"
#include "intra.cuh"
#include "tables.h"
#include "uavs3e_cuda_internal.h"
#include "quant_tables.cuh"

#include <type_traits>

namespace uc {

__device__ __constant__ static const u32 kDqScale[80] = {
    32768, 36061, 38968, 42495, 46341, 50535, 55437, 60424, 32932, 35734, 38968, 42495, 46177, 50535, 55109, 59933,
    65535, 35734, 38968, 42577, 46341, 50617, 55027, 60097, 32809, 35734, 38968, 42454, 46382, 50576, 55109, 60056,
    65535, 35734, 38968, 42495, 46320, 50515, 55109, 60076, 65535, 35744, 38968, 42495, 46341, 50535, 55099, 60087,
    65535, 35734, 38973, 42500, 46341, 50535, 55109, 60097, 32771, 35734, 38965, 42497, 46341, 50535, 55109, 60099,
    32768, 36061, 38968, 42495, 46341, 50535, 55437, 60424, 32932, 35734, 38968, 42495, 46177, 50535, 55109, 59933,
};
__device__ __constant__ static const u8 kDqShift[80] = {
    14, 14, 14, 14, 14, 14, 14, 14, 13, 13, 13, 13, 13, 13, 13, 13, 13, 12, 12, 12, 12, 12, 12, 12,
    11, 11, 11, 11, 11, 11, 11, 11, 11, 10, 10, 10, 10, 10, 10, 10, 10, 9, 9, 9, 9, 9, 9, 9,
    9, 8, 8, 8, 8, 8, 8, 8, 7, 7, 7, 7, 7, 7, 7, 7, 6, 6, 6, 6, 6, 6, 6, 6, 5, 5, 5, 5, 5, 5, 5, 5,
};

// weight of raster position p in the level hash of a record: odd, spread over 32 bits, so the
// hash sum_p level[p] * weight(p) (mod 2^32) changes with any single level, any sign and any
// exchange of two different levels
__host__ __device__ __forceinline__ constexpr u32 lat_pos_weight(u32 p) { return (p * 0x9E3779B1u + 0x7F4A7C15u) | 1u; }

// sum of 4 (unsigned byte of a) x (signed byte of b) products + c
__device__ __forceinline__ int dp4a_us(u32 a, u32 b, int c)
{
    int d;
    asm("dp4a.u32.s32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}
// sum of the 2 signed halfwords of a times signed bytes 0,1 (lo) or 2,3 (hi) of b, + c
__device__ __forceinline__ int dp2a_lo(u32 a, u32 b, int c)
{
    int d;
    asm("dp2a.lo.s32.s32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}
__device__ __forceinline__ int dp2a_hi(u32 a, u32 b, int c)
{
    int d;
    asm("dp2a.hi.s32.s32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

struct LatCu { s16 x, y; u8 w, h; u16 pad; };
struct LatQ { u32 ssd; u32 coef_hash; u16 num_nz; s16 last_nz; u32 sum_abs; };

constexpr int LAT_THREADS = 256;
constexpr int LAT_BUDGET = 48 * 1024;   // default dynamic shared bytes per CTA (4 CTAs per SM with the static part)
constexpr int LAT_MAX_QP = 4;
constexpr int LAT_SMEM_MAX = 96 * 1024;   // dynamic shared memory admitted by the kernel attribute
constexpr int LAT_MAX_G = 8;            // CUs per CTA
constexpr int LAT_MAX_JOBS = 33 * LAT_MAX_G;
constexpr int LAT_NB = 592;             // neighbour buffer per CU (INTRA_NEIB_SIZE + pad)
constexpr int LAT_SHAPES = 25;          // log2 sides 2..6

// shared-memory layout of one shape's CTAs (host and device compute it the same way)
struct LatLayout {
    int w, h, lw, lh, kw, kh, lkw, lkh;
    int ps;            // prediction / org row stride (bytes): 16-byte aligned rows
    int ts;            // forward row-pass output row stride (s16): 16-byte aligned rows
    int cs;            // coefficient row stride (s16): kw + 2
    int ds;            // transposed dequantised row stride (s16): 16-byte aligned rows
    int t2s;           // inverse column-pass output row stride (s16): 16-byte aligned rows
    int fw_ws, fh_ws, fht_ws, fwt_ws;   // table row strides in words
    int o_fw, o_fh, o_fht, o_fwt;       // table offsets
    int o_scan;                         // scan index of each kept coefficient, [v][u] (u16)
    int o_cu, cu_bytes;                 // per-CU blocks: org, neighbours, org row-pass sums
    int c_org, c_nb, c_torg;
    int o_job, job_bytes;               // per-job blocks: prediction, T, C, DQ^T, T2
    int j_pred, j_t, j_c, j_dqt, j_t2;
    int G, MC, nchunk;                  // CUs per CTA, modes per CTA, mode chunks per CU
    int smem;
};

__host__ __device__ __forceinline__ int lat_up16(int v) { return (v + 15) & ~15; }

// the layout of a CTA for (2^lw) x (2^lh) CUs and nm modes within `budget` bytes of dynamic
// shared memory: how many CUs (or which chunk of one CU's modes) a CTA takes
__host__ __device__ inline void lat_layout(int lw, int lh, int nm, int budget, LatLayout &L)
{
    L.lw = lw; L.lh = lh; L.w = 1 << lw; L.h = 1 << lh;
    L.kw = L.w < 32 ? L.w : 32; L.kh = L.h < 32 ? L.h : 32;
    L.lkw = lw < 5 ? lw : 5; L.lkh = lh < 5 ? lh : 5;
    // rows that are read whole by every lane of a warp (broadcast) start on 16 bytes; the
    // strides also keep the rows 8 lanes read at once on distinct banks
    L.ps = L.w <= 8 ? 16 : L.w <= 32 ? 48 : 80;
    L.ts = L.h >= 8 ? L.h + 8 : 8;
    L.cs = L.kw + 2;
    L.ds = L.kh >= 8 ? L.kh + 8 : 8;
    L.t2s = L.kw >= 8 ? L.kw + 8 : 8;
    // matrix rows are read one per lane: strides of an odd number of words
    L.fw_ws = L.w / 4 + 1; L.fh_ws = L.h / 4 + 1; L.fht_ws = L.kh / 4 + 1; L.fwt_ws = L.kw / 4 + 1;
    int o = 0;
    L.o_fw = o; o += lat_up16(L.kw * L.fw_ws * 4);
    L.o_fh = o; o += lat_up16(L.kh * L.fh_ws * 4);
    L.o_fht = o; o += lat_up16(L.h * L.fht_ws * 4);
    L.o_fwt = o; o += lat_up16(L.w * L.fwt_ws * 4);
    L.o_scan = o; o += lat_up16(L.kw * L.kh * 2);
    int c = 0;
    L.c_org = c; c += lat_up16(L.h * L.ps);
    L.c_nb = c; c += lat_up16(LAT_NB);
    L.c_torg = c; c += lat_up16(L.kw * L.h * 4);
    L.cu_bytes = c;
    int j = 0;
    L.j_pred = j; j += lat_up16(L.h * L.ps);
    L.j_t = j; j += lat_up16(L.kw * L.ts * 2);
    L.j_c = j; j += lat_up16(L.kh * L.cs * 2);
    L.j_dqt = j; j += lat_up16(L.kw * L.ds * 2);
    L.j_t2 = j; j += lat_up16(L.h * L.t2s * 2);
    L.job_bytes = j;
    const int avail = budget - o;
    // several whole CUs when nm jobs of the shape fit, else one CU and a chunk of its modes
    int G = avail / (nm * L.job_bytes + L.cu_bytes);
    if (G >= 1) {
        L.G = G < LAT_MAX_G ? G : LAT_MAX_G;
        L.MC = nm; L.nchunk = 1;
    } else {
        int J = (avail - L.cu_bytes) / L.job_bytes;
        J = J < 1 ? 1 : J;
        L.G = 1;
        L.nchunk = (nm + J - 1) / J;
        L.MC = (nm + L.nchunk - 1) / L.nchunk;
    }
    L.o_cu = o; o += L.G * L.cu_bytes;
    L.o_job = o; o += L.G * L.MC * L.job_bytes;
    L.smem = o;
}

struct LatParams {
    const pel *org; int i_org;
    int org_words;            // org and i_org are multiples of 4: org blocks are read by words
    const pel *rec; int i_rec;
    int W, H;
    const LatCu *cus;
    int ipf, n_qp, is_intra;
    int qp[LAT_MAX_QP];
    u32 *satd_out; LatQ *q_out;
    const s8 *fold[7];        // folded DCT2 matrices per log2 size
    const u16 *scanpos[7][7]; // raster -> scan index per (log2 w, log2 h)
    const u8 *modes;          // [CU][n_modes] modes to evaluate, or null for all 33 in order
    int n_modes;
    int budget[LAT_SHAPES];   // dynamic shared bytes of each shape class's layout (lat_layout)
    double sq32, sq128;
    u64 k32, k128;       // had_scale_k of sq32, sq128
    // the device work queue (written by k_lat_plan for each launch)
    const int *counts;        // [LAT_SHAPES] CUs per shape class
    const int *cu_off;        // [LAT_SHAPES] first entry of each class in perm
    const int *tile_off;      // [LAT_SHAPES + 1] first tile of the class of each launch rank; [25] = total
    const int *perm;          // CU indices grouped by class
    int *next;                // the next tile to take
};

// per-CTA shared scalars of a tile (the static part of the tile's shared memory)
struct LatShared {
    IpredBlock B[LAT_MAX_G];
    int cu[LAT_MAX_G];
    u8 mode[LAT_MAX_JOBS];
    u32 satd[LAT_MAX_JOBS], flag[LAT_MAX_JOBS];
    u32 nz[LAT_MAX_JOBS], sum[LAT_MAX_JOBS], hash[LAT_MAX_JOBS], ssd[LAT_MAX_JOBS];
    int last[LAT_MAX_JOBS];
    int tables;   // shape class whose matrices and scan table are in place (-1: none)
};

// lanes [k*seg, (k+1)*seg) of a warp hold one job's elements (seg = 16 or 32): the sum, max
// or or over the lane's segment, with the warp-wide reduction instructions
__device__ __forceinline__ u32 seg_sum(u32 v, int seg, int lane)
{
    if (seg == 32) return __reduce_add_sync(0xFFFFFFFFu, v);
    const u32 lo = __reduce_add_sync(0xFFFFFFFFu, lane < 16 ? v : 0u);
    const u32 hi = __reduce_add_sync(0xFFFFFFFFu, lane < 16 ? 0u : v);
    return lane < 16 ? lo : hi;
}
__device__ __forceinline__ int seg_max(int v, int seg, int lane)
{
    if (seg == 32) return __reduce_max_sync(0xFFFFFFFFu, v);
    const int lo = __reduce_max_sync(0xFFFFFFFFu, lane < 16 ? v : -1);
    const int hi = __reduce_max_sync(0xFFFFFFFFu, lane < 16 ? -1 : v);
    return lane < 16 ? lo : hi;
}
__device__ __forceinline__ u32 seg_or(u32 v, int seg, int lane)
{
    if (seg == 32) return __reduce_or_sync(0xFFFFFFFFu, v);
    const u32 lo = __reduce_or_sync(0xFFFFFFFFu, lane < 16 ? v : 0u);
    const u32 hi = __reduce_or_sync(0xFFFFFFFFu, lane < 16 ? 0u : v);
    return lane < 16 ? lo : hi;
}

// NW words of a row that every lane of a warp reads (16-byte aligned): vector loads
template <int NW>
__device__ __forceinline__ void lat_row(const void *p, u32 (&r)[NW])
{
    if constexpr (NW >= 4) {
#pragma unroll
        for (int k = 0; k < NW / 4; k++) {
            const uint4 v = reinterpret_cast<const uint4 *>(p)[k];
            r[4 * k] = v.x; r[4 * k + 1] = v.y; r[4 * k + 2] = v.z; r[4 * k + 3] = v.w;
        }
    } else if constexpr (NW == 2) {
        const uint2 v = *reinterpret_cast<const uint2 *>(p);
        r[0] = v.x; r[1] = v.y;
    } else {
        r[0] = *reinterpret_cast<const u32 *>(p);
    }
}

// position of index k in a row of n entries stored in even/odd order (the even k first)
__host__ __device__ __forceinline__ constexpr int lat_eo(int k, int n) { return (k & 1) ? (n >> 1) + (k >> 1) : (k >> 1); }

// the even part E and the odd part O of sum_k F[k] D[k] over N entries, D as s16 pairs and F as
// bytes, both in even/odd order (D: N/2 words, F: N/4 words)
template <int N>
__device__ __forceinline__ void lat_eo_sums(const u32 (&d)[N / 2], const u32 (&f)[N / 4], int &e, int &o)
{
#pragma unroll
    for (int p = 0; p < N / 4; p++) {
        constexpr int H = N / 2;
        const int be = 2 * p, bo = H + 2 * p;   // byte of the pair's first entry in F
        e = ((be >> 1) & 1) ? dp2a_hi(d[p], f[be >> 2], e) : dp2a_lo(d[p], f[be >> 2], e);
        o = ((bo >> 1) & 1) ? dp2a_hi(d[N / 4 + p], f[bo >> 2], o) : dp2a_lo(d[N / 4 + p], f[bo >> 2], o);
    }
}

// sum over aligned groups of SEG lanes (SEG a power of two <= 32)
template <int SEG>
__device__ __forceinline__ u32 lat_seg_sum(u32 v, int lane)
{
    if constexpr (SEG >= 16) {
        return seg_sum(v, SEG, lane);
    } else {
#pragma unroll
        for (int d = 1; d < SEG; d <<= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, d);
        return v;
    }
}

// maximum over aligned groups of SEG lanes
template <int SEG>
__device__ __forceinline__ int lat_seg_max(int v, int lane)
{
    if constexpr (SEG >= 16) {
        return seg_max(v, SEG, lane);
    } else {
#pragma unroll
        for (int d = 1; d < SEG; d <<= 1) v = max(v, __shfl_xor_sync(0xFFFFFFFFu, v, d));
        return v;
    }
}

// com_had tile of a (2^LW) x (2^LH) block (src/com_cost.c:712-812), as constants
constexpr int lat_tw(int w, int h)
{
    return w == h ? (w == 4 ? 4 : 8) : w > h ? (h == 4 ? 8 : 16) : (w == 4 ? 4 : 8);
}
constexpr int lat_th(int w, int h)
{
    return w == h ? (w == 4 ? 4 : 8) : w > h ? (h == 4 ? 4 : 8) : (w == 4 ? 8 : 16);
}

// SATD of every (job, tile) by groups of R lanes (R = 4 or 8, the transform size): lane k of a
// group holds row k of the tile's difference (of both halves for the 16x8 / 8x16 / 8x4 / 4x8
// tiles, which combine two R x R transforms), transforms it in registers, and the column
// transform runs across the group's lanes with shuffles.  Same coefficients, sums and
// normalisation as satd_tile.
template <int TW, int TH>
__device__ __forceinline__ void lat_satd_tiles(int n_tiles, int lnt, int ntx, const u8 *cub, int cu_bytes, int c_org,
                                               const u8 *jobb, int job_bytes, int j_pred, int ps, int MCv,
                                               u32 *s_satd, double sq32, double sq128, u64 k32, u64 k128)
{
    constexpr int R = (TW == 4 || TH == 4) ? 4 : 8;
    constexpr bool PAIR = TW != TH, SIDE = TW > TH;
    constexpr int GPW = 32 / R;                       // groups per warp
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int k = lane % R, grp = lane / R;
    for (int base = warp * GPW; base < n_tiles; base += (LAT_THREADS / 32) * GPW) {
        const int ti = base + grp;
        const bool act = ti < n_tiles;
        const int tt = act ? ti : base;
        const int j = tt >> lnt, t = tt & ((1 << lnt) - 1);
        const int ox = (t % ntx) * TW, oy = (t / ntx) * TH;
        const u8 *o = cub + (j / MCv) * cu_bytes + c_org + (oy + k) * ps + ox;
        const u8 *p = jobb + j * job_bytes + j_pred + (oy + k) * ps + ox;
        int a[R], b[R];
#pragma unroll
        for (int c = 0; c < R; c++) a[c] = (int)o[c] - (int)p[c];
        if (PAIR) {
            const int bo = SIDE ? R : R * ps;
#pragma unroll
            for (int c = 0; c < R; c++) b[c] = (int)o[bo + c] - (int)p[bo + c];
        }
        wht<R>(a);
        if (PAIR) wht<R>(b);
#pragma unroll
        for (int d = 1; d < R; d <<= 1) {
#pragma unroll
            for (int c = 0; c < R; c++) {
                const int x = __shfl_xor_sync(0xFFFFFFFFu, a[c], d);
                a[c] = (k & d) ? x - a[c] : a[c] + x;
                if (PAIR) {
                    const int y = __shfl_xor_sync(0xFFFFFFFFu, b[c], d);
                    b[c] = (k & d) ? y - b[c] : b[c] + y;
                }
            }
        }
        int sum = 0;
#pragma unroll
        for (int c = 0; c < R; c++) sum += PAIR ? 2 * max(abs(a[c]), abs(b[c])) : abs(a[c]);
#pragma unroll
        for (int d = 1; d < R; d <<= 1) sum += __shfl_xor_sync(0xFFFFFFFFu, sum, d);
        if (act && k == 0) {
            u32 v;
            if (!PAIR) v = R == 8 ? (u32)((sum + 2) >> 2) : (u32)((sum + 1) >> 1);
            else v = R == 8 ? had_scale(sum, sq128, k128) : had_scale(sum, sq32, k32);
            atomicAdd(&s_satd[j], v);
        }
    }
}

// Optional per-stage clocks (built with UAVS3E_LAT_STAGE_CLOCKS, off in the library): thread 0
// of each CTA adds the SM cycles between consecutive CTA barriers of a tile to
// g_lat_stage_clk[class][stage].  Stages: 0 tables and job setup, 1 org block and neighbours,
// 2 org row-pass sums and block setup, 3 prediction, 4 SATD and forward row pass, 5 forward
// column pass, then per QP 6 quantisation, 7 inverse column pass, 8 inverse row pass,
// reconstruction and SSD, 9 records.
constexpr int LAT_STAGES = 10;
#ifdef UAVS3E_LAT_STAGE_CLOCKS
__device__ unsigned long long g_lat_stage_clk[LAT_SHAPES][LAT_STAGES];
#define LAT_STAGE_BEGIN() long long lat_clk0 = clock64()
#define LAT_STAGE(k)                                                                                       \
    do {                                                                                                  \
        if (threadIdx.x == 0) {                                                                           \
            const long long t_ = clock64();                                                               \
            atomicAdd(&g_lat_stage_clk[(LW - 2) * 5 + (LH - 2)][k], (unsigned long long)(t_ - lat_clk0)); \
            lat_clk0 = t_;                                                                                \
        }                                                                                                 \
    } while (0)
#else
#define LAT_STAGE_BEGIN() do { } while (0)
#define LAT_STAGE(k) do { } while (0)
#endif

// One tile of shape class (LW, LH): a few whole CUs, or one CU and a chunk of its modes, as the
// class's layout says.  Called by every thread of the CTA; the tile's data lives in `sm` (the
// layout's dynamic shared memory) and `S`.
template <int LW, int LH>
__device__ __forceinline__ void lat_tile(const LatParams &P, const int *perm, int n_shape, int tile, u8 *sm,
                                         LatShared &S)
{
    IpredBlock *sB = S.B;
    int *s_cu = S.cu;
    u8 *s_mode = S.mode;
    u32 *s_satd = S.satd, *s_flag = S.flag, *s_nz = S.nz, *s_sum = S.sum, *s_hash = S.hash, *s_ssd = S.ssd;
    int *s_last = S.last;

    LatLayout L;
    LAT_STAGE_BEGIN();
    // compile-time shape: the indices and trip counts below are constants
    lat_layout(LW, LH, P.n_modes, P.budget[(LW - 2) * 5 + (LH - 2)], L);
    const int w = L.w, h = L.h, lw = L.lw, lh = L.lh, kw = L.kw, kh = L.kh, lkw = L.lkw, lkh = L.lkh;
    const int N = w * h, lN = lw + lh;
    constexpr int W_ = 1 << LW, H_ = 1 << LH, KW_ = W_ < 32 ? W_ : 32, KH_ = H_ < 32 ? H_ : 32;
    constexpr int LKW_ = LW < 5 ? LW : 5, LKH_ = LH < 5 ? LH : 5;
    // row passes: a task is one matrix row (in registers) against RY data rows; column passes:
    // against RU data columns.  Lanes of a warp take consecutive matrix rows, so the data row
    // they read is the same (one broadcast load).
    constexpr int RY = H_ < 8 ? H_ : 8, NYC = H_ / RY;
    constexpr int RU = KW_ < 8 ? KW_ : 8, NUC = KW_ / RU;
    const int tid = threadIdx.x, lane = tid & 31, wbase = tid & ~31;

    // this tile's CUs and modes
    const int grp = tile / L.nchunk, chunk = tile % L.nchunk;
    const int cu0 = grp * L.G;
    const int Gv = min(L.G, n_shape - cu0);
    const int m0 = chunk * L.MC;
    const int MCv = min(L.MC, P.n_modes - m0);
    const int J = Gv * MCv;
    if (Gv <= 0 || MCv <= 0) return;
    // j / MCv as a multiply: with m = ceil(2^16 / MCv), (j m) >> 16 = j / MCv for every
    // j * MCv < 2^16 (here j < 8 * 33 and MCv <= 33)
    const u32 mc_magic = (65536u + (u32)MCv - 1u) / (u32)MCv;

    u32 *fw = (u32 *)(sm + L.o_fw), *fh = (u32 *)(sm + L.o_fh);
    u32 *fht = (u32 *)(sm + L.o_fht), *fwt = (u32 *)(sm + L.o_fwt);
    u8 *cub = sm + L.o_cu, *jobb = sm + L.o_job;

    // ---- matrices: rows packed 4 bytes to a word.  The inverse passes use the even/odd
    // symmetry of the folded DCT2 (row k of an N-point matrix satisfies F[k][N-1-n] =
    // (-1)^k F[k][n], as the encoder's butterflies build it): for the first half of the outputs
    // n they keep column n with the even-k entries first and the odd-k entries after them
    // (Fw^T, Fh^T in even/odd order), and each sum over k splits into an even part E and an odd
    // part O with out[n] = E + O and out[N-1-n] = E - O.
    // A CTA takes its tiles from the queue in class order, so consecutive tiles mostly share
    // the class: the tables of the previous tile are kept (the layout of a class is fixed
    // within a launch).
    const int cls = (LW - 2) * 5 + (LH - 2);
    const bool tables_in_place = S.tables == cls;
    for (int i = tid; i < (tables_in_place ? 0 : kw * w); i += LAT_THREADS) {
        const int u = i >> lw, x = i & (w - 1);
        const u8 v = (u8)P.fold[LW][u * w + x];
        ((u8 *)fw)[u * L.fw_ws * 4 + x] = v;        // Fw[u][x]
        if (x < (w >> 1)) ((u8 *)fwt)[x * L.fwt_ws * 4 + lat_eo(u, kw)] = v;
    }
    for (int i = tid; i < (tables_in_place ? 0 : kh * h); i += LAT_THREADS) {
        const int v = i >> lh, y = i & (h - 1);
        const u8 c = (u8)P.fold[LH][v * h + y];
        ((u8 *)fh)[v * L.fh_ws * 4 + y] = c;        // Fh[v][y]
        if (y < (h >> 1)) ((u8 *)fht)[y * L.fht_ws * 4 + lat_eo(v, kh)] = c;
    }
    u16 *s_scan = (u16 *)(sm + L.o_scan);
    for (int i = tid; i < (tables_in_place ? 0 : kw * kh); i += LAT_THREADS)
        s_scan[i] = P.scanpos[LW][LH][(i >> lkw) * w + (i & (kw - 1))];
    if (tid < Gv) s_cu[tid] = perm[cu0 + tid];
    for (int j = tid; j < J; j += LAT_THREADS) {
        const int g = j / MCv, mi = m0 + (j - g * MCv);
        s_mode[j] = P.modes ? P.modes[(size_t)perm[cu0 + g] * P.n_modes + mi] : (u8)mi;
        s_satd[j] = 0; s_flag[j] = 0; s_nz[j] = 0; s_sum[j] = 0; s_hash[j] = 0; s_ssd[j] = 0; s_last[j] = -1;
    }
    __syncthreads(); LAT_STAGE(0);
    if (tid == 0) S.tables = cls;   // every thread has read S.tables above

    // ---- per CU: org block, neighbours (com_intra_get_nbr with every in-picture sample
    // reconstructed)
    // four samples per thread (CU x positions are multiples of 4): one word load where the
    // picture and its pitch are word-aligned
    for (int i = tid; i < Gv * (N >> 2); i += LAT_THREADS) {
        const int g = i >> (lN - 2), p = (i & ((N >> 2) - 1)) << 2;
        const LatCu cu = P.cus[s_cu[g]];
        const pel *src = P.org + (long long)(cu.y + (p >> lw)) * P.i_org + cu.x + (p & (w - 1));
        u32 v;
        if (P.org_words) v = __ldg(reinterpret_cast<const u32 *>(src));
        else v = (u32)src[0] | (u32)src[1] << 8 | (u32)src[2] << 16 | (u32)src[3] << 24;
        *reinterpret_cast<u32 *>(cub + g * L.cu_bytes + L.c_org + (p >> lw) * L.ps + (p & (w - 1))) = v;
    }
    const int range = max(w, h) * 4 + 4;
    for (int i = tid; i < Gv * range; i += LAT_THREADS) {
        const int g = i / range, k = i - g * range;
        const LatCu cu = P.cus[s_cu[g]];
        const int x = cu.x, y = cu.y;
        const int avail = (y > 0 ? 1 : 0) | (x > 0 ? 2 : 0);
        const int up_cnt = (y > 0) ? min(w >> 2, max(0, (P.W - (x + w)) >> 2)) : 0;
        const int le_cnt = (x > 0) ? min(h >> 2, max(0, (P.H - (y + h)) >> 2)) : 0;
        pel *nbm = cub + g * L.cu_bytes + L.c_nb + 288;
        nbm[1 + k] = (avail & 1) ? P.rec[(long long)(y - 1) * P.i_rec + x + min(k, w + 4 * up_cnt - 1)] : (pel)128;
        nbm[-1 - k] = (avail & 2) ? P.rec[(long long)(y + min(k, h + 4 * le_cnt - 1)) * P.i_rec + x - 1] : (pel)128;
        if (k == 0) {
            pel c;
            if (x > 0 && y > 0) c = P.rec[(long long)(y - 1) * P.i_rec + x - 1];
            else if (y > 0) c = P.rec[(long long)(y - 1) * P.i_rec + x];
            else if (x > 0) c = P.rec[(long long)y * P.i_rec + x - 1];
            else c = 128;
            nbm[0] = c;
        }
    }
    __syncthreads(); LAT_STAGE(1);
    if (tid < Gv) {
        const LatCu cu = P.cus[s_cu[tid]];
        const int avail = (cu.y > 0 ? 1 : 0) | (cu.x > 0 ? 2 : 0) | ((cu.x > 0 && cu.y > 0) ? 4 : 0);
        ipred_block_setup(cub + tid * L.cu_bytes + L.c_nb + 288, w, h, avail, 8, sB[tid]);
    }
    // org part of the forward row pass: Torg[y][u] = sum_x Fw[u][x] org[y][x] (no transform
    // stage runs when no QP is asked: SATD records only)
    for (int i = tid; i < (P.n_qp > 0 ? Gv * kw * h : 0); i += LAT_THREADS) {
        const int u = i & (kw - 1), y = (i >> lkw) & (h - 1), g = i >> (lkw + lh);
        const u8 *c = cub + g * L.cu_bytes;
        const u32 *o = (const u32 *)(c + L.c_org + y * L.ps), *f = fw + u * L.fw_ws;
        int acc = 0;
        #pragma unroll
        for (int k = 0; k < (w >> 2); k++) acc = dp4a_us(o[k], f[k], acc);
        ((int *)(c + L.c_torg))[y * kw + u] = acc;
    }
    __syncthreads(); LAT_STAGE(2);

    // job j -> (CU g, mode m): j = g * MCv + (m - m0)
#define JG(j) ((int)(((u32)(j) * mc_magic) >> 16))
#define JPRED(j) (jobb + (j) * L.job_bytes + L.j_pred)
#define JT(j) ((s16 *)(jobb + (j) * L.job_bytes + L.j_t))
#define JC(j) ((s16 *)(jobb + (j) * L.job_bytes + L.j_c))
#define JDQT(j) ((s16 *)(jobb + (j) * L.job_bytes + L.j_dqt))
#define JT2(j) ((s16 *)(jobb + (j) * L.job_bytes + L.j_t2))
#define CORG(g) (cub + (g) * L.cu_bytes + L.c_org)

    // ---- prediction
    for (int i = tid; i < (J << lN); i += LAT_THREADS) {
        const int j = i >> lN, p = i & (N - 1);
        const int g = JG(j), m = s_mode[j];
        const int x = p & (w - 1), y = p >> lw;
        JPRED(j)[y * L.ps + x] = (pel)ipred_sample<W_, H_>(cub + g * L.cu_bytes + L.c_nb + 288, sB[g], m, P.ipf, x, y);
    }
    __syncthreads(); LAT_STAGE(3);

    // ---- SATD (com_had tiling) and forward row pass T[u][y] = (Torg - sum_x Fw pred + rnd) >> sh1
    {
        constexpr int TW = lat_tw(1 << LW, 1 << LH), TH = lat_th(1 << LW, 1 << LH);
        constexpr int lnt = LW + LH - (TW == 16 ? 4 : TW == 8 ? 3 : 2) - (TH == 16 ? 4 : TH == 8 ? 3 : 2);
        lat_satd_tiles<TW, TH>(J << lnt, lnt, (1 << LW) / TW, cub, L.cu_bytes, L.c_org, jobb, L.job_bytes, L.j_pred, L.ps,
                               MCv, s_satd, P.sq32, P.sq128, P.k32, P.k128);
    }
    {
        const int sh1 = lw - 2, rnd1 = sh1 > 0 ? 1 << (sh1 - 1) : 0;
        for (int i = tid; i < (P.n_qp > 0 ? J * NYC * KW_ : 0); i += LAT_THREADS) {
            const int u = i & (KW_ - 1), yc = (i >> LKW_) % NYC, j = i / (KW_ * NYC);
            u32 f[W_ / 4];
#pragma unroll
            for (int k = 0; k < W_ / 4; k++) f[k] = fw[u * L.fw_ws + k];
            const int *torg = (const int *)(cub + JG(j) * L.cu_bytes + L.c_torg);
            s16 *T = JT(j);
#pragma unroll
            for (int r = 0; r < RY; r++) {
                const int y = yc * RY + r;
                u32 pw[W_ / 4];
                lat_row<W_ / 4>(JPRED(j) + y * L.ps, pw);
                int sacc = 0;
#pragma unroll
                for (int k = 0; k < W_ / 4; k++) sacc = dp4a_us(pw[k], f[k], sacc);
                T[u * L.ts + y] = (s16)((torg[y * KW_ + u] - sacc + rnd1) >> sh1);
            }
        }
    }
    __syncthreads(); LAT_STAGE(4);

    // quantisation parameters per QP
    const int odd = lN & 1, log2_size = lN >> 1;
    const int q_bits = 14 + (15 - 8 - log2_size);
    const int offset = (P.is_intra ? 201 : 153) << (q_bits - 9);
    const u32 qadd = 1u << (q_bits - 1);

    // ---- forward column pass C[v][u] = (sum_y Fh[v][y] T[u][y] + rnd2) >> sh2, and the
    // quant_check flags of every QP (bit q: some |C| above that QP's all-zero threshold)
    {
        int nz_thr[LAT_MAX_QP];
#pragma unroll
        for (int q = 0; q < LAT_MAX_QP; q++) {
            const int qp = P.qp[q];
            const int q_value = ((int)kQScale[qp] * (odd ? 181 : 1) + (odd ? 64 : 0)) >> (odd ? 7 : 0);
            nz_thr[q] = ((((1 << q_bits) - offset) << 10) / q_value - 1) >> 10;
        }
        const int sh2 = lh + 5, rnd2 = 1 << (sh2 - 1);
        for (int i = tid; i < (P.n_qp > 0 ? J * NUC * KH_ : 0); i += LAT_THREADS) {
            const int v = i & (KH_ - 1), uc = (i >> LKH_) % NUC, j = i / (KH_ * NUC);
            u32 f[H_ / 4];
#pragma unroll
            for (int k = 0; k < H_ / 4; k++) f[k] = fh[v * L.fh_ws + k];
            u32 fl = 0;
#pragma unroll
            for (int r = 0; r < RU; r++) {
                const int u = uc * RU + r;
                u32 tw[H_ / 2];
                lat_row<H_ / 2>(JT(j) + u * L.ts, tw);
                int acc = 0;
#pragma unroll
                for (int k = 0; k < H_ / 4; k++) {
                    acc = dp2a_lo(tw[2 * k], f[k], acc);
                    acc = dp2a_hi(tw[2 * k + 1], f[k], acc);
                }
                const int c = (acc + rnd2) >> sh2;
                JC(j)[v * L.cs + u] = (s16)c;
                const int a = c < 0 ? -(int)(s16)c : (int)(s16)c;
#pragma unroll
                for (int q = 0; q < LAT_MAX_QP; q++)
                    if (q < P.n_qp && a > nz_thr[q]) fl |= 1u << q;
            }
            if (fl) atomicOr(&s_flag[j], fl);
        }
    }
    __syncthreads(); LAT_STAGE(5);
    for (int j = tid; j < J; j += LAT_THREADS)
        P.satd_out[(size_t)s_cu[JG(j)] * 33 + s_mode[j]] = s_satd[j];

    for (int q = 0; q < P.n_qp; q++) {
        const int qp = P.qp[q];
        const u32 q_value = (u32)(((int)kQScale[qp] * (odd ? 181 : 1) + (odd ? 64 : 0)) >> (odd ? 7 : 0));
        const int thr = ((1 << (q_bits - 1)) - 1) / (int)q_value + 1;
        const int dq_scale = (int)kDqScale[qp];
        const int dq_shift = (int)kDqShift[qp] - (15 - 8 - log2_size) + 1;
        const int dq_off = dq_shift == 0 ? 0 : 1 << (dq_shift - 1);
        // first-pass levels, statistics, dequantisation (stored transposed, DQ^T[u][v], each row
        // in even/odd order of v).  The
        // level (|c| q_value + 2^(q_bits-1)) >> q_bits is exact in 32 bits: |c| <= 2^15 and
        // q_value < 2^15.
        // A task is one coefficient row v of a job over RU columns (lanes take consecutive v):
        // the statistics are summed in registers and reduced once per task.
        {
            constexpr int TPJ = KH_ * NUC, SEG = TPJ < 32 ? TPJ : 32;
            for (int base = wbase; base < J * TPJ; base += LAT_THREADS) {
                const int i = base + lane;
                const bool act = i < J * TPJ;
                const int ii = act ? i : base;
                const int v = ii & (KH_ - 1), uc = (ii >> LKH_) % NUC, j = ii / TPJ;
                const bool coded = act && (s_flag[j] >> q & 1);
                u32 nz = 0, sa = 0, hs = 0;
                int last = -1;
#pragma unroll
                for (int r = 0; r < RU; r++) {
                    // branch-free: a zero level adds nothing to the statistics and dequantises
                    // to zero ((0 * scale + 2^(shift-1)) >> shift)
                    const int u = uc * RU + r;
                    const int c = coded ? (int)JC(j)[v * L.cs + u] : 0;
                    const int a = c < 0 ? -c : c;
                    const int l = a >= thr ? (int)(s16)(((u32)a * q_value + qadd) >> q_bits) : 0;
                    const int lev = c < 0 ? -l : l;
                    nz += lev != 0 ? 1u : 0u;
                    sa += (u32)(lev < 0 ? -lev : lev);
                    hs += (u32)lev * lat_pos_weight((u32)(v * w + u));
                    if (lev) last = max(last, (int)s_scan[v * KW_ + u]);
                    int d = (lev * dq_scale + dq_off) >> dq_shift;
                    d = min(32767, max(-32768, d));
                    const int dq = odd ? (d * 181 + 128) >> 8 : d;
                    if (act) JDQT(j)[u * L.ds + lat_eo(v, KH_)] = (s16)dq;
                }
                if (__any_sync(0xFFFFFFFFu, nz != 0)) {
                    nz = lat_seg_sum<SEG>(nz, lane);
                    sa = lat_seg_sum<SEG>(sa, lane);
                    hs = lat_seg_sum<SEG>(hs, lane);
                    last = lat_seg_max<SEG>(last, lane);
                    if (act && (lane & (SEG - 1)) == 0 && nz) {
                        atomicAdd(&s_nz[j], nz);
                        atomicAdd(&s_sum[j], sa);
                        atomicAdd(&s_hash[j], hs);
                        atomicMax(&s_last[j], last);
                    }
                }
            }
        }
        __syncthreads(); LAT_STAGE(6);
        // inverse column pass T2[y][u] = clip16((sum_v Fh[v][y] DQ[v][u] + 16) >> 5), only
        // for jobs with coded levels; a task forms rows y and H-1-y from the even-v and odd-v
        // sums over CU columns u (T2 rows are stored in even/odd order of u).  Tiles with few
        // jobs take CU/2 columns per task so that the CTA's threads still have a task each.
        auto inv_col = [&](auto cu_tag) {
            constexpr int CU = decltype(cu_tag)::value, NCU = KW_ / CU;
            for (int i = tid; i < J * NCU * (H_ / 2); i += LAT_THREADS) {
                const int y = i & (H_ / 2 - 1), uc = (i >> (LH - 1)) % NCU, j = i / ((H_ / 2) * NCU);
                if (!s_nz[j]) continue;
                u32 f[KH_ / 4];
#pragma unroll
                for (int k = 0; k < KH_ / 4; k++) f[k] = fht[y * L.fht_ws + k];
#pragma unroll 2   // two columns per step: a full unroll spills at the 64-register limit
                for (int r = 0; r < CU; r++) {
                    const int u = uc * CU + r;
                    u32 dw[KH_ / 2];
                    lat_row<KH_ / 2>(JDQT(j) + u * L.ds, dw);
                    int e = 0, o = 0;
                    lat_eo_sums<KH_>(dw, f, e, o);
                    s16 *t2 = JT2(j) + lat_eo(u, KW_);
                    t2[y * L.t2s] = (s16)min(32767, max(-32768, (e + o + 16) >> 5));
                    t2[(H_ - 1 - y) * L.t2s] = (s16)min(32767, max(-32768, (e - o + 16) >> 5));
                }
            }
        };
        if (RU > 2 && J * NUC * (H_ / 2) < LAT_THREADS) inv_col(std::integral_constant<int, (RU > 2 ? RU / 2 : RU)>{});
        else inv_col(std::integral_constant<int, RU>{});
        __syncthreads(); LAT_STAGE(7);
        // inverse row pass, reconstruction, SSD: a task is the column pair x, W-1-x over CY
        // rows (the even-u and odd-u sums of the T2 row give both); CY = RY / 2 for tiles with
        // few jobs
        auto inv_row = [&](auto cy_tag) {
            constexpr int CY = decltype(cy_tag)::value, NCY = H_ / CY;
            constexpr int TPJ = (W_ / 2) * NCY, SEG = TPJ < 32 ? TPJ : 32;
            for (int base = wbase; base < J * TPJ; base += LAT_THREADS) {
                const int i = base + lane;
                const bool act = i < J * TPJ;
                const int ii = act ? i : base;
                const int x = ii & (W_ / 2 - 1), yc = (ii >> (LW - 1)) % NCY, j = ii / TPJ;
                const bool coded = s_nz[j] != 0;
                u32 f[KW_ / 4];
#pragma unroll
                for (int k = 0; k < KW_ / 4; k++) f[k] = fwt[x * L.fwt_ws + k];
                const pel *po = CORG(JG(j));
                const pel *pp = JPRED(j);
                u32 e = 0;
#pragma unroll
                for (int r = 0; r < CY; r++) {
                    const int y = yc * CY + r;
                    int rv0 = pp[y * L.ps + x], rv1 = pp[y * L.ps + W_ - 1 - x];
                    if (coded) {
                        u32 tw[KW_ / 2];
                        lat_row<KW_ / 2>(JT2(j) + y * L.t2s, tw);
                        int se = 0, so = 0;
                        lat_eo_sums<KW_>(tw, f, se, so);
                        const int res0 = min(255, max(-256, (se + so + 2048) >> 12));
                        const int res1 = min(255, max(-256, (se - so + 2048) >> 12));
                        rv0 = min(255, max(0, rv0 + res0));
                        rv1 = min(255, max(0, rv1 + res1));
                    }
                    const int d0 = (int)po[y * L.ps + x] - rv0, d1 = (int)po[y * L.ps + W_ - 1 - x] - rv1;
                    e += (u32)(d0 * d0) + (u32)(d1 * d1);
                }
                if (!act) e = 0;
                e = lat_seg_sum<SEG>(e, lane);
                if (act && (lane & (SEG - 1)) == 0) atomicAdd(&s_ssd[j], e);
            }
        };
        if (RY > 2 && J * (W_ / 2) * NYC < LAT_THREADS) inv_row(std::integral_constant<int, (RY > 2 ? RY / 2 : RY)>{});
        else inv_row(std::integral_constant<int, RY>{});
        __syncthreads(); LAT_STAGE(8);
        for (int j = tid; j < J; j += LAT_THREADS) {
            const int g = JG(j);
            LatQ o;
            o.ssd = s_ssd[j];
            o.coef_hash = s_hash[j];
            o.num_nz = (u16)s_nz[j];
            o.last_nz = (s16)s_last[j];
            o.sum_abs = s_sum[j];
            P.q_out[((size_t)s_cu[g] * 33 + s_mode[j]) * P.n_qp + q] = o;
            s_ssd[j] = 0; s_hash[j] = 0; s_nz[j] = 0; s_last[j] = -1; s_sum[j] = 0;
        }
        __syncthreads(); LAT_STAGE(9);
    }
#undef JG
#undef JPRED
#undef JT
#undef JC
#undef JDQT
#undef JT2
#undef CORG
}

// the size classes in launch order, largest CUs first (their tiles are the longest): rank r
// takes class (log2 w - 2) * 5 + (log2 h - 2) = lat_order(r)
__host__ __device__ constexpr int lat_order(int r) { return (4 - r / 5) * 5 + (4 - r % 5); }

}  // namespace uc
