// Batched intra lattice: for every CU of a frame's QT/BT lattice and every luma intra mode,
// prediction -> SATD -> residual -> forward DCT2 -> (per QP) quantisation -> dequantisation ->
// inverse DCT2 -> reconstruction -> SSD, bit-exact with the encoder's functions
// (com_intra_get_nbr src/com_ipred.c:40, com_intra_pred :733, calc_satd_intra src/util.c:200,
// trans_dct2 src/transform.c:253-412, quant_check / quant_rdoq src/com_itdq.c:910-954 with the
// rdoq_quant_block parameters src/quant.c:196-231, com_dquant src/com_itdq.c:807,
// itrans_dct2 :264-423, com_recon src/com_util.c:3107).
//
// One CTA per CU.  All per-mode data live in shared memory; the 33 modes are processed in
// chunks of as many modes as fit, and every stage is a flat loop over (mode, element) pairs so
// small CUs keep all threads busy.  Transforms are matrix products with the folded DCT2
// matrices (identical results to the encoder's partial butterflies).
#include "common.cuh"
#include "intra.cuh"
#include "tables.h"
#include "uavs3e_cuda_internal.h"
#include "../../include/uavs3e_cuda.h"

namespace uc {

__device__ __constant__ static const u16 kQScale[80] = {
    16302, 15024, 13777, 12634, 11626, 10624, 9742, 8958, 8192, 7512, 6889, 6305, 5793, 5303, 4878, 4467,
    4091, 3756, 3444, 3161, 2894, 2654, 2435, 2235, 2048, 1878, 1722, 1579, 1449, 1329, 1218, 1117,
    1024, 939, 861, 790, 724, 664, 609, 558, 512, 470, 430, 395, 362, 332, 304, 279,
    256, 235, 215, 197, 181, 166, 152, 140, 128, 116, 108, 99, 91, 83, 76, 69,
    64, 59, 54, 49, 45, 41, 38, 35, 32, 30, 27, 25, 23, 21, 19, 18,
};
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

__device__ __forceinline__ u32 fmix32(u32 h)
{
    h ^= h >> 16; h *= 0x85ebca6bu; h ^= h >> 13; h *= 0xc2b2ae35u; h ^= h >> 16;
    return h;
}

struct LatCu { s16 x, y; u8 w, h; u16 pad; };
struct LatQ { u32 ssd; u32 coef_hash; u16 num_nz; s16 last_nz; u32 sum_abs; };

constexpr int LAT_THREADS = 256;
constexpr int LAT_MODE_BUDGET = 56 * 1024;   // shared bytes for per-mode buffers
constexpr int LAT_MAX_QP = 4;

struct LatParams {
    const pel *org; int i_org;
    const pel *rec; int i_rec;
    int W, H;
    const LatCu *cus; int n_cus;
    int ipf, n_qp, is_intra;
    int qp[LAT_MAX_QP];
    u32 *satd_out; LatQ *q_out;
    DevTables tab;
    double sq32, sq128;
};

__host__ __device__ __forceinline__ int lat_mode_bytes(int w, int h)
{
    int kw = w < 32 ? w : 32, kh = h < 32 ? h : 32;
    int b = w * h + 2 * (kw * h) + 2 * (kw * kh) + 2 * (kw * kh) + 2 * (h * kw);
    return (b + 15) & ~15;
}

__host__ __device__ __forceinline__ int lat_modes_per_chunk(int w, int h)
{
    int m = LAT_MODE_BUDGET / lat_mode_bytes(w, h);
    return m < 1 ? 1 : (m > 33 ? 33 : m);
}

__global__ void __launch_bounds__(LAT_THREADS) k_intra_lattice(LatParams P)
{
    extern __shared__ __align__(16) u8 sm[];
    __shared__ IpredBlock sB;
    __shared__ u32 s_satd[33];
    __shared__ u32 s_flag[33], s_nz[33], s_sum[33], s_hash[33], s_ssd[33];
    __shared__ int s_last[33];

    const LatCu cu = P.cus[blockIdx.x];
    const int x = cu.x, y = cu.y, w = cu.w, h = cu.h;
    // a CU outside the supported set (power-of-two sides 4..64 inside the picture) is skipped
    // with zeroed outputs
    if (w < 4 || w > 64 || h < 4 || h > 64 || (w & (w - 1)) || (h & (h - 1)) || x < 0 || y < 0 ||
        x + w > P.W || y + h > P.H) {
        for (int i = threadIdx.x; i < 33; i += blockDim.x) {
            P.satd_out[(size_t)blockIdx.x * 33 + i] = 0;
            for (int q = 0; q < P.n_qp; q++) P.q_out[((size_t)blockIdx.x * 33 + i) * P.n_qp + q] = LatQ{};
        }
        return;
    }
    const int lw = ilog2d(w), lh = ilog2d(h), lwh = lw + lh, wh = 1 << lwh;
    const int kw = min(w, 32), kh = min(h, 32), lkw = ilog2d(kw), lkh = ilog2d(kh);
    const int tid = threadIdx.x;
    const int MC = lat_modes_per_chunk(w, h);

    // ---- shared memory carve-out
    pel *s_org = sm;                                   // wh
    pel *s_nb = s_org + ((wh + 15) & ~15);             // 576 (+pad)
    s8 *s_fw = (s8 *)(s_nb + 592);                     // kw x w
    s8 *s_fh = s_fw + ((kw * w + 15) & ~15);           // kh x h
    u8 *s_modes = (u8 *)(s_fh + ((kh * h + 15) & ~15));
    const int mbytes = lat_mode_bytes(w, h);

    // ---- neighbours (com_intra_get_nbr with every in-picture sample reconstructed)
    const int avail = (y > 0 ? 1 : 0) | (x > 0 ? 2 : 0) | ((x > 0 && y > 0) ? 4 : 0);
    const int range = max(w, h) * 4 + 4;
    const int up_cnt = (y > 0) ? min(w >> 2, max(0, (P.W - (x + w)) >> 2)) : 0;
    const int le_cnt = (x > 0) ? min(h >> 2, max(0, (P.H - (y + h)) >> 2)) : 0;
    pel *nbm = s_nb + 288;
    for (int k = tid; k < range; k += LAT_THREADS) {
        nbm[1 + k] = (avail & 1) ? P.rec[(long long)(y - 1) * P.i_rec + x + min(k, w + 4 * up_cnt - 1)] : (pel)128;
        nbm[-1 - k] = (avail & 2) ? P.rec[(long long)(y + min(k, h + 4 * le_cnt - 1)) * P.i_rec + x - 1] : (pel)128;
    }
    if (tid == 0) {
        pel c;
        if (avail & 4) c = P.rec[(long long)(y - 1) * P.i_rec + x - 1];
        else if (avail & 1) c = P.rec[(long long)(y - 1) * P.i_rec + x];
        else if (avail & 2) c = P.rec[(long long)y * P.i_rec + x - 1];
        else c = 128;
        nbm[0] = c;
    }
    for (int p = tid; p < wh; p += LAT_THREADS) s_org[p] = P.org[(long long)(y + (p >> lw)) * P.i_org + x + (p & (w - 1))];
    for (int p = tid; p < kw * w; p += LAT_THREADS) s_fw[p] = P.tab.fold[lw][p];
    for (int p = tid; p < kh * h; p += LAT_THREADS) s_fh[p] = P.tab.fold[lh][p];
    __syncthreads();
    if (tid == 0) ipred_block_setup(nbm, w, h, avail, 8, sB);
    __syncthreads();
    const IpredBlock B = sB;

    int tw, th;
    had_tile_shape(w, h, &tw, &th);
    const int ltw = ilog2d(tw), lth = ilog2d(th);
    const int lnt = lwh - ltw - lth;                  // log2 tiles per block
    const int sh1 = lw - 2, rnd1 = sh1 > 0 ? 1 << (sh1 - 1) : 0;
    const int sh2 = lh + 5, rnd2 = 1 << (sh2 - 1);
    const u16 *scanpos = P.tab.scanpos[lw][lh];

    for (int m0 = 0; m0 < 33; m0 += MC) {
        const int nm = min(MC, 33 - m0);
        // per-mode buffer views
#define PRED(m) (s_modes + (m) * mbytes)
#define TBUF(m) ((s16 *)(PRED(m) + wh))
#define COEF(m) (TBUF(m) + kw * h)
#define DQ(m) (COEF(m) + kw * kh)
#define T2(m) (DQ(m) + kw * kh)
        // prediction
        for (int idx = tid; idx < (nm << lwh); idx += LAT_THREADS) {
            int m = idx >> lwh, p = idx & (wh - 1);
            PRED(m)[p] = (pel)ipred_sample(nbm, B, m0 + m, P.ipf, p & (w - 1), p >> lw);
        }
        if (tid < nm) s_satd[tid] = 0;
        __syncthreads();
        // SATD (com_had tiling) and forward row pass
        for (int idx = tid; idx < (nm << lnt); idx += LAT_THREADS) {
            int m = idx >> lnt, t = idx & ((1 << lnt) - 1);
            int ntx = w >> ltw;
            int ox = (t % ntx) << ltw, oy = (t / ntx) << lth;
            u32 v = satd_tile(tw, th, s_org + oy * w + ox, w, PRED(m) + oy * w + ox, w, P.sq32, P.sq128);
            atomicAdd(&s_satd[m], v);
        }
        for (int idx = tid; idx < nm * kw * h; idx += LAT_THREADS) {
            int m = idx / (kw * h), r = idx - m * (kw * h);
            int u = r >> lh, yy = r & (h - 1);
            const pel *o = s_org + yy * w, *pr = PRED(m) + yy * w;
            const s8 *f = s_fw + u * w;
            int acc = 0;
            for (int xx = 0; xx < w; xx++) acc += f[xx] * ((int)o[xx] - (int)pr[xx]);
            TBUF(m)[u * h + yy] = (s16)((acc + rnd1) >> sh1);
        }
        __syncthreads();
        if (tid < nm) P.satd_out[(size_t)blockIdx.x * 33 + m0 + tid] = s_satd[tid];
        // forward column pass
        for (int idx = tid; idx < nm * kw * kh; idx += LAT_THREADS) {
            int m = idx >> (lkw + lkh), r = idx & ((kw * kh) - 1);
            int v = r >> lkw, u = r & (kw - 1);
            const s16 *t = TBUF(m) + u * h;
            const s8 *f = s_fh + v * h;
            int acc = 0;
            for (int yy = 0; yy < h; yy++) acc += f[yy] * t[yy];
            COEF(m)[v * kw + u] = (s16)((acc + rnd2) >> sh2);
        }
        __syncthreads();

        for (int q = 0; q < P.n_qp; q++) {
            const int qp = P.qp[q];
            const int odd = lwh & 1;
            const int log2_size = lwh >> 1;
            const int q_bits = 14 + (15 - 8 - log2_size);
            const int q_value = ((int)kQScale[qp] * (odd ? 181 : 1) + (odd ? 64 : 0)) >> (odd ? 7 : 0);
            const int offset = (P.is_intra ? 201 : 153) << (q_bits - 9);
            const int nz_thr = ((((1 << q_bits) - offset) << 10) / q_value - 1) >> 10;
            const int thr = ((1 << (q_bits - 1)) - 1) / q_value + 1;
            const u32 qadd = 1u << (q_bits - 1);
            const int dq_scale = (int)kDqScale[qp];
            const int dq_shift = (int)kDqShift[qp] - (15 - 8 - log2_size) + 1;
            const int dq_off = dq_shift == 0 ? 0 : 1 << (dq_shift - 1);
            if (tid < nm) { s_flag[tid] = 0; s_nz[tid] = 0; s_sum[tid] = 0; s_hash[tid] = 0; s_ssd[tid] = 0; s_last[tid] = -1; }
            __syncthreads();
            // quant_check: any coefficient above the all-zero threshold
            for (int idx = tid; idx < nm * kw * kh; idx += LAT_THREADS) {
                int m = idx >> (lkw + lkh), r = idx & ((kw * kh) - 1);
                int c = COEF(m)[r];
                if (c > nz_thr || c < -nz_thr) s_flag[m] = 1;
            }
            __syncthreads();
            // first-pass levels, statistics, dequantisation
            for (int idx = tid; idx < nm * kw * kh; idx += LAT_THREADS) {
                int m = idx >> (lkw + lkh), r = idx & ((kw * kh) - 1);
                int lev = 0;
                if (s_flag[m]) {
                    int c = COEF(m)[r];
                    int a = c < 0 ? -c : c;
                    if (a >= thr) {
                        u32 ld = (u32)a * (u32)q_value;
                        int l = (int)(s16)(u32)(((u64)ld + qadd) >> q_bits);
                        lev = c < 0 ? -l : l;
                    }
                }
                int dq = 0;
                if (lev) {
                    int v = r >> lkw, u = r & (kw - 1);
                    int pos = v * w + u;
                    atomicAdd(&s_nz[m], 1u);
                    atomicAdd(&s_sum[m], (u32)(lev < 0 ? -lev : lev));
                    atomicAdd(&s_hash[m], fmix32(((u32)pos << 16) | (u16)(s16)lev));
                    atomicMax(&s_last[m], (int)scanpos[pos]);
                    int d = (lev * dq_scale + dq_off) >> dq_shift;
                    d = min(32767, max(-32768, d));
                    dq = odd ? (d * 181 + 128) >> 8 : d;
                }
                DQ(m)[r] = (s16)dq;
            }
            __syncthreads();
            // inverse column pass (only modes with coded levels)
            for (int idx = tid; idx < nm * kw * h; idx += LAT_THREADS) {
                int m = idx / (kw * h), r = idx - m * (kw * h);
                if (!s_nz[m]) continue;
                int yy = r >> lkw, u = r & (kw - 1);
                const s16 *d = DQ(m) + u;
                int acc = 0;
                for (int v = 0; v < kh; v++) acc += s_fh[v * h + yy] * d[v * kw];
                T2(m)[yy * kw + u] = (s16)min(32767, max(-32768, (acc + 16) >> 5));
            }
            __syncthreads();
            // inverse row pass, reconstruction, SSD
            for (int idx = tid; idx < (nm << lwh); idx += LAT_THREADS) {
                int m = idx >> lwh, p = idx & (wh - 1);
                int yy = p >> lw, xx = p & (w - 1);
                int rv = PRED(m)[p];
                if (s_nz[m]) {
                    const s16 *t = T2(m) + yy * kw;
                    int acc = 0;
                    for (int u = 0; u < kw; u++) acc += s_fw[u * w + xx] * t[u];
                    int r = min(255, max(-256, (acc + 2048) >> 12));
                    rv = min(255, max(0, rv + r));
                }
                int d = (int)s_org[p] - rv;
                atomicAdd(&s_ssd[m], (u32)(d * d));
            }
            __syncthreads();
            if (tid < nm) {
                LatQ o;
                o.ssd = s_ssd[tid];
                o.coef_hash = s_hash[tid];
                o.num_nz = (u16)s_nz[tid];
                o.last_nz = (s16)s_last[tid];
                o.sum_abs = s_sum[tid];
                P.q_out[((size_t)blockIdx.x * 33 + m0 + tid) * P.n_qp + q] = o;
            }
            __syncthreads();
        }
#undef PRED
#undef TBUF
#undef COEF
#undef DQ
#undef T2
    }
}

size_t lattice_smem_bytes(int w, int h)
{
    int kw = w < 32 ? w : 32, kh = h < 32 ? h : 32;
    size_t fixed = ((w * h + 15) & ~15) + 592 + ((kw * w + 15) & ~15) + ((kh * h + 15) & ~15);
    return fixed + (size_t)lat_modes_per_chunk(w, h) * lat_mode_bytes(w, h);
}

int launch_intra_lattice(const pel *org, int i_org, const pel *rec, int i_rec, int W, int H, const LatCu *cus,
                         int n_cus, int ipf, const int *qps, int n_qp, int is_intra, u32 *satd_out, LatQ *q_out,
                         cudaStream_t st)
{
    int dev = 0;
    UC_CHECK(cudaGetDevice(&dev));
    const DevTables *tab = device_tables(dev);
    if (!tab) return set_status(UC_ERR_MEMORY, "intra_lattice: table upload failed");
    if (n_qp < 1 || n_qp > LAT_MAX_QP || n_cus < 0) return set_status(UC_ERR_ARG, "intra_lattice: bad qp count");
    if (n_cus == 0) return UC_OK;
    LatParams P;
    P.org = org; P.i_org = i_org; P.rec = rec; P.i_rec = i_rec; P.W = W; P.H = H;
    P.cus = cus; P.n_cus = n_cus; P.ipf = ipf; P.n_qp = n_qp; P.is_intra = is_intra;
    for (int i = 0; i < LAT_MAX_QP; i++) P.qp[i] = i < n_qp ? qps[i] : 0;
    for (int i = 0; i < n_qp; i++)
        if (qps[i] < 0 || qps[i] > 63) return set_status(UC_ERR_ARG, "intra_lattice: qp out of range");
    P.satd_out = satd_out; P.q_out = q_out; P.tab = *tab;
    P.sq32 = sqrt(32.0); P.sq128 = sqrt(128.0);
    size_t smem = 0;
    for (int lw = 2; lw <= 6; lw++)
        for (int lh = 2; lh <= 6; lh++) smem = std::max(smem, lattice_smem_bytes(1 << lw, 1 << lh));
    static bool attr[64];
    if (dev < 64 && !attr[dev]) {
        UC_CHECK(cudaFuncSetAttribute(k_intra_lattice, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr[dev] = true;
    }
    prof_begin(PROF_LATTICE, st);
    k_intra_lattice<<<n_cus, LAT_THREADS, smem, st>>>(P);
    UC_CHECK(cudaGetLastError());
    count_launch(1);
    prof_end(PROF_LATTICE, st);
    return UC_OK;
}

}  // namespace uc

using namespace uc;

static_assert(sizeof(LatCu) == sizeof(uavs3e_cuda_cu_t), "cu record layout");
static_assert(sizeof(LatQ) == sizeof(uavs3e_cuda_lat_q_t), "lattice record layout");

extern "C" {

UAVS3E_CUDA_API int uavs3e_cuda_lattice_cus(int width, int height, uavs3e_cuda_cu_t *out, int cap)
{
    // the 23 shapes w, h in {4..64} with aspect ratio <= 8 (largest first), every position
    // aligned to the shape inside the picture
    int n = 0;
    for (int lw = 6; lw >= 2; lw--)
        for (int lh = 6; lh >= 2; lh--) {
            if (lw - lh > 3 || lh - lw > 3) continue;
            int w = 1 << lw, h = 1 << lh;
            for (int y = 0; y + h <= height; y += h)
                for (int x = 0; x + w <= width; x += w) {
                    if (out && n < cap) { out[n].x = (int16_t)x; out[n].y = (int16_t)y; out[n].w = (uint8_t)w; out[n].h = (uint8_t)h; out[n].pad = 0; }
                    n++;
                }
        }
    return n;
}

UAVS3E_CUDA_API int uavs3e_cuda_intra_lattice_device(const uint8_t *d_org, int i_org, const uint8_t *d_rec, int i_rec,
                                                     int width, int height, const uavs3e_cuda_cu_t *d_cus, int n_cus,
                                                     int ipf, const int *qps, int n_qp, int is_intra_slice,
                                                     uint32_t *d_satd, uavs3e_cuda_lat_q_t *d_q, void *stream)
{
    int r = ensure_init();
    if (r) return r;
    if (!d_org || !d_rec || !d_cus || !d_satd || !d_q || !qps) return set_status(UC_ERR_ARG, "intra_lattice: null pointer");
    if (width % 4 || height % 4) return set_status(UC_ERR_ARG, "intra_lattice: picture size must be a multiple of 4");
    return launch_intra_lattice(d_org, i_org, d_rec, i_rec, width, height, (const LatCu *)d_cus, n_cus, ipf, qps, n_qp,
                                is_intra_slice, d_satd, (LatQ *)d_q, (cudaStream_t)stream);
}

}  // extern "C"
