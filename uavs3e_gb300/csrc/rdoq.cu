// RDOQ of transform blocks for lists of blocks: quant_non_zero with flat quantisation
// (src/quant.c:315-383) -> rdoq_quant_block (:196-313), each block with the bin-cost estimates
// the encoder derived from its entropy-coder state (rdoq_init_cu_est_bits, :139-156) -- the
// levels and the count of coded coefficients bit-exact with the reference's call.
//
// One warp per 32 blocks.  First the warp takes its blocks one by one: zeroes the coefficients
// past 32 columns / rows, runs quant_check, and lists in scan order the positions whose
// first-pass level (quant_rdoq) is not zero (ballot + prefix count).  The decision pass is a
// chain (each coded level selects the contexts of the next), so then every lane walks the chain
// of one block over its listed positions: a run of z zero levels adds
// est_run[last_b_zero][0] + (z - 1) est_run[1][0] bits at once, as the reference's per-position
// loop accumulates them.
#include "common.cuh"
#include "quant_tables.cuh"
#include "tables.h"
#include "uavs3e_cuda_internal.h"
#include "../../include/uavs3e_cuda.h"

#include <math.h>
#include <mutex>
#include <string.h>

namespace uc {

constexpr int RQ_WARPS = 4;

struct RdoqReq {
    u32 coef_offset; u8 log2w, log2h, qp, is_intra, ch_type, slice_type; u16 est; u32 pad; s64 lambda;
};
struct RdoqEst {
    s32 ctp[2]; s32 cbf[3][2]; s32 run[24][2]; s32 lvl[24][2]; s32 lst[2][6][12][2];
};
static_assert(sizeof(RdoqReq) == sizeof(uavs3e_cuda_rdoq_req_t), "request layout");
static_assert(sizeof(RdoqEst) == sizeof(uavs3e_cuda_rdoq_est_t), "estimate layout");

struct RdoqParams {
    const RdoqReq *reqs;
    int n, n_est;
    const RdoqEst *ests;
    s16 *coefs;
    unsigned long long n_coefs;
    s32 *num_nz;
    u32 *scratch;             // per coefficient: the listed positions of each block
    const u16 *scan[7][7];
    const u16 *scanpos[7][7];
    s32 err_scale[80][6];     // tbl_rdoq_err_scale (rdoq_init_err_scale, src/quant.c:69-83), 8-bit
};

// rdoq_one_coef (src/quant.c:158-194)
__device__ __forceinline__ u32 rq_coef(s64 uncoded, s64 *coded, u32 level_double, u32 abs_level, const s32 *est_run,
                                       const s32 (*est_level)[2], int q_bits, s32 err_scale, s64 lambda, bool last_pos)
{
    u32 best = 0;
    *coded = uncoded + (s64)est_run[0] * lambda;
    for (int checks = 2; abs_level && checks; checks--, abs_level--) {
        const s32 diff = (s32)(level_double - (abs_level << q_bits));
        const s64 err = ((s64)diff * err_scale) >> 20;
        s32 rate = 32768;
        if (!last_pos) rate += est_run[1];
        if (abs_level == 1) rate += est_level[0][1];
        else if (abs_level < 9) rate += est_level[0][0] + est_level[1][0] * (s32)(abs_level - 2) + est_level[1][1];
        else rate += est_level[0][0] + est_level[1][0] * 7 + (((31 - __clz((int)abs_level - 8)) << 1) + 1) * 32768;
        const s64 cost = err * err + (s64)rate * lambda;
        if (cost < *coded) { best = abs_level; *coded = cost; }
    }
    return best;
}

__global__ void __launch_bounds__(32 * RQ_WARPS) k_rdoq(const RdoqParams P)
{
    __shared__ int s_cnt[RQ_WARPS][32];        // marked positions of each of the warp's blocks, -1: done
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r0 = (blockIdx.x * RQ_WARPS + warp) * 32;
    if (r0 >= P.n) return;
    // phase 1, the warp over each of its 32 blocks in turn
    for (int b = 0; b < 32; b++) {
        const int r = r0 + b;
        if (r >= P.n) break;
        const RdoqReq q = P.reqs[r];
        const int lw = q.log2w, lh = q.log2h, w = 1 << lw, h = 1 << lh;
        // blocks outside the supported domain are left untouched, with num_nz = -1
        if (lw < 2 || lw > 6 || lh < 2 || lh > 6 || q.qp > 79 || q.ch_type > 2 || q.est >= P.n_est ||
            (unsigned long long)q.coef_offset + (unsigned long long)(w * h) > P.n_coefs) {
            if (lane == 0) { P.num_nz[r] = -1; s_cnt[warp][b] = -1; }
            continue;
        }
        s16 *coef = P.coefs + q.coef_offset;
        const int max_num = w * h, max_used = 1 << (lw + min(5, lh));
        // quant_non_zero: coefficients past 32 columns / rows are zeroed
        if (w > 32 || h > 32)
            for (int p = lane; p < max_num; p += 32)
                if ((p & (w - 1)) >= 32 || (p >> lw) >= 32) coef[p] = 0;
        __syncwarp();
        // rdoq_quant_block: quant_check over the first max_used coefficients (raster order)
        const int odd = (lw + lh) & 1, log2_size = (lw + lh) >> 1;
        const int q_bits = 14 + (15 - 8 - log2_size);
        const int q_value = odd ? ((int)kQScale[q.qp] * 181 + 64) >> 7 : (int)kQScale[q.qp];
        const int offset = (q.slice_type == 1 ? 201 : 153) << (q_bits - 9);
        const int nz_thr = ((((1 << q_bits) - offset) << 10) / q_value - 1) >> 10;
        bool above = false;
        for (int p = lane; p < max_used; p += 32) {
            const int c = coef[p];
            above |= c > nz_thr || c < -nz_thr;
        }
        if (!__any_sync(0xffffffffu, above)) {
            if (lane == 0) { P.num_nz[r] = 0; s_cnt[warp][b] = -1; }
            continue;
        }
        // scan order; the positions whose first-pass level (quant_rdoq) is not zero -- exactly
        // those with |c| >= thr -- are listed in order as (position << 16 | coefficient)
        const u16 *scan = P.scan[lw][lh];
        const int thr = ((1 << (q_bits - 1)) - 1) / q_value + 1;
        u32 *list = P.scratch + q.coef_offset;
        int cnt = 0;
        for (int base = 0; base < max_num; base += 32) {
            const int i = base + lane;
            const int c = i < max_num ? coef[scan[i]] : 0;
            const bool mark = abs(c) >= thr;
            const u32 m = __ballot_sync(0xffffffffu, mark);
            if (mark) list[cnt + __popc(m & ((1u << lane) - 1))] = ((u32)i << 16) | (u16)c;
            cnt += __popc(m);
        }
        __syncwarp();
        for (int p = lane; p < max_num; p += 32) coef[p] = 0;   // levels are written over the block
        if (lane == 0) s_cnt[warp][b] = cnt;
        __syncwarp();
    }
    __syncwarp();
    // phase 2: lane b walks the decision chain of block b
    const int r = r0 + lane;
    if (r >= P.n) return;
    const int cnt = s_cnt[warp][lane];
    if (cnt < 0) return;
    const RdoqReq q = P.reqs[r];
    const int lw = q.log2w, lh = q.log2h, ch = q.ch_type, max_num = 1 << (lw + lh);
    const int odd = (lw + lh) & 1, log2_size = (lw + lh) >> 1;
    const int q_bits = 14 + (15 - 8 - log2_size);
    const int q_value = odd ? ((int)kQScale[q.qp] * 181 + 64) >> 7 : (int)kQScale[q.qp];
    s16 *coef = P.coefs + q.coef_offset;
    const u16 *scan = P.scan[lw][lh];
    const u32 *list = P.scratch + q.coef_offset;
    const RdoqEst &E = P.ests[q.est];
    const s32 err_scale = P.err_scale[q.qp][log2_size - 1];
    const s64 lambda = q.lambda;
    const u32 add = 1u << (q_bits - 1);
    s64 best_delta, curr_delta;
    if (!q.is_intra && ch == 0) { best_delta = (s64)E.ctp[1] * lambda; curr_delta = (s64)E.ctp[0] * lambda; }
    else { best_delta = (s64)E.cbf[ch][0] * lambda; curr_delta = (s64)E.cbf[ch][1] * lambda; }
    const int base = ch == 0 ? 0 : 12;
    const s32 (*lst)[2] = E.lst[ch != 0][5];
    const s32 (*est_run)[2] = E.run + 10 + base, (*est_lvl)[2] = E.lvl + 10 + base;
    u32 last_b_zero = 0;
    int end_pos = 0, last_checked = 0, tmp_nz = 0, num_nz = 0, zero_bins = 0, prev = -1;
    for (int k = 0; k < cnt; k++) {
        const u32 ent = list[k];
        const int i = (int)(ent >> 16), c = (s16)(ent & 0xffffu);
        const int z = i - prev - 1;                // zero levels since the previous listed position
        if (z > 0) {
            zero_bins += est_run[last_b_zero][0] + (z - 1) * est_run[1][0];
            last_b_zero = 1;
        }
        prev = i;
        if (zero_bins) { curr_delta += (s64)zero_bins * lambda; zero_bins = 0; }
        const u32 ld = (u32)abs(c) * (u32)q_value;
        const s64 e = ((s64)ld * err_scale) >> 20;
        const s64 zerr = e * e;
        const u32 abs_level = (u32)(s16)(u32)(((u64)ld + add) >> q_bits);
        s64 cc;
        const u32 level = rq_coef(zerr, &cc, ld, abs_level, est_run[last_b_zero], est_lvl, q_bits, err_scale, lambda,
                                  i == max_num - 1);
        curr_delta += cc - zerr;
        if (level) {
            last_checked = i;
            coef[scan[i]] = (s16)(c < 0 ? -(int)level : (int)level);
            const int lg = 31 - __clz(i + 1);
            const s64 end_cost = curr_delta + (s64)lst[lg][1] * lambda;
            curr_delta += (s64)lst[lg][0] * lambda;
            tmp_nz++;
            if (end_cost < best_delta) { best_delta = end_cost; end_pos = i; num_nz += tmp_nz; tmp_nz = 0; }
            last_b_zero = 0;
            const int cls = min((int)level - 1, 5);
            est_lvl = E.lvl + (cls << 1) + base;
            est_run = E.run + (cls << 1) + base;
            lst = E.lst[ch != 0][cls];
        } else {
            last_b_zero = 1;
        }
    }
    if (num_nz)
        for (int k = 0; k < cnt; k++) {            // positions after the chosen last one, back to zero
            const int i = (int)(list[k] >> 16);
            if (i > end_pos && i <= last_checked) coef[scan[i]] = 0;
        }
    P.num_nz[r] = num_nz;
}

int launch_rdoq(const void *reqs, int n, const void *ests, int n_est, s16 *coefs, unsigned long long n_coefs,
                s32 *num_nz, cudaStream_t st)
{
    if (!reqs || !ests || !coefs || !num_nz || n < 0 || n_est < 1) return set_status(UC_ERR_ARG, "rdoq: null argument");
    if (n == 0) return UC_OK;
    int dev = 0;
    UC_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_status(UC_ERR_UNSUPPORTED, "rdoq: device index");
    const DevTables *tab = device_tables(dev);
    if (!tab) return set_status(UC_ERR_MEMORY, "rdoq: table upload failed");
    RdoqParams P;
    memset(&P, 0, sizeof(P));
    P.reqs = (const RdoqReq *)reqs; P.n = n; P.ests = (const RdoqEst *)ests; P.n_est = n_est;
    P.coefs = coefs; P.n_coefs = n_coefs; P.num_nz = num_nz;
    for (int a = 0; a < 7; a++)
        for (int b = 0; b < 7; b++) { P.scan[a][b] = tab->scan[a][b]; P.scanpos[a][b] = tab->scanpos[a][b]; }
    // rdoq_init_err_scale for 8-bit: 2^(15 - tr_shift) / q_value in 20-bit fixed point
    static const u16 qs[80] = {
        16302, 15024, 13777, 12634, 11626, 10624, 9742, 8958, 8192, 7512, 6889, 6305, 5793, 5303, 4878, 4467,
        4091, 3756, 3444, 3161, 2894, 2654, 2435, 2235, 2048, 1878, 1722, 1579, 1449, 1329, 1218, 1117,
        1024, 939, 861, 790, 724, 664, 609, 558, 512, 470, 430, 395, 362, 332, 304, 279,
        256, 235, 215, 197, 181, 166, 152, 140, 128, 116, 108, 99, 91, 83, 76, 69,
        64, 59, 54, 49, 45, 41, 38, 35, 32, 30, 27, 25, 23, 21, 19, 18,
    };
    for (int qp = 0; qp < 80; qp++)
        for (int i = 0; i < 6; i++) {
            const int tr_shift = 15 - 8 - (i + 1);
            double es = pow(2.0, 15 - tr_shift);
            es = es / qs[qp] / 1;
            P.err_scale[qp][i] = (s32)(es * (double)(1 << 20));
        }
    // the position lists: one word per coefficient, kept per device and grown on demand
    {
        static u32 *scratch[64] = { nullptr };
        static unsigned long long cap[64] = { 0 };
        static std::mutex mu;
        std::lock_guard<std::mutex> lk(mu);
        if (cap[dev] < n_coefs) {
            if (scratch[dev]) UC_CHECK(cudaFree(scratch[dev]));
            scratch[dev] = nullptr;
            cap[dev] = 0;
            UC_CHECK(cudaMalloc(&scratch[dev], n_coefs * sizeof(u32)));
            cap[dev] = n_coefs;
        }
        P.scratch = scratch[dev];
    }
    prof_begin(PROF_RDOQ, st);
    const int warps = (n + 31) / 32;
    k_rdoq<<<(unsigned)((warps + RQ_WARPS - 1) / RQ_WARPS), 32 * RQ_WARPS, 0, st>>>(P);
    UC_CHECK(cudaGetLastError());
    count_launch(1);
    prof_end(PROF_RDOQ, st);
    return UC_OK;
}

}  // namespace uc

using namespace uc;

// per device: buffers of the host-memory entry point
// quant_non_zero's weighted branch (pic_wq_enable, src/quant.c:335-380) for lists of blocks: the
// zero-out past 32 columns / rows, then every level (s16)((|c| scale ns_scale 64 / weight + offset)
// >> shift) in 64-bit arithmetic with the weight of the sample's cell of the 4x4 (4x4 blocks) or
// 8x8 matrix (one cell per 2^(max(log2 w, log2 h) - 3) samples each way).  A warp per block.
__global__ void __launch_bounds__(128) k_quant_wq(const RdoqReq *reqs, int n, const u8 *wq4, const u8 *wq8,
                                                  s16 *coefs, unsigned long long n_coefs, s32 *num_nz)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.x * 4 + warp;
    if (r >= n) return;
    const RdoqReq q = reqs[r];
    const int lw = q.log2w, lh = q.log2h, w = 1 << lw, h = 1 << lh;
    if (lw < 2 || lw > 6 || lh < 2 || lh > 6 || q.qp > 79 || q.ch_type > 2 ||
        (unsigned long long)q.coef_offset + (unsigned long long)(w * h) > n_coefs) {
        if (lane == 0) num_nz[r] = -1;       // outside the supported domain: block untouched
        return;
    }
    s16 *coef = coefs + q.coef_offset;
    const int log2_size = (lw + lh) >> 1, odd = (lw + lh) & 1;
    const int ns_shift = odd ? 7 : 0, ns_scale = odd ? 181 : 1;
    const int shift = 14 + 15 - 8 - (log2_size - ns_shift);
    const long long offset = (long long)(q.slice_type == 1 ? 171 : 85) << (shift - 9);
    const long long scale = (long long)kQScale[q.qp] * ns_scale * 64;
    const bool small = lw == 2 && lh == 2;
    const u8 *wq = small ? wq4 : wq8;
    const int idx_shift = small ? 0 : max(lw, lh) - 3, width = small ? 4 : 8;
    int nz = 0;
    for (int p = lane; p < w * h; p += 32) {
        const int i = p >> lw, j = p & (w - 1);
        const int c = (i >= 32 || j >= 32) ? 0 : coef[p];
        const int weight = wq[(i >> idx_shift) * width + (j >> idx_shift)];
        const int lev = (s16)(u16)(unsigned long long)((((long long)abs(c) * scale) / weight + offset) >> shift);
        const s16 v = (s16)(c < 0 ? -lev : lev);
        coef[p] = v;
        nz += v != 0;
    }
#pragma unroll
    for (int m = 16; m; m >>= 1) nz += __shfl_xor_sync(0xffffffffu, nz, m);
    if (lane == 0) num_nz[r] = nz;
}

int launch_quant_wq(const void *reqs, int n, const u8 *wq4, const u8 *wq8, s16 *coefs, unsigned long long n_coefs,
                    s32 *num_nz, cudaStream_t st)
{
    if (n < 0 || (n > 0 && (!reqs || !wq4 || !wq8 || !coefs || !num_nz)))
        return set_status(UC_ERR_ARG, "quant_wq: null argument");
    if (n == 0) return UC_OK;
    prof_begin(PROF_RDOQ, st);
    k_quant_wq<<<(unsigned)((n + 3) / 4), 128, 0, st>>>((const RdoqReq *)reqs, n, wq4, wq8, coefs, n_coefs, num_nz);
    UC_CHECK(cudaGetLastError());
    count_launch(1);
    prof_end(PROF_RDOQ, st);
    return UC_OK;
}

struct RdoqScratch {
    std::mutex mu;
    cudaStream_t st = nullptr;
    void *buf = nullptr;
    size_t cap = 0;
};
static RdoqScratch g_rdoq[64];

extern "C" UAVS3E_CUDA_API int uavs3e_cuda_rdoq(const uavs3e_cuda_rdoq_req_t *reqs, int n,
                                                const uavs3e_cuda_rdoq_est_t *ests, int n_est, int16_t *coefs,
                                                size_t n_coefs, int32_t *num_nz)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (n < 0 || n_est < 1 || (n > 0 && (!reqs || !ests || !coefs || !num_nz)))
        return set_status(UC_ERR_ARG, "rdoq: bad argument");
    if (n == 0) return UC_OK;
    int dev = 0;
    UC_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_status(UC_ERR_UNSUPPORTED, "rdoq: device index");
    RdoqScratch &S = g_rdoq[dev];
    std::lock_guard<std::mutex> lk(S.mu);
    if (!S.st) UC_CHECK(cudaStreamCreateWithFlags(&S.st, cudaStreamNonBlocking));
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t b_req = up((size_t)n * sizeof(*reqs)), b_est = up((size_t)n_est * sizeof(*ests));
    const size_t b_coef = up(n_coefs * sizeof(int16_t)), b_nz = up((size_t)n * sizeof(int32_t));
    const size_t need = b_req + b_est + b_coef + b_nz;
    if (S.cap < need) {
        if (S.buf) UC_CHECK(cudaFree(S.buf));
        S.buf = nullptr;
        S.cap = 0;
        UC_CHECK(cudaMalloc(&S.buf, need));
        S.cap = need;
    }
    char *b = (char *)S.buf;
    void *d_req = b, *d_est = b + b_req;
    int16_t *d_coef = (int16_t *)(b + b_req + b_est);
    int32_t *d_nz = (int32_t *)(b + b_req + b_est + b_coef);
    UC_CHECK(cudaMemcpyAsync(d_req, reqs, (size_t)n * sizeof(*reqs), cudaMemcpyHostToDevice, S.st));
    UC_CHECK(cudaMemcpyAsync(d_est, ests, (size_t)n_est * sizeof(*ests), cudaMemcpyHostToDevice, S.st));
    UC_CHECK(cudaMemcpyAsync(d_coef, coefs, n_coefs * sizeof(int16_t), cudaMemcpyHostToDevice, S.st));
    rc = launch_rdoq(d_req, n, d_est, n_est, d_coef, (unsigned long long)n_coefs, d_nz, S.st);
    if (rc) return rc;
    UC_CHECK(cudaMemcpyAsync(coefs, d_coef, n_coefs * sizeof(int16_t), cudaMemcpyDeviceToHost, S.st));
    UC_CHECK(cudaMemcpyAsync(num_nz, d_nz, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, S.st));
    UC_CHECK(cudaStreamSynchronize(S.st));
    return UC_OK;
}

extern "C" UAVS3E_CUDA_API int uavs3e_cuda_rdoq_device(const uavs3e_cuda_rdoq_req_t *d_reqs, int n,
                                                       const uavs3e_cuda_rdoq_est_t *d_ests, int n_est,
                                                       int16_t *d_coefs, size_t n_coefs, int32_t *d_num_nz,
                                                       void *stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    return launch_rdoq(d_reqs, n, d_ests, n_est, d_coefs, (unsigned long long)n_coefs, d_num_nz, (cudaStream_t)stream);
}

extern "C" UAVS3E_CUDA_API int uavs3e_cuda_quant_wq(const uavs3e_cuda_rdoq_req_t *reqs, int n, const uint8_t *wq4,
                                                   const uint8_t *wq8, int16_t *coefs, size_t n_coefs,
                                                   int32_t *num_nz)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (n < 0 || (n > 0 && (!reqs || !wq4 || !wq8 || !coefs || !num_nz)))
        return set_status(UC_ERR_ARG, "quant_wq: bad argument");
    if (n == 0) return UC_OK;
    int dev = 0;
    UC_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_status(UC_ERR_UNSUPPORTED, "quant_wq: device index");
    RdoqScratch &S = g_rdoq[dev];
    std::lock_guard<std::mutex> lk(S.mu);
    if (!S.st) UC_CHECK(cudaStreamCreateWithFlags(&S.st, cudaStreamNonBlocking));
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t b_req = up((size_t)n * sizeof(*reqs)), b_wq = 256;
    const size_t b_coef = up(n_coefs * sizeof(int16_t)), b_nz = up((size_t)n * sizeof(int32_t));
    const size_t need = b_req + b_wq + b_coef + b_nz;
    if (S.cap < need) {
        if (S.buf) UC_CHECK(cudaFree(S.buf));
        S.buf = nullptr;
        S.cap = 0;
        UC_CHECK(cudaMalloc(&S.buf, need));
        S.cap = need;
    }
    char *b = (char *)S.buf;
    void *d_req = b;
    u8 *d_wq = (u8 *)(b + b_req);
    int16_t *d_coef = (int16_t *)(b + b_req + b_wq);
    int32_t *d_nz = (int32_t *)(b + b_req + b_wq + b_coef);
    UC_CHECK(cudaMemcpyAsync(d_req, reqs, (size_t)n * sizeof(*reqs), cudaMemcpyHostToDevice, S.st));
    UC_CHECK(cudaMemcpyAsync(d_wq, wq4, 16, cudaMemcpyHostToDevice, S.st));
    UC_CHECK(cudaMemcpyAsync(d_wq + 16, wq8, 64, cudaMemcpyHostToDevice, S.st));
    UC_CHECK(cudaMemcpyAsync(d_coef, coefs, n_coefs * sizeof(int16_t), cudaMemcpyHostToDevice, S.st));
    rc = launch_quant_wq(d_req, n, d_wq, d_wq + 16, d_coef, (unsigned long long)n_coefs, d_nz, S.st);
    if (rc) return rc;
    UC_CHECK(cudaMemcpyAsync(coefs, d_coef, n_coefs * sizeof(int16_t), cudaMemcpyDeviceToHost, S.st));
    UC_CHECK(cudaMemcpyAsync(num_nz, d_nz, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, S.st));
    UC_CHECK(cudaStreamSynchronize(S.st));
    return UC_OK;
}

extern "C" UAVS3E_CUDA_API int uavs3e_cuda_quant_wq_device(const uavs3e_cuda_rdoq_req_t *d_reqs, int n,
                                                          const uint8_t *d_wq4, const uint8_t *d_wq8,
                                                          int16_t *d_coefs, size_t n_coefs, int32_t *d_num_nz,
                                                          void *stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    return launch_quant_wq(d_reqs, n, d_wq4, d_wq8, d_coefs, (unsigned long long)n_coefs, d_num_nz,
                           (cudaStream_t)stream);
}
