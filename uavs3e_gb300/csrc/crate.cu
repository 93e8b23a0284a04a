// Coefficient rate for lists of transform blocks: lbac_enc_run_length_cc_rdo (src/entropy.c:1688-
// 1950), the counting-mode coder the encoder's RDO runs on each candidate's levels -- per non-zero
// level in zig-zag order its run of zeros (truncated unary, cap 16, exp-Golomb escape), level - 1
// (cap 8, escape), sign and last flag (the averaged last1 / last2 pair), every bin on the context
// model it selects, the models updated as they go -- from the coder state the caller passes
// (range and the channel's run, run_rdoq, level, last1, last2 models).  Results: the bits
// counted, the range and the models after the block, bit-exact with the reference.
//
// The scan of each block runs over the warp's lanes; the coding is one chain per block (each bin
// updates the model and range the next one reads), one lane per block, the models in registers /
// local memory.  The model update is the rule the
// reference tabulates in tbl_plps / tbl_plps_ext (src/entropy.c:41), computed.
#include "common.cuh"
#include "tables.h"
#include "uavs3e_cuda_internal.h"
#include "../../include/uavs3e_cuda.h"

#include <mutex>
#include <string.h>

namespace uc {

struct CoefCtx { s16 run[12], run_rdoq[12], level[12], last1[6], last2[12]; };
struct CrReq { u32 coef_offset; u8 log2w, log2h, ch_type, pad; u16 num_sig, range; CoefCtx ctx; };
struct CrOut { u32 bits; u16 range, pad; CoefCtx ctx; };
static_assert(sizeof(CrReq) == sizeof(uavs3e_cuda_coef_rate_req_t), "coef rate request layout");
static_assert(sizeof(CrOut) == sizeof(uavs3e_cuda_coef_rate_out_t), "coef rate result layout");

struct CrParams {
    const CrReq *reqs;
    int n;
    const s16 *levels;
    unsigned long long n_levels;
    CrOut *out;
    const u16 *scan[7][7];
};

// the model after one bin: window state (bits 11-12: windows 3, 3, 4, 5), LPS probability (bits
// 1-10), MPS (bit 0); an MPS shrinks the probability by p >> w + p >> (w + 2), an LPS grows it by
// 197 / 95 / 46 (reflected about 1023 with the MPS flipped) and steps the state up
__device__ __forceinline__ s16 cr_next(int model, bool mps)
{
    const int c = (model >> 11) & 3, w = c < 2 ? 3 : c + 2;
    int p = (model >> 1) & 1023, m = model & 1;
    if (mps) {
        p -= (p >> w) + (p >> (w + 2));
        return (s16)(((c == 0 ? 1 : c) << 11) | (p << 1) | m);
    }
    p += w == 3 ? 197 : (w == 4 ? 95 : 46);
    if (p > 1023) { p = 2047 - p; m ^= 1; }
    return (s16)((min(c + 1, 3) << 11) | (p << 1) | m);
}

// counting-mode coding of one bin (lbac_encode_bin with no bitstream)
__device__ __forceinline__ void cr_bin(u32 &range, u32 &bits, s16 &mdl, int bin)
{
    const u32 lps = (u32)(mdl & 2047) >> 3;
    u32 mps = range - lps;
    const int s = mps < 256;
    mps |= 0x100;
    if (bin == (mdl & 1)) {
        bits += s;
        range = mps;
        mdl = cr_next(mdl, true);
    } else {
        const u32 l = (range << s) - mps;
        const int sh = __clz(l) - 23;
        range = l << sh;
        bits += sh + s;
        mdl = cr_next(mdl, false);
    }
}

// truncated unary symbol: first bin ('1' for 0) on m0, then '0' per unit and the closing '1' on
// m1, the closing bin omitted at the cap
__device__ __forceinline__ void cr_unary(u32 &range, u32 &bits, s16 &m0, s16 &m1, int sym, int cap)
{
    cr_bin(range, bits, m0, sym == 0);
    for (int k = 1; k <= sym && k < cap; k++) cr_bin(range, bits, m1, k == sym);
}

__device__ __forceinline__ u32 cr_egk(int v)
{
    int order = 1;
    for (int s = v; s >= 0; order++) s -= 1 << order;
    return (u32)((order << 1) - 1);
}

__device__ __forceinline__ bool cr_valid(const CrReq &q, unsigned long long n_levels)
{
    const int lw = q.log2w, lh = q.log2h, top = q.ch_type ? 5 : 6;
    const unsigned long long nc = 1ull << (lw + lh);
    bool ok = lw >= 2 && lw <= top && lh >= 2 && lh <= top && q.num_sig >= 1 && q.num_sig <= nc &&
              q.range >= 256 && q.range <= 511 && (unsigned long long)q.coef_offset + nc <= n_levels;
    const s16 *mdl = &q.ctx.run[0];
    const int nchk = q.ch_type ? 52 : 54;             // chroma codes no last2 context past 9
#pragma unroll
    for (int k = 0; k < 54; k++)
        ok = ok && (k >= nchk || (((mdl[k] >> 1) & 1023) >= 4 && mdl[k] >= 0 && mdl[k] < 8192));
    return ok;
}

// Warp per 32 blocks.  First the warp takes its blocks one by one and lists, in scan order, the
// positions and values of their first num_sig non-zero levels (a ballot and a prefix count per 32
// positions) in list[] at the block's own level offset; then each lane codes its block's chain
// from that list.  A run of zeros steps the run_rdoq model once per zero; the steps stop changing
// the model once its probability is too small to move (p >> w == 0 after an MPS), so the walk ends
// there.
__global__ void __launch_bounds__(128) k_coef_rate(const CrParams P, u32 *list_all)
{
    __shared__ int s_cnt[4][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r0 = (blockIdx.x * 4 + warp) * 32;
    if (r0 >= P.n) return;
    for (int r = 0; r < 32 && r0 + r < P.n; r++) {
        const CrReq q = P.reqs[r0 + r];
        int cnt = 0;
        if (cr_valid(q, P.n_levels)) {
            const int n = 1 << (q.log2w + q.log2h);
            const s16 *coef = P.levels + q.coef_offset;
            const u16 *scan = P.scan[q.log2w][q.log2h];
            u32 *list = list_all + q.coef_offset;
            for (int base = 0; base < n && cnt < q.num_sig; base += 32) {
                const int i = base + lane;
                const int c = i < n ? coef[scan[i]] : 0;
                const u32 m = __ballot_sync(0xffffffffu, c != 0);
                const int at = cnt + __popc(m & ((1u << lane) - 1));
                if (c != 0 && at < q.num_sig) list[at] = ((u32)i << 16) | (u16)(s16)c;
                cnt += __popc(m);
            }
        }
        if (lane == 0) s_cnt[warp][r] = min(cnt, 65535);
    }
    __syncwarp();
    const int i = r0 + lane;
    if (i >= P.n) return;
    const CrReq q = P.reqs[i];
    CrOut o;
    o.ctx = q.ctx;
    o.pad = 0;
    o.bits = ~0u;                     // outside the domain, or fewer levels than num_sig: state unchanged
    o.range = q.range;
    if (!cr_valid(q, P.n_levels) || s_cnt[warp][lane] < q.num_sig) {
        P.out[i] = o;
        return;
    }
    CoefCtx &c = o.ctx;
    const u32 *list = list_all + q.coef_offset;
    const int n = 1 << (q.log2w + q.log2h);
    u32 range = q.range, bits = 0;
    int t0 = 10, last = -1;
    for (int k = 0; k < q.num_sig; k++) {
        const u32 e = list[k];
        const int pos = (int)(e >> 16), level = abs((int)(s16)(e & 0xFFFF));
        const int run = pos - last - 1;
        last = pos;
        cr_unary(range, bits, c.run[t0], c.run[t0 + 1], min(run, 16), 16);
        if (run >= 16) bits += cr_egk(run - 17);
        c.run_rdoq[t0] = cr_next(c.run_rdoq[t0], (run == 0) == (c.run_rdoq[t0] & 1));
        s16 m = c.run_rdoq[t0 + 1];
        for (int z = 1; z < run; z++) {                // zeros: bin 0
            const s16 nm = cr_next(m, (m & 1) == 0);
            if (nm == m) break;                        // a fixed point: the remaining zeros keep it
            m = nm;
        }
        if (run > 0) m = cr_next(m, (m & 1) == 1);     // the closing '1'
        c.run_rdoq[t0 + 1] = m;
        cr_unary(range, bits, c.level[t0], c.level[t0 + 1], min(level - 1, 8), 8);
        if (level >= 9) bits += cr_egk(level - 10);
        bits++;                                       // sign
        if (pos == n - 1) break;
        s16 &m1 = c.last1[t0 >> 1];
        s16 &m2 = c.last2[31 - __clz(pos + 1)];
        t0 = min(level - 1, 5) << 1;
        const int p1 = (m1 & 2047) >> 1, p2 = (m2 & 2047) >> 1, c1 = m1 & 1, c2 = m2 & 1;
        int cm, pl;
        if (c1 == c2) { cm = c1; pl = (p1 + p2) >> 1; }
        else if (p1 < p2) { cm = c1; pl = 1023 - ((p2 - p1) >> 1); }
        else { cm = c2; pl = 1023 - ((p1 - p2) >> 1); }
        const int flag = k == q.num_sig - 1;
        u32 mps = range - ((u32)pl >> 2);
        const int s = mps < 256;
        mps |= 0x100;
        if (flag == cm) { bits += s; range = mps; }
        else {
            const u32 l = (range << s) - mps;
            const int sh = __clz(l) - 23;
            range = l << sh;
            bits += sh + s;
        }
        m1 = cr_next(m1, flag == c1);
        m2 = cr_next(m2, flag == c2);
    }
    o.bits = bits;
    o.range = (u16)range;
    P.out[i] = o;
}

int launch_coef_rate(const void *reqs, int n, const s16 *levels, unsigned long long n_levels, void *out,
                     cudaStream_t st)
{
    if (n < 0 || (n > 0 && (!reqs || !levels || !out))) return set_status(UC_ERR_ARG, "coef_rate: null argument");
    if (n == 0) return UC_OK;
    int dev = 0;
    UC_CHECK(cudaGetDevice(&dev));
    const DevTables *tab = device_tables(dev);
    if (!tab) return set_status(UC_ERR_MEMORY, "coef_rate: table upload failed");
    CrParams P;
    memset(&P, 0, sizeof(P));
    P.reqs = (const CrReq *)reqs; P.n = n; P.levels = levels; P.n_levels = n_levels; P.out = (CrOut *)out;
    for (int a = 0; a < 7; a++)
        for (int b = 0; b < 7; b++) P.scan[a][b] = tab->scan[a][b];
    u32 *list = nullptr;                              // one word per level, at the levels' offsets
    UC_CHECK(cudaMallocAsync((void **)&list, (size_t)n_levels * sizeof(u32), st));
    k_coef_rate<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(P, list);
    UC_CHECK(cudaGetLastError());
    UC_CHECK(cudaFreeAsync(list, st));
    count_launch(1);
    return UC_OK;
}

struct CrScratch {
    std::mutex mu;
    cudaStream_t st = nullptr;
    void *buf = nullptr;
    size_t cap = 0;
};
static CrScratch g_cr[64];

}  // namespace uc

using namespace uc;

extern "C" UAVS3E_CUDA_API int uavs3e_cuda_coef_rate(const uavs3e_cuda_coef_rate_req_t *reqs, int n,
                                                    const int16_t *levels, size_t n_levels,
                                                    uavs3e_cuda_coef_rate_out_t *out)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (n < 0 || (n > 0 && (!reqs || !levels || !out))) return set_status(UC_ERR_ARG, "coef_rate: bad argument");
    if (n == 0) return UC_OK;
    int dev = 0;
    UC_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_status(UC_ERR_UNSUPPORTED, "coef_rate: device index");
    CrScratch &S = g_cr[dev];
    std::lock_guard<std::mutex> lk(S.mu);
    if (!S.st) UC_CHECK(cudaStreamCreateWithFlags(&S.st, cudaStreamNonBlocking));
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t b_req = up((size_t)n * sizeof(*reqs)), b_lev = up(n_levels * sizeof(int16_t));
    const size_t need = b_req + b_lev + up((size_t)n * sizeof(*out));
    if (S.cap < need) {
        if (S.buf) UC_CHECK(cudaFree(S.buf));
        S.buf = nullptr;
        S.cap = 0;
        UC_CHECK(cudaMalloc(&S.buf, need));
        S.cap = need;
    }
    char *b = (char *)S.buf;
    void *d_req = b, *d_out = b + b_req + b_lev;
    s16 *d_lev = (s16 *)(b + b_req);
    UC_CHECK(cudaMemcpyAsync(d_req, reqs, (size_t)n * sizeof(*reqs), cudaMemcpyHostToDevice, S.st));
    UC_CHECK(cudaMemcpyAsync(d_lev, levels, n_levels * sizeof(int16_t), cudaMemcpyHostToDevice, S.st));
    rc = launch_coef_rate(d_req, n, d_lev, (unsigned long long)n_levels, d_out, S.st);
    if (rc) return rc;
    UC_CHECK(cudaMemcpyAsync(out, d_out, (size_t)n * sizeof(*out), cudaMemcpyDeviceToHost, S.st));
    UC_CHECK(cudaStreamSynchronize(S.st));
    return UC_OK;
}

extern "C" UAVS3E_CUDA_API int uavs3e_cuda_coef_rate_device(const uavs3e_cuda_coef_rate_req_t *d_reqs, int n,
                                                           const int16_t *d_levels, size_t n_levels,
                                                           uavs3e_cuda_coef_rate_out_t *d_out, void *stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    return launch_coef_rate(d_reqs, n, d_levels, (unsigned long long)n_levels, d_out, (cudaStream_t)stream);
}
