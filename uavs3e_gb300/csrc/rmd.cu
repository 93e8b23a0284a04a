// Intra mode candidates for lists of prediction blocks: make_ipred_list (src/intra.c:226-367)
// with check_one_mode (:209) -- cost = SATD + bits x sqrt_lambda in double, the staged fast search
// (10 coarse modes, +-2 of the best 7, +-1 of the first 3 angular entries, the untried MPMs) or the
// full one, the MPM completion and the inter-SATD cut -- bit-exact with the reference.  The SATD
// of each mode comes from an array with the intra lattice's record layout (satd[row * 33 + mode]);
// the bits of each mode are the counting-mode LBAC coding of intra_dir (lbac_enc_intra_dir,
// src/entropy.c:2118; lbac_encode_bin :1168) from the block's coder state (range and the 7
// intra_dir context models), which is the part of the rate estimation this decision needs.
//
// One thread per block: the decision is a short sequential chain over at most 33 candidates; its
// list and per-mode costs live in shared memory.  Costs are non-negative doubles, so the list's
// comparisons run on their bit patterns.
#include "common.cuh"
#include "uavs3e_cuda_internal.h"
#include "../../include/uavs3e_cuda.h"

#include <mutex>

namespace uc {

struct RmdReq {
    u32 satd_row; u8 pb_w, pb_h; u8 mpm[2]; u8 skip_ipd; u8 fast; u16 range; s16 ctx[7]; u8 pad[6];
    double sqrt_lambda; u64 inter_satd; double satd_threshold;
};
struct RmdOut { s8 list[5]; u8 count; u8 pad[2]; };
static_assert(sizeof(RmdReq) == sizeof(uavs3e_cuda_rmd_req_t), "rmd request layout");
static_assert(sizeof(RmdOut) == sizeof(uavs3e_cuda_rmd_out_t), "rmd result layout");

constexpr unsigned long long RMD_MAX_COST = 0x7fee42d130773b76ull;   // bits of 1.7e+308 (MAX_D_COST)

// one bin of lbac_encode_bin in counting mode: the range after it and the bits it adds (each
// intra_dir model is used once per syntax element, so its update does not change the count)
__device__ __forceinline__ void rmd_bin(u32 &range, int &bits, int bin, int model)
{
    const u32 lps = (u32)(model & 2047) >> 3;
    u32 mps = range - lps;
    const int s = mps < 256;
    mps |= 0x100;
    if (bin == (model & 1)) {
        bits += s;
        range = mps;
    } else {
        const u32 l = (range << s) - mps;           // 1..510
        const int sh = __clz(l) - 23;               // get_shift
        range = l << sh;
        bits += sh + s;
    }
}

// lbac_enc_intra_dir: an MPM as flag 1 + its index, another mode as flag 0 + its 5-bit rank
__device__ __forceinline__ int rmd_bits(const RmdReq &q, int ipm)
{
    const int m0 = q.mpm[0], m1 = q.mpm[1];
    const int code = ipm == m0 ? -2 : (ipm == m1 ? -1 : (ipm < m0 ? ipm : (ipm < m1 ? ipm - 1 : ipm - 2)));
    u32 r = q.range;
    int bits = 0;
    if (code < 0) {
        rmd_bin(r, bits, 1, q.ctx[0]);
        rmd_bin(r, bits, code + 2, q.ctx[6]);
    } else {
        rmd_bin(r, bits, 0, q.ctx[0]);
#pragma unroll
        for (int i = 4; i >= 0; i--) rmd_bin(r, bits, (code >> i) & 1, q.ctx[1 + (4 - i)]);
    }
    return bits;
}

constexpr int RMD_THREADS = 128;

// a thread's candidate list and per-mode costs (bit patterns of the non-negative double costs),
// in shared memory, mode-major so that the threads of a warp touch consecutive words
struct RmdState {
    unsigned long long (*cost)[RMD_THREADS];
    s8 (*list)[RMD_THREADS];
    int t;
    __device__ int l(int k) const { return list[k][t]; }
    __device__ void set_l(int k, int v) { list[k][t] = (s8)v; }
    __device__ unsigned long long c(int m) const { return cost[m][t]; }
};

// check_one_mode + com_update_cand_list (src/intra.c:187-224)
__device__ void rmd_check(RmdState &S, const RmdReq &q, const u32 *satd, int ipm, int len)
{
    const double c = __dadd_rn((double)satd[ipm], __dmul_rn((double)rmd_bits(q, ipm), q.sqrt_lambda));
    const unsigned long long cb = (unsigned long long)__double_as_longlong(c);
    S.cost[ipm][S.t] = cb;
    int shift = 0, p = len - 1;
    while (shift < len && (S.l(p) < 0 || cb < S.c(S.l(p)))) { p--; shift++; }
    if (shift) {
        int k = len - 1;
        for (shift--; shift; shift--, k--) S.set_l(k, S.l(k - 1));
        S.set_l(k, ipm);
    }
}

__global__ void __launch_bounds__(RMD_THREADS) k_intra_rmd(const u32 *satd_all, unsigned long long n_rows,
                                                           const RmdReq *reqs, int n, RmdOut *out)
{
    __shared__ unsigned long long s_cost[33][RMD_THREADS];
    __shared__ s8 s_list[33][RMD_THREADS];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const RmdReq q = reqs[i];
    RmdOut o;
    o.pad[0] = o.pad[1] = 0;
    const int w = q.pb_w, h = q.pb_h;
    bool ok = q.satd_row < n_rows && w >= 4 && w <= 64 && !(w & (w - 1)) && h >= 4 && h <= 64 && !(h & (h - 1)) &&
              q.mpm[0] <= 33 && q.mpm[1] <= 33 && q.range >= 256 && q.range <= 511 &&
              q.sqrt_lambda >= 0.0 && q.sqrt_lambda <= 1e300;
#pragma unroll
    for (int k = 0; k < 7; k++) ok = ok && (q.ctx[k] & 2047) >= 8;     // a non-zero LPS range
    if (!ok) {                       // outside the supported domain: no list, count 255
        for (int k = 0; k < 5; k++) o.list[k] = -1;
        o.count = 255;
        out[i] = o;
        return;
    }
    const u32 *satd = satd_all + (size_t)q.satd_row * 33;
    RmdState S;
    S.cost = s_cost;
    S.list = s_list;
    S.t = threadIdx.x;
    for (int k = 0; k < 33; k++) { S.set_l(k, -1); s_cost[k][S.t] = RMD_MAX_COST; }
    int cnt = (w >= h * 4 || h >= w * 4) ? 4 : 5;
    if (q.fast) {
        const int r4[10] = { 0, 1, 2, 6, 10, 14, 18, 22, 26, 30 };
        u64 map = 0;                                     // ipm_check_map as bits
        for (int k = 0; k < 10; k++) map |= 1ull << r4[k];
        for (int k = q.skip_ipd ? 3 : 0; k < 10; k++) rmd_check(S, q, satd, r4[k], k + 1);
        int r2[12], n2 = 0;
        for (int k = 0; k < 7; k++) {
            const int ipm = S.l(k);
            if (ipm >= 6) {
                if (!(map >> (ipm - 2) & 1)) { r2[n2++] = ipm - 2; map |= 1ull << (ipm - 2); }
                if (!(map >> (ipm + 2) & 1)) { r2[n2++] = ipm + 2; map |= 1ull << (ipm + 2); }
            }
        }
        for (int k = 0; k < n2; k++) rmd_check(S, q, satd, r2[k], max(cnt, 3));
        int r1[8], n1 = 0;
        for (int k = 0, j = 0; k < 3 && j < 10;) {
            const int ipm = S.l(j++);
            if (ipm >= 4) {
                k++;
                if (!(map >> (ipm - 1) & 1)) { r1[n1++] = ipm - 1; map |= 1ull << (ipm - 1); }
                if (ipm + 1 < 33 && !(map >> (ipm + 1) & 1)) { r1[n1++] = ipm + 1; map |= 1ull << (ipm + 1); }
            }
        }
        for (int k = 0; k < n1; k++) rmd_check(S, q, satd, r1[k], min(cnt, 5));
        for (int k = 0; k < 2; k++) {
            const int m = q.mpm[k];
            if (m < 33 && !(q.skip_ipd && m <= 2) && !(map >> m & 1)) rmd_check(S, q, satd, m, min(cnt, 5));
        }
    } else {
        for (int m = q.skip_ipd ? 3 : 0; m < 33; m++) rmd_check(S, q, satd, m, cnt);
    }
    // the MPMs the first cnt entries lack replace the last ones
    int need0 = q.mpm[0] != 33 && !(q.skip_ipd && q.mpm[0] <= 2);
    int need1 = q.mpm[1] != 33 && !(q.skip_ipd && q.mpm[1] <= 2);
    for (int k = 0; k < cnt; k++) {
        if (need0 && S.l(k) == q.mpm[0]) need0 = 0;
        if (need1 && S.l(k) == q.mpm[1]) need1 = 0;
    }
    if (need0 && need1) {
        const bool first = S.c(q.mpm[0]) <= S.c(q.mpm[1]);
        S.set_l(cnt - 2, first ? q.mpm[0] : q.mpm[1]);
        S.set_l(cnt - 1, first ? q.mpm[1] : q.mpm[0]);
    } else if (need0 || need1) {
        const int add = need0 ? 0 : 1;
        if (S.l(cnt - 1) == q.mpm[1 - add]) S.set_l(cnt - 2, S.l(cnt - 1));
        S.set_l(cnt - 1, q.mpm[add]);
    }
    // candidates costlier than the inter SATD x threshold leave from the end
    if (q.inter_satd != ~0ull) {
        const double lim = __dmul_rn((double)q.inter_satd, q.satd_threshold);
        while (cnt > 0 && S.l(cnt - 1) >= 0 && __longlong_as_double((long long)S.c(S.l(cnt - 1))) > lim) cnt--;
    }
    for (int k = 0; k < 5; k++) o.list[k] = (s8)S.l(k);
    o.count = (u8)cnt;
    out[i] = o;
}

int launch_intra_rmd(const u32 *satd, unsigned long long n_rows, const void *reqs, int n, void *out, cudaStream_t st)
{
    if (!satd || n < 0 || (n > 0 && (!reqs || !out))) return set_status(UC_ERR_ARG, "intra_rmd: null argument");
    if (n == 0) return UC_OK;
    k_intra_rmd<<<(unsigned)((n + RMD_THREADS - 1) / RMD_THREADS), RMD_THREADS, 0, st>>>(satd, n_rows,
                                                                                       (const RmdReq *)reqs, n,
                                                                                       (RmdOut *)out);
    UC_CHECK(cudaGetLastError());
    count_launch(1);
    return UC_OK;
}

struct RmdScratch {
    std::mutex mu;
    cudaStream_t st = nullptr;
    void *buf = nullptr;
    size_t cap = 0;
};
static RmdScratch g_rmd[64];

}  // namespace uc

using namespace uc;

extern "C" UAVS3E_CUDA_API int uavs3e_cuda_intra_rmd(const uint32_t *satd, size_t n_rows,
                                                    const uavs3e_cuda_rmd_req_t *reqs, int n,
                                                    uavs3e_cuda_rmd_out_t *out)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (!satd || n < 0 || (n > 0 && (!reqs || !out))) return set_status(UC_ERR_ARG, "intra_rmd: bad argument");
    if (n == 0) return UC_OK;
    int dev = 0;
    UC_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_status(UC_ERR_UNSUPPORTED, "intra_rmd: device index");
    RmdScratch &S = g_rmd[dev];
    std::lock_guard<std::mutex> lk(S.mu);
    if (!S.st) UC_CHECK(cudaStreamCreateWithFlags(&S.st, cudaStreamNonBlocking));
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t b_satd = up(n_rows * 33 * sizeof(uint32_t)), b_req = up((size_t)n * sizeof(*reqs));
    const size_t need = b_satd + b_req + up((size_t)n * sizeof(*out));
    if (S.cap < need) {
        if (S.buf) UC_CHECK(cudaFree(S.buf));
        S.buf = nullptr;
        S.cap = 0;
        UC_CHECK(cudaMalloc(&S.buf, need));
        S.cap = need;
    }
    char *b = (char *)S.buf;
    u32 *d_satd = (u32 *)b;
    void *d_req = b + b_satd, *d_out = b + b_satd + b_req;
    UC_CHECK(cudaMemcpyAsync(d_satd, satd, n_rows * 33 * sizeof(uint32_t), cudaMemcpyHostToDevice, S.st));
    UC_CHECK(cudaMemcpyAsync(d_req, reqs, (size_t)n * sizeof(*reqs), cudaMemcpyHostToDevice, S.st));
    rc = launch_intra_rmd(d_satd, n_rows, d_req, n, d_out, S.st);
    if (rc) return rc;
    UC_CHECK(cudaMemcpyAsync(out, d_out, (size_t)n * sizeof(*out), cudaMemcpyDeviceToHost, S.st));
    UC_CHECK(cudaStreamSynchronize(S.st));
    return UC_OK;
}

extern "C" UAVS3E_CUDA_API int uavs3e_cuda_intra_rmd_device(const uint32_t *d_satd, size_t n_rows,
                                                           const uavs3e_cuda_rmd_req_t *d_reqs, int n,
                                                           uavs3e_cuda_rmd_out_t *d_out, void *stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    return launch_intra_rmd(d_satd, n_rows, d_reqs, n, d_out, (cudaStream_t)stream);
}
