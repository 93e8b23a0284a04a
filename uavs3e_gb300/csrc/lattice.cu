// Batched intra lattice: for every CU of a frame's QT/BT lattice and every luma intra mode,
// prediction -> SATD -> residual -> forward DCT2 -> (per QP) quantisation -> dequantisation ->
// inverse DCT2 -> reconstruction -> SSD, bit-exact with the encoder's functions
// (com_intra_get_nbr src/com_ipred.c:40, com_intra_pred :733, calc_satd_intra src/util.c:200,
// trans_dct2 src/transform.c:253-412, quant_check / quant_rdoq src/com_itdq.c:910-954 with the
// rdoq_quant_block parameters src/quant.c:196-231, com_dquant src/com_itdq.c:807,
// itrans_dct2 :264-423, com_recon src/com_util.c:3107).
//
// The whole lattice of a frame is one launch of a persistent kernel walking a device work queue.
// A classify kernel counts the CUs of each of the 25 power-of-two shape classes (4..64 per side),
// a planning kernel turns the counts into each class's run of tiles (a tile = several whole CUs,
// or one CU and a chunk of its modes, per the class's shared-memory layout) in the order largest
// CUs first, a scatter kernel lists the CUs per class, and the persistent CTAs then take tiles
// from a global counter until the queue is empty, each running the compile-time body of the
// tile's class.  Nothing waits on the host between the launches, so a frame's intra lattice can
// be captured into one CUDA graph.  Within a tile every stage is a flat loop over (job,
// element), and per-job sums are reduced across the lanes of a warp before one shared-memory
// atomic.  An autotuner picks each class's layout (how many CUs or which mode chunk a tile
// takes) under a common shared-memory size, by timing the queue restricted to that class.
//
// Transforms are products with the folded DCT2 matrices (identical results to the encoder's
// partial butterflies) on the byte/halfword dot-product instructions: the forward row pass is
// the CU's org part (computed once per CU) minus a dp4a product with the u8 prediction; the
// column pass and both inverse passes are dp2a products of s16 pairs with s8 matrix rows.
#include "lattice_kernel.cuh"

#include <mutex>
#include "../../include/uavs3e_cuda.h"

#include <algorithm>

namespace uc {

// shape class of a CU: (log2 w - 2) * 5 + (log2 h - 2), or -1 outside the supported set
// (power-of-two sides 4..64 inside the picture, on the 4x4 grid the encoder's CUs lie on)
__device__ __forceinline__ int lat_class(const LatCu &cu, int W, int H)
{
    const int w = cu.w, h = cu.h;
    if (w < 4 || w > 64 || h < 4 || h > 64 || (w & (w - 1)) || (h & (h - 1)) || cu.x < 0 || cu.y < 0 ||
        (cu.x & 3) || (cu.y & 3) || cu.x + w > W || cu.y + h > H)
        return -1;
    return (ilog2d(w) - 2) * 5 + (ilog2d(h) - 2);
}

// CUs per thread in the shape-grouping kernels; blocks of 256 threads count in shared memory
// and touch each global counter once
constexpr int LAT_GROUP_K = 4;

// counts CUs per shape; a CU outside the supported set gets zeroed outputs here
__global__ void __launch_bounds__(256) k_lat_count(const LatCu *cus, int n, int W, int H, int n_qp, int *counts,
                                                   u32 *satd_out, LatQ *q_out)
{
    __shared__ int s_cnt[32];
    if (threadIdx.x < 32) s_cnt[threadIdx.x] = 0;
    __syncthreads();
    for (int k = 0; k < LAT_GROUP_K; k++) {
        const int i = (blockIdx.x * LAT_GROUP_K + k) * blockDim.x + threadIdx.x;
        if (i >= n) break;
        const int c = lat_class(cus[i], W, H);
        if (c >= 0) {
            atomicAdd(&s_cnt[c], 1);
            continue;
        }
        for (int m = 0; m < 33; m++) {
            satd_out[(size_t)i * 33 + m] = 0;
            for (int q = 0; q < n_qp; q++) q_out[((size_t)i * 33 + m) * n_qp + q] = LatQ{};
        }
    }
    __syncthreads();
    if (threadIdx.x < LAT_SHAPES && s_cnt[threadIdx.x]) atomicAdd(&counts[threadIdx.x], s_cnt[threadIdx.x]);
}

// lists the CUs of each shape (order within a shape is irrelevant: outputs go by CU index):
// a block reserves one range per shape, its threads fill it
__global__ void __launch_bounds__(256) k_lat_scatter(const LatCu *cus, int n, int W, int H, const int *offsets,
                                                     int *cursor, int *perm)
{
    __shared__ int s_cnt[32], s_base[32];
    if (threadIdx.x < 32) s_cnt[threadIdx.x] = 0;
    __syncthreads();
    int cls[LAT_GROUP_K], rank[LAT_GROUP_K];
#pragma unroll
    for (int k = 0; k < LAT_GROUP_K; k++) {
        const int i = (blockIdx.x * LAT_GROUP_K + k) * blockDim.x + threadIdx.x;
        cls[k] = i < n ? lat_class(cus[i], W, H) : -1;
        rank[k] = cls[k] >= 0 ? atomicAdd(&s_cnt[cls[k]], 1) : 0;
    }
    __syncthreads();
    if (threadIdx.x < LAT_SHAPES && s_cnt[threadIdx.x])
        s_base[threadIdx.x] = offsets[threadIdx.x] + atomicAdd(&cursor[threadIdx.x], s_cnt[threadIdx.x]);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < LAT_GROUP_K; k++) {
        const int i = (blockIdx.x * LAT_GROUP_K + k) * blockDim.x + threadIdx.x;
        if (cls[k] >= 0) perm[s_base[cls[k]] + rank[k]] = i;
    }
}

// plans the queue of one launch: exclusive offsets of the classes' CUs in perm, the classes'
// tile runs in launch order (only the classes in the mask), the cursors and the tile counter reset
struct LatPlan { int tiles_per_cu[LAT_SHAPES], nchunk[LAT_SHAPES]; u32 mask; };

__global__ void k_lat_plan(int *counters, const LatPlan Q)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int *counts = counters, *cursor = counters + 32, *cu_off = counters + 64, *tile_off = counters + 96;
    int o = 0;
    for (int c = 0; c < LAT_SHAPES; c++) { cu_off[c] = o; o += counts[c]; cursor[c] = 0; }
    int t = 0;
    for (int r = 0; r < LAT_SHAPES; r++) {
        const int c = lat_order(r);
        tile_off[r] = t;
        if ((Q.mask >> c) & 1) t += (counts[c] + Q.tiles_per_cu[c] - 1) / Q.tiles_per_cu[c] * Q.nchunk[c];
    }
    tile_off[LAT_SHAPES] = t;
    counters[127] = 0;      // the tile counter
}

// the persistent lattice: tiles from the queue until it is empty.  Its static shared memory is
// the tile's LatShared and one word: with a 48 KB layout, four CTAs then still fit an SM (the
// queue's tile offsets are read from global memory, not copied to shared memory, for that)
__global__ void __launch_bounds__(LAT_THREADS, 4) k_intra_lattice(const __grid_constant__ LatParams P)
{
    extern __shared__ __align__(16) u8 sm[];
    __shared__ LatShared S;
    __shared__ int s_t;
    const int tid = threadIdx.x;
    const int total = __ldg(P.tile_off + LAT_SHAPES);
    if (tid == 0) S.tables = -1;
    for (;;) {
        if (tid == 0) s_t = atomicAdd(P.next, 1);
        __syncthreads();
        const int t = s_t;
        __syncthreads();
        if (t >= total) break;
        int r = 0;
        while (t >= __ldg(P.tile_off + r + 1)) r++;
        const int c = lat_order(r), lt = t - __ldg(P.tile_off + r);
        const int *perm = P.perm + P.cu_off[c];
        const int n = P.counts[c];
        switch (c) {
#define LAT_CASE(lw, lh) case ((lw) - 2) * 5 + ((lh) - 2): lat_tile<lw, lh>(P, perm, n, lt, sm, S); break;
#define LAT_ROW(lw) LAT_CASE(lw, 2) LAT_CASE(lw, 3) LAT_CASE(lw, 4) LAT_CASE(lw, 5) LAT_CASE(lw, 6)
            LAT_ROW(2) LAT_ROW(3) LAT_ROW(4) LAT_ROW(5) LAT_ROW(6)
#undef LAT_ROW
#undef LAT_CASE
        default: break;
        }
    }
}

size_t lattice_smem_bytes(int w, int h, int nm)
{
    int lw = 0, lh = 0;
    while ((1 << lw) < w) lw++;
    while ((1 << lh) < h) lh++;
    LatLayout L;
    lat_layout(lw, lh, nm, LAT_BUDGET, L);
    return (size_t)L.smem;
}

// Autotuning of the tile layouts: per device and mode count, the first call with at least
// LAT_TUNE_MIN_CUS CUs of a class times the queue restricted to that class for each distinct
// layout the candidate budgets give (every run writes the same records) and keeps the fastest.
// All budgets are at most LAT_BUDGET, the launch's shared-memory size, so four CTAs share an SM.
constexpr int LAT_TUNE_MIN_CUS = 512;
static const int kLatBudgets[] = { 16 * 1024, 24 * 1024, 32 * 1024, 40 * 1024, 48 * 1024 };
struct LatTune {
    std::mutex mu;
    int budget[34][LAT_SHAPES] = {};   // 0: the default LAT_BUDGET (not tuned)
    bool done[34] = {};                // the tuning pass of this mode count has run
};
static LatTune g_tune[64];
static bool g_tune_on = true;

// per device: the CU permutation and the queue's counters
struct LatScratch {
    int *perm = nullptr;
    int *counters = nullptr;   // [0, 32) counts, [32, 64) cursors, [64, 96) CU offsets, [96, 122) tile
                               // offsets, [127] tile counter
    size_t cap = 0;
    int sms = 0, occ = 0;      // SMs and resident CTAs per SM at LAT_BUDGET
};
static LatScratch g_lat[64];

// one launch of the plan + scatter + persistent lattice for the classes in `mask`
static int lat_run(LatParams P, const LatCu *cus, int n_cus, int W, int H, const int *budgets, u32 mask,
                   LatScratch &S, cudaStream_t st, int *launches)
{
    LatPlan Q;
    int smem = 0;
    for (int c = 0; c < LAT_SHAPES; c++) {
        LatLayout L;
        lat_layout(c / 5 + 2, c % 5 + 2, P.n_modes, budgets[c], L);
        Q.tiles_per_cu[c] = L.G; Q.nchunk[c] = L.nchunk;
        if ((mask >> c) & 1) smem = std::max(smem, L.smem);
        P.budget[c] = budgets[c];
    }
    Q.mask = mask;
    if (smem > LAT_SMEM_MAX) return set_status(UC_ERR_ARG, "intra_lattice: shared memory layout");
    k_lat_plan<<<1, 32, 0, st>>>(S.counters, Q);
    UC_CHECK(cudaGetLastError());
    const int nb = (n_cus + 256 * LAT_GROUP_K - 1) / (256 * LAT_GROUP_K);
    k_lat_scatter<<<nb, 256, 0, st>>>(cus, n_cus, W, H, S.counters + 64, S.counters + 32, S.perm);
    UC_CHECK(cudaGetLastError());
    k_intra_lattice<<<S.sms * S.occ, LAT_THREADS, smem, st>>>(P);
    UC_CHECK(cudaGetLastError());
    *launches += 3;
    return UC_OK;
}

// times the lattice restricted to class c for each distinct layout of the candidate budgets
static int lat_tune_class(int c, const LatParams &P, const LatCu *cus, int n_cus, int W, int H, const int *budgets,
                          LatScratch &S, cudaStream_t st, int *launches, int *best_out)
{
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    UC_CHECK(cudaEventCreate(&e0));
    UC_CHECK(cudaEventCreate(&e1));
    float best_ms = 3.0e38f;
    int best = LAT_BUDGET, seen = 0, seen_g[8], seen_mc[8];
    int bud[LAT_SHAPES];
    for (int k = 0; k < LAT_SHAPES; k++) bud[k] = budgets[k];
    for (int b : kLatBudgets) {
        LatLayout L;
        lat_layout(c / 5 + 2, c % 5 + 2, P.n_modes, b, L);
        if (L.smem > LAT_BUDGET || L.G < 1) continue;
        bool dup = false;
        for (int k = 0; k < seen; k++) dup |= seen_g[k] == L.G && seen_mc[k] == L.MC;
        if (dup) continue;
        seen_g[seen] = L.G; seen_mc[seen] = L.MC; seen++;
        bud[c] = b;
        float ms = 3.0e38f;
        for (int rep = 0; rep < 2; rep++) {
            UC_CHECK(cudaEventRecord(e0, st));
            int r = lat_run(P, cus, n_cus, W, H, bud, 1u << c, S, st, launches);
            if (r) { cudaEventDestroy(e0); cudaEventDestroy(e1); return r; }
            UC_CHECK(cudaEventRecord(e1, st));
            UC_CHECK(cudaEventSynchronize(e1));
            float t = 0;
            UC_CHECK(cudaEventElapsedTime(&t, e0, e1));
            ms = t < ms ? t : ms;
        }
        if (ms < best_ms) { best_ms = ms; best = b; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *best_out = best;
    return UC_OK;
}

int launch_intra_lattice(const pel *org, int i_org, const pel *rec, int i_rec, int W, int H, const LatCu *cus,
                         int n_cus, const u8 *modes, int n_modes, int ipf, const int *qps, int n_qp, int is_intra,
                         u32 *satd_out, LatQ *q_out, cudaStream_t st)
{
    int dev = 0;
    UC_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_status(UC_ERR_UNSUPPORTED, "intra_lattice: device index");
    const DevTables *tab = device_tables(dev);
    if (!tab) return set_status(UC_ERR_MEMORY, "intra_lattice: table upload failed");
    if (n_qp < 0 || n_qp > LAT_MAX_QP || n_cus < 0 || (n_qp > 0 && !q_out))
        return set_status(UC_ERR_ARG, "intra_lattice: bad qp count");
    if (n_modes < 1 || n_modes > 33 || (!modes && n_modes != 33))
        return set_status(UC_ERR_ARG, "intra_lattice: mode list");
    for (int i = 0; i < n_qp; i++)
        if (qps[i] < 0 || qps[i] > 63) return set_status(UC_ERR_ARG, "intra_lattice: qp out of range");
    if (n_cus == 0) return UC_OK;
    LatScratch &S = g_lat[dev];
    if (!S.counters) {
        UC_CHECK(cudaDeviceGetAttribute(&S.sms, cudaDevAttrMultiProcessorCount, dev));
        UC_CHECK(cudaFuncSetAttribute(k_intra_lattice, cudaFuncAttributeMaxDynamicSharedMemorySize, LAT_SMEM_MAX));
        UC_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&S.occ, k_intra_lattice, LAT_THREADS, LAT_BUDGET));
        S.occ = std::max(S.occ, 1);      // 4 on GB300 (64 registers, 56 KB of shared memory per CTA)
        UC_CHECK(cudaMalloc(&S.counters, 128 * sizeof(int)));
    }
    if (S.cap < (size_t)n_cus) {
        if (S.perm) UC_CHECK(cudaFree(S.perm));
        S.perm = nullptr;
        UC_CHECK(cudaMalloc(&S.perm, (size_t)n_cus * sizeof(int)));
        S.cap = (size_t)n_cus;
    }
    prof_begin(PROF_LATTICE, st);
    UC_CHECK(cudaMemsetAsync(S.counters, 0, 128 * sizeof(int), st));
    const int nb = (n_cus + 256 * LAT_GROUP_K - 1) / (256 * LAT_GROUP_K);
    k_lat_count<<<nb, 256, 0, st>>>(cus, n_cus, W, H, n_qp, S.counters, satd_out, q_out);
    UC_CHECK(cudaGetLastError());
    int launches = 1;
    LatParams P;
    memset(&P, 0, sizeof(P));
    P.org = org; P.i_org = i_org; P.rec = rec; P.i_rec = i_rec; P.W = W; P.H = H;
    P.org_words = ((uintptr_t)org % 4 == 0 && i_org % 4 == 0) ? 1 : 0;
    P.cus = cus; P.ipf = ipf; P.n_qp = n_qp; P.is_intra = is_intra;
    for (int i = 0; i < LAT_MAX_QP; i++) P.qp[i] = i < n_qp ? qps[i] : 0;
    P.satd_out = satd_out; P.q_out = q_out;
    P.modes = modes; P.n_modes = n_modes;
    P.sq32 = sqrt(32.0); P.sq128 = sqrt(128.0);
    P.k32 = had_scale_k(P.sq32); P.k128 = had_scale_k(P.sq128);
    for (int l = 0; l < 7; l++) {
        P.fold[l] = tab->fold[l];
        for (int m = 0; m < 7; m++) P.scanpos[l][m] = tab->scanpos[l][m];
    }
    P.counts = S.counters; P.cu_off = S.counters + 64; P.tile_off = S.counters + 96; P.perm = S.perm;
    P.next = S.counters + 127;
    // the classes' layouts: tuned on the first call with QPs per device and mode count (that call
    // waits for the CU counts and times the candidates of every class with enough CUs; later
    // calls, and every SATD-only call, do not wait -- make the first call before any capture)
    int budgets[LAT_SHAPES];
    {
        LatTune &T = g_tune[dev];
        std::lock_guard<std::mutex> lk(T.mu);
        for (int c = 0; c < LAT_SHAPES; c++) budgets[c] = T.budget[n_modes][c] ? T.budget[n_modes][c] : LAT_BUDGET;
        if (g_tune_on && !T.done[n_modes] && n_qp > 0) {
            T.done[n_modes] = true;   // one pass: classes with too few CUs keep the default
            int counts[32];
            UC_CHECK(cudaMemcpyAsync(counts, S.counters, 32 * sizeof(int), cudaMemcpyDeviceToHost, st));
            UC_CHECK(cudaStreamSynchronize(st));
            for (int c = 0; c < LAT_SHAPES; c++) {
                if (T.budget[n_modes][c] || counts[c] < LAT_TUNE_MIN_CUS) continue;
                int best = LAT_BUDGET;
                int r = lat_tune_class(c, P, cus, n_cus, W, H, budgets, S, st, &launches, &best);
                if (r) return r;
                T.budget[n_modes][c] = budgets[c] = best;
            }
        }
    }
    int r = lat_run(P, cus, n_cus, W, H, budgets, (1u << LAT_SHAPES) - 1, S, st, &launches);
    if (r) return r;
    count_launch(launches);
    prof_end(PROF_LATTICE, st);
    return UC_OK;
}

// host-buffer entry: per device, the device copies of the inputs and outputs (grown as needed)
// and a stream of its own; calls on one device are serialised by its mutex
constexpr int LAT_HOST_CHUNKS = 4;       // CU ranges whose record downloads overlap the next range's lattice
constexpr int LAT_HOST_CHUNK_MIN = 65536; // CUs below which a call runs as one range

struct LatHost {
    std::mutex mu;
    cudaStream_t st = nullptr;               // the lattice launches
    cudaStream_t cp = nullptr;               // the record downloads
    cudaEvent_t ev[LAT_HOST_CHUNKS] = {};
    u8 *org = nullptr, *rec = nullptr;
    LatCu *cus = nullptr;
    u32 *satd = nullptr;
    LatQ *q = nullptr;
    size_t org_cap = 0, rec_cap = 0, cu_cap = 0, satd_cap = 0, q_cap = 0;   // elements
};
static LatHost g_lat_host[64];

template <typename T> static int grow(T **p, size_t *cap, size_t n)
{
    if (*cap >= n) return UC_OK;
    if (*p) UC_CHECK(cudaFree(*p));
    *p = nullptr;
    *cap = 0;
    UC_CHECK(cudaMalloc((void **)p, n * sizeof(T)));
    *cap = n;
    return UC_OK;
}

}  // namespace uc

using namespace uc;

static_assert(sizeof(LatCu) == sizeof(uavs3e_cuda_cu_t), "cu record layout");
static_assert(sizeof(LatQ) == sizeof(uavs3e_cuda_lat_q_t), "lattice record layout");

extern "C" {

UAVS3E_CUDA_API void uavs3e_cuda_lattice_autotune(int on) { g_tune_on = on != 0; }

UAVS3E_CUDA_API int uavs3e_cuda_lattice_budgets(int n_modes, int out[25])
{
    if (!out || n_modes < 1 || n_modes > 33) return set_status(UC_ERR_ARG, "lattice_budgets: bad argument");
    int dev = 0;
    UC_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_status(UC_ERR_UNSUPPORTED, "lattice_budgets: device index");
    LatTune &T = g_tune[dev];
    std::lock_guard<std::mutex> lk(T.mu);
    for (int c = 0; c < 25; c++) out[c] = T.budget[n_modes][c];
    return UC_OK;
}

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

UAVS3E_CUDA_API int uavs3e_cuda_intra_lattice_modes_device(const uint8_t *d_org, int i_org, const uint8_t *d_rec,
                                                           int i_rec, int width, int height,
                                                           const uavs3e_cuda_cu_t *d_cus, int n_cus,
                                                           const uint8_t *d_modes, int n_modes, int ipf, const int *qps,
                                                           int n_qp, int is_intra_slice, uint32_t *d_satd,
                                                           uavs3e_cuda_lat_q_t *d_q, void *stream)
{
    int r = ensure_init();
    if (r) return r;
    if (!d_org || !d_rec || !d_cus || !d_satd || (n_qp > 0 && (!d_q || !qps)))
        return set_status(UC_ERR_ARG, "intra_lattice: null pointer");
    if (width % 4 || height % 4) return set_status(UC_ERR_ARG, "intra_lattice: picture size must be a multiple of 4");
    return launch_intra_lattice(d_org, i_org, d_rec, i_rec, width, height, (const LatCu *)d_cus, n_cus, d_modes, n_modes,
                                ipf, qps, n_qp, is_intra_slice, d_satd, (LatQ *)d_q, (cudaStream_t)stream);
}

UAVS3E_CUDA_API int uavs3e_cuda_intra_lattice(const uint8_t *org, int i_org, const uint8_t *rec, int i_rec, int width,
                                              int height, const uavs3e_cuda_cu_t *cus, int n_cus, int ipf,
                                              const int *qps, int n_qp, int is_intra_slice, uint32_t *satd,
                                              uavs3e_cuda_lat_q_t *q)
{
    int r = ensure_init();
    if (r) return r;
    if (!org || !rec || !cus || !satd || (n_qp > 0 && (!q || !qps)) || n_cus < 0)
        return set_status(UC_ERR_ARG, "intra_lattice: null pointer");
    if (width <= 0 || height <= 0 || width % 4 || height % 4 || i_org < width || i_rec < width)
        return set_status(UC_ERR_ARG, "intra_lattice: picture size must be a positive multiple of 4");
    if (n_qp < 0 || n_qp > LAT_MAX_QP) return set_status(UC_ERR_ARG, "intra_lattice: bad qp count");
    if (n_cus == 0) return UC_OK;
    int dev = 0;
    UC_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_status(UC_ERR_UNSUPPORTED, "intra_lattice: device index");
    LatHost &S = g_lat_host[dev];
    std::lock_guard<std::mutex> lk(S.mu);
    if (!S.st) UC_CHECK(cudaStreamCreateWithFlags(&S.st, cudaStreamNonBlocking));
    const size_t pic = (size_t)width * height;
    const size_t nq = (size_t)n_cus * 33 * (size_t)(n_qp > 0 ? n_qp : 1);
    if ((r = grow(&S.org, &S.org_cap, pic)) || (r = grow(&S.rec, &S.rec_cap, pic)) ||
        (r = grow(&S.cus, &S.cu_cap, (size_t)n_cus)) || (r = grow(&S.satd, &S.satd_cap, (size_t)n_cus * 33)) ||
        (r = grow(&S.q, &S.q_cap, nq)))
        return r;
    if (!S.cp) {
        UC_CHECK(cudaStreamCreateWithFlags(&S.cp, cudaStreamNonBlocking));
        for (int c = 0; c < LAT_HOST_CHUNKS; c++) UC_CHECK(cudaEventCreateWithFlags(&S.ev[c], cudaEventDisableTiming));
    }
    UC_CHECK(cudaMemcpy2DAsync(S.org, width, org, i_org, width, height, cudaMemcpyHostToDevice, S.st));
    UC_CHECK(cudaMemcpy2DAsync(S.rec, width, rec, i_rec, width, height, cudaMemcpyHostToDevice, S.st));
    UC_CHECK(cudaMemcpyAsync(S.cus, cus, (size_t)n_cus * sizeof(LatCu), cudaMemcpyHostToDevice, S.st));
    // the records of a large call come back in CU ranges: range c's download (copy stream) overlaps
    // range c + 1's lattice (compute stream); a range's records are contiguous because records go
    // by CU index
    const int nqp = n_qp > 0 ? n_qp : 0;
    const int chunks = n_cus >= LAT_HOST_CHUNKS * LAT_HOST_CHUNK_MIN ? LAT_HOST_CHUNKS : 1;
    for (int c = 0; c < chunks; c++) {
        const int a = (int)((long long)n_cus * c / chunks), b = (int)((long long)n_cus * (c + 1) / chunks);
        r = launch_intra_lattice(S.org, width, S.rec, width, width, height, S.cus + a, b - a, nullptr, 33, ipf, qps,
                                 n_qp, is_intra_slice, S.satd + (size_t)a * 33,
                                 nqp > 0 ? S.q + (size_t)a * 33 * nqp : nullptr, S.st);
        if (r) {
            cudaStreamSynchronize(S.cp);
            return r;
        }
        UC_CHECK(cudaEventRecord(S.ev[c], S.st));
        UC_CHECK(cudaStreamWaitEvent(S.cp, S.ev[c], 0));
        UC_CHECK(cudaMemcpyAsync(satd + (size_t)a * 33, S.satd + (size_t)a * 33, (size_t)(b - a) * 33 * sizeof(u32),
                                 cudaMemcpyDeviceToHost, S.cp));
        if (nqp > 0)
            UC_CHECK(cudaMemcpyAsync(q + (size_t)a * 33 * nqp, S.q + (size_t)a * 33 * nqp,
                                     (size_t)(b - a) * 33 * nqp * sizeof(LatQ), cudaMemcpyDeviceToHost, S.cp));
    }
    UC_CHECK(cudaStreamSynchronize(S.cp));
    UC_CHECK(cudaStreamSynchronize(S.st));
    return UC_OK;
}

UAVS3E_CUDA_API int uavs3e_cuda_intra_lattice_device(const uint8_t *d_org, int i_org, const uint8_t *d_rec, int i_rec,
                                                     int width, int height, const uavs3e_cuda_cu_t *d_cus, int n_cus,
                                                     int ipf, const int *qps, int n_qp, int is_intra_slice,
                                                     uint32_t *d_satd, uavs3e_cuda_lat_q_t *d_q, void *stream)
{
    return uavs3e_cuda_intra_lattice_modes_device(d_org, i_org, d_rec, i_rec, width, height, d_cus, n_cus, nullptr, 33,
                                                  ipf, qps, n_qp, is_intra_slice, d_satd, d_q, stream);
}

}  // extern "C"

// per-stage SM cycles of the lattice tiles since the last clear, [25 classes][10 stages] (a
// library built with UAVS3E_LAT_STAGE_CLOCKS; otherwise UC_ERR_UNSUPPORTED, nothing written)
UAVS3E_CUDA_API int uavs3e_cuda_lattice_stage_clocks(unsigned long long *out, int clear)
{
#ifdef UAVS3E_LAT_STAGE_CLOCKS
    if (!out) return UC_ERR_ARG;
    if (cudaMemcpyFromSymbol(out, uc::g_lat_stage_clk, sizeof(uc::g_lat_stage_clk)) != cudaSuccess) return UC_ERR_CUDA;
    if (clear) {
        static unsigned long long zero[uc::LAT_SHAPES][uc::LAT_STAGES];
        if (cudaMemcpyToSymbol(uc::g_lat_stage_clk, zero, sizeof(zero)) != cudaSuccess) return UC_ERR_CUDA;
    }
    return UC_OK;
#else
    (void)out; (void)clear;
    return UC_ERR_UNSUPPORTED;
#endif
}
