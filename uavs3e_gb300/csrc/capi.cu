// C ABI of libuavs3e_cuda: library state, status, frame interpolation and the batched
// motion-search session (include/uavs3e_cuda.h).
#include "common.cuh"
#include "tma.cuh"
#include "uavs3e_cuda_internal.h"
#include "../../include/uavs3e_cuda.h"

#include <cudaTypedefs.h>
#include <mutex>
#include <stdio.h>
#include <string.h>
#include <vector>

namespace uc {

static std::mutex g_mu;
static int g_status = UC_OK;
static char g_status_text[256] = "ok";
static int g_device = -1;

int set_status(int code, const char *what)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_status == UC_OK && code != UC_OK) {
        g_status = code;
        snprintf(g_status_text, sizeof(g_status_text), "%s", what ? what : "error");
    }
    return code;
}

int check_cuda(cudaError_t e, const char *what)
{
    char buf[200];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return set_status(UC_ERR_CUDA, buf);
}

int ensure_init()
{
    if (g_device >= 0) {
        UC_CHECK(cudaSetDevice(g_device));
        return UC_OK;
    }
    return uavs3e_cuda_init(0);
}

// edge replication of a padded plane (com_img_padding with ext_size 0, one plane)
__global__ void k_pad_plane(pel *p, int W, int H, int pad, int stride)
{
    const int tw = W + 2 * pad, th = H + 2 * pad;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)tw * th;
         i += (long long)gridDim.x * blockDim.x) {
        int x = (int)(i % tw) - pad, y = (int)(i / tw) - pad;
        if (x >= 0 && x < W && y >= 0 && y < H) continue;
        int cx = min(max(x, 0), W - 1), cy = min(max(y, 0), H - 1);
        p[(long long)y * stride + x] = p[(long long)cy * stride + cx];
    }
}

// ---- kernel timing: pairs of events recorded around launches while profiling is on
static bool g_prof = false;
static unsigned long long g_launches = 0;   // kernels launched by this library

void count_launch(int n)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_launches += (unsigned long long)n;
}
static std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_prof_ev[PROF_N];
static std::vector<cudaEvent_t> g_prof_open[PROF_N];
static std::vector<cudaEvent_t> g_ev_pool;

static cudaEvent_t prof_event()
{
    if (!g_ev_pool.empty()) { cudaEvent_t e = g_ev_pool.back(); g_ev_pool.pop_back(); return e; }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// a stream being captured into a graph records no timing events
static bool capturing(cudaStream_t st)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone;
}

void prof_begin(int k, cudaStream_t st)
{
    if (!g_prof || capturing(st)) return;
    std::lock_guard<std::mutex> lk(g_mu);
    cudaEvent_t e = prof_event();
    cudaEventRecord(e, st);
    g_prof_open[k].push_back(e);
}

void prof_end(int k, cudaStream_t st)
{
    if (!g_prof || capturing(st)) return;
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_prof_open[k].empty()) return;
    cudaEvent_t b = g_prof_open[k].back();
    g_prof_open[k].pop_back();
    cudaEvent_t e = prof_event();
    cudaEventRecord(e, st);
    g_prof_ev[k].push_back({ b, e });
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link against libcuda)
static PFN_cuTensorMapEncodeTiled_v12000 g_encode_tiled = nullptr;
static std::once_flag g_encode_once;

int encode_tensor_map_u8(CUtensorMap *map, const void *base, uint64_t row_bytes, uint64_t rows, uint64_t pitch,
                         uint32_t box_w, uint32_t box_h)
{
    std::call_once(g_encode_once, [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            g_encode_tiled = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    });
    if (!g_encode_tiled) return set_status(UC_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
    if (((uintptr_t)base & 15) || (pitch & 15) || (box_w & 15) || box_w > 256 || box_h > 256 || !box_w || !box_h)
        return set_status(UC_ERR_ARG, "tensor map: alignment or box size");
    const cuuint64_t dims[2] = { row_bytes, rows };
    const cuuint64_t strides[1] = { pitch };
    const cuuint32_t box[2] = { box_w, box_h };
    const cuuint32_t elem[2] = { 1, 1 };
    const CUresult r = g_encode_tiled(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void *>(base), dims, strides,
                                      box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_status(UC_ERR_ARG, "cuTensorMapEncodeTiled failed");
    return UC_OK;
}

int launch_pad_plane(pel *p, int W, int H, int pad, int stride, cudaStream_t st)
{
    if (!p || W <= 0 || H <= 0 || pad < 0 || stride < W + 2 * pad) return set_status(UC_ERR_ARG, "pad_plane: bad geometry");
    if (pad == 0) return UC_OK;
    long long n = (long long)(W + 2 * pad) * (H + 2 * pad);
    int blocks = (int)std::min<long long>((n + 255) / 256, 152 * 16);
    prof_begin(PROF_PAD, st);
    k_pad_plane<<<blocks, 256, 0, st>>>(p, W, H, pad, stride);
    count_launch(1);
    prof_end(PROF_PAD, st);
    UC_CHECK(cudaGetLastError());
    return UC_OK;
}

}  // namespace uc

using namespace uc;

extern "C" {

UAVS3E_CUDA_API int uavs3e_cuda_init(int device)
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return set_status(UC_ERR_NOT_INIT, "uavs3e_cuda_init: no CUDA device");
    if (device < 0 || device >= n) return set_status(UC_ERR_ARG, "uavs3e_cuda_init: bad device index");
    UC_CHECK(cudaSetDevice(device));
    g_device = device;
    return UC_OK;
}

UAVS3E_CUDA_API int uavs3e_cuda_status(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    return g_status;
}

UAVS3E_CUDA_API const char *uavs3e_cuda_status_string(void) { return g_status_text; }

UAVS3E_CUDA_API void uavs3e_cuda_clear_status(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_status = UC_OK;
    snprintf(g_status_text, sizeof(g_status_text), "ok");
}

UAVS3E_CUDA_API const char *uavs3e_cuda_version(void) { return "uavs3e_cuda 0.1 (sm_103a)"; }

UAVS3E_CUDA_API unsigned long long uavs3e_cuda_launch_count(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    return g_launches;
}

UAVS3E_CUDA_API void uavs3e_cuda_profile_enable(int on)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_prof = on != 0;
}

UAVS3E_CUDA_API int uavs3e_cuda_profile_collect(double ms[], int counts[], int n)
{
    std::lock_guard<std::mutex> lk(g_mu);
    for (int k = 0; k < PROF_N; k++) {
        double tot = 0;
        for (auto &pr : g_prof_ev[k]) {
            float t = 0;
            if (cudaEventSynchronize(pr.second) == cudaSuccess && cudaEventElapsedTime(&t, pr.first, pr.second) == cudaSuccess)
                tot += t;
            g_ev_pool.push_back(pr.first);
            g_ev_pool.push_back(pr.second);
        }
        if (k < n) { ms[k] = tot; counts[k] = (int)g_prof_ev[k].size(); }
        g_prof_ev[k].clear();
    }
    return UC_OK;
}

UAVS3E_CUDA_API int uavs3e_cuda_subpel_planes(const uint8_t *d_plane0, uint8_t *const d_planes[15], int width,
                                              int height, int pad, int stride, void *stream)
{
    int r = ensure_init();
    if (r) return r;
    if (!d_planes) return set_status(UC_ERR_ARG, "subpel_planes: null plane list");
    PlaneSet15 ps;
    for (int i = 0; i < 15; i++) ps.p[i] = d_planes[i];
    return launch_subpel_planes(d_plane0, stride, width, height, pad, ps, (cudaStream_t)stream);
}

UAVS3E_CUDA_API int uavs3e_cuda_pad_plane(uint8_t *d_plane0, int width, int height, int pad, int stride, void *stream)
{
    int r = ensure_init();
    if (r) return r;
    return launch_pad_plane(d_plane0, width, height, pad, stride, (cudaStream_t)stream);
}

UAVS3E_CUDA_API int uavs3e_cuda_me_block_table(int out[169][4])
{
    CtuBlock t[ME_BLOCKS_PER_CTU];
    ctu_block_table(t);
    for (int i = 0; i < ME_BLOCKS_PER_CTU; i++) {
        out[i][0] = t[i].x; out[i][1] = t[i].y; out[i][2] = t[i].w; out[i][3] = t[i].h;
    }
    return UC_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ motion-search session

struct uavs3e_cuda_me {
    int W, H, n_refs, range, pad, stride, rows;
    size_t plane_bytes;
    pel *planes_buf = nullptr;        // [n_refs][16][rows*stride]
    pel *org_buf = nullptr;           // W x H for host runs
    pel *ref_stage = nullptr;         // W x H: a new reference's host samples (one-call frames)
    MeResult *out_buf = nullptr;      // device results for host runs
    u64 *keys = nullptr;              // per-block integer winners
    u32 *sub = nullptr;               // per-candidate SATD sums of the refinement
    pel *shift = nullptr;             // byte-shifted reference copies of the integer search
    u32 *q2 = nullptr;                // device search tables
    u16 *r2m = nullptr;
    MeTables tab;
    bool tab_ok = false;
    int n_ctu;
    cudaStream_t st = nullptr;
    std::vector<u32> h_q2;
    std::vector<u16> h_r2m;
    void *tz_buf = nullptr;           // TZ / affine-search requests and results of host runs
    size_t tz_cap = 0;
    struct Graph {                    // captured frames (uavs3e_cuda_me_frame_graph)
        int slot, i_src, i_org;
        const void *ref, *org;
        void *out;
        u32 lambda;
        cudaGraphExec_t exec;
        unsigned long long launches, used;
    };
    std::vector<Graph> graphs;
    unsigned long long graph_tick = 0;
    pel *chroma_buf = nullptr;        // [n_refs][2][rows_c * stride_c], padded by 72
    int stride_c = 0, rows_c = 0;
    void *mc_buf = nullptr;           // CU MC requests and predictions of host runs
    size_t mc_cap = 0;
};

static const int kPadC = 72;          // PIC_PAD_SIZE_C

static pel *me_chroma_ptr(uavs3e_cuda_me *m, int slot, int c)
{
    return m->chroma_buf + ((size_t)slot * 2 + c) * m->stride_c * m->rows_c + (size_t)kPadC * m->stride_c + kPadC;
}

static const int kNdy = ME_NDY;
static_assert(sizeof(MeResult) == sizeof(uavs3e_cuda_me_result_t), "result record layout");

static pel *me_plane_ptr(uavs3e_cuda_me *m, int slot, int phase)
{
    return m->planes_buf + ((size_t)slot * 16 + phase) * m->plane_bytes + (size_t)m->pad * m->stride + m->pad;
}

static int me_prepare_tables(uavs3e_cuda_me *m, u32 lambda, cudaStream_t st)
{
    if (m->tab_ok && m->tab.lambda_mv == lambda) return UC_OK;
    size_t cap = me_q2_entries(m->range, kNdy);
    m->h_q2.assign(cap, 0xFFFFFFFFu);
    m->h_r2m.assign((size_t)ME_R2M_ENTRIES, 0);
    std::vector<MeCand> cand(ME_MAX_GROUP);
    if (me_build_tables(m->W, m->H, m->range, lambda, kNdy, &m->tab, m->h_q2.data(), m->h_r2m.data(), cap,
                        cand.data()))
        return set_status(UC_ERR_ARG, "me: cannot build search tables for this size/range");
    // synchronous upload: tables change only with lambda (per slice QP)
    UC_CHECK(cudaStreamSynchronize(st));
    UC_CHECK(cudaMemcpy(m->q2, m->h_q2.data(), cap * sizeof(u32), cudaMemcpyHostToDevice));
    UC_CHECK(cudaMemcpy(m->r2m, m->h_r2m.data(), m->h_r2m.size() * sizeof(u16), cudaMemcpyHostToDevice));
    m->tab_ok = true;
    return UC_OK;
}

extern "C" {

UAVS3E_CUDA_API uavs3e_cuda_me *uavs3e_cuda_me_open(int width, int height, int n_refs, int range, int pad)
{
    if (ensure_init()) return nullptr;
    if (width < 64 || height < 64 || n_refs < 1 || n_refs > ME_MAX_REFS || range < 1 || range > 64 || pad < 144) {
        set_status(UC_ERR_ARG, "me_open: unsupported size/refs/range/pad");
        return nullptr;
    }
    uavs3e_cuda_me *m = new uavs3e_cuda_me();
    m->W = width; m->H = height; m->n_refs = n_refs; m->range = range; m->pad = pad;
    m->stride = ((width + 2 * pad) + 15) & ~15;
    m->rows = height + 2 * pad;
    m->plane_bytes = (size_t)m->stride * m->rows;
    m->n_ctu = ((width + 63) / 64) * ((height + 63) / 64);
    size_t nres = (size_t)m->n_ctu * ME_BLOCKS_PER_CTU * n_refs;
    bool ok = cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&m->planes_buf, m->plane_bytes * 16 * n_refs) == cudaSuccess &&
              cudaMalloc(&m->org_buf, (size_t)width * height) == cudaSuccess &&
              cudaMalloc(&m->out_buf, nres * sizeof(MeResult)) == cudaSuccess &&
              cudaMalloc(&m->keys, me_key_scratch_bytes(width, height, n_refs)) == cudaSuccess &&
              cudaMalloc(&m->sub, me_sub_scratch_bytes(width, height, n_refs)) == cudaSuccess &&
              cudaMalloc(&m->shift, me_shift_scratch_bytes(width, height, n_refs)) == cudaSuccess &&
              cudaMalloc(&m->q2, me_q2_entries(range, kNdy) * sizeof(u32)) == cudaSuccess &&
              cudaMalloc(&m->r2m, (size_t)ME_R2M_ENTRIES * sizeof(u16)) == cudaSuccess &&
              cudaMemset(m->planes_buf, 0, m->plane_bytes * 16 * n_refs) == cudaSuccess &&
              cudaMemset(m->shift, 0, me_shift_scratch_bytes(width, height, n_refs)) == cudaSuccess;
    if (!ok) {
        set_status(UC_ERR_MEMORY, "me_open: device allocation failed");
        uavs3e_cuda_me_close(m);
        return nullptr;
    }
    return m;
}

UAVS3E_CUDA_API void uavs3e_cuda_me_close(uavs3e_cuda_me *m)
{
    if (!m) return;
    if (m->st) cudaStreamSynchronize(m->st);
    cudaFree(m->planes_buf); cudaFree(m->org_buf); cudaFree(m->out_buf); cudaFree(m->ref_stage);
    cudaFree(m->keys); cudaFree(m->sub); cudaFree(m->shift); cudaFree(m->q2); cudaFree(m->r2m); cudaFree(m->tz_buf);
    cudaFree(m->chroma_buf); cudaFree(m->mc_buf);
    for (auto &g : m->graphs) cudaGraphExecDestroy(g.exec);
    if (m->st) cudaStreamDestroy(m->st);
    delete m;
}

UAVS3E_CUDA_API int uavs3e_cuda_me_num_results(const uavs3e_cuda_me *m)
{
    return m ? m->n_ctu * ME_BLOCKS_PER_CTU * m->n_refs : 0;
}

// a slot's new integer plane: padding, the 15 fractional planes and the byte-shifted copies the
// integer search's windows are staged from
static int me_interp_slot(uavs3e_cuda_me *m, int slot, cudaStream_t st)
{
    pel *p0 = me_plane_ptr(m, slot, 0);
    int r = launch_pad_plane(p0, m->W, m->H, m->pad, m->stride, st);
    if (r) return r;
    PlaneSet15 ps;
    for (int i = 0; i < 15; i++) ps.p[i] = me_plane_ptr(m, slot, i + 1);
    r = launch_subpel_planes(p0, m->stride, m->W, m->H, m->pad, ps, st);
    if (r) return r;
    const pel *src[1] = { p0 };
    return launch_shift_planes(src, 1, m->stride, m->W, m->H,
                               m->shift + (size_t)slot * (me_shift_scratch_bytes(m->W, m->H, 1)), st);
}

UAVS3E_CUDA_API int uavs3e_cuda_me_set_ref(uavs3e_cuda_me *m, int slot, const uint8_t *plane, int stride)
{
    if (!m || !plane || slot < 0 || slot >= m->n_refs || stride < m->W) return set_status(UC_ERR_ARG, "me_set_ref: bad argument");
    if (ensure_init()) return uavs3e_cuda_status();
    UC_CHECK(cudaMemcpy2DAsync(me_plane_ptr(m, slot, 0), m->stride, plane, stride, m->W, m->H, cudaMemcpyHostToDevice, m->st));
    int r = me_interp_slot(m, slot, m->st);
    if (r) return r;
    UC_CHECK(cudaStreamSynchronize(m->st));
    return UC_OK;
}

UAVS3E_CUDA_API int uavs3e_cuda_me_set_ref_device(uavs3e_cuda_me *m, int slot, const uint8_t *d_plane, int stride,
                                                  void *stream)
{
    if (!m || !d_plane || slot < 0 || slot >= m->n_refs || stride < m->W) return set_status(UC_ERR_ARG, "me_set_ref_device: bad argument");
    if (ensure_init()) return uavs3e_cuda_status();
    cudaStream_t st = (cudaStream_t)stream;
    UC_CHECK(cudaMemcpy2DAsync(me_plane_ptr(m, slot, 0), m->stride, d_plane, stride, m->W, m->H, cudaMemcpyDeviceToDevice, st));
    return me_interp_slot(m, slot, st);
}

static int me_launch(uavs3e_cuda_me *m, const pel *d_org, int i_org, u32 lambda, MeResult *d_out, cudaStream_t st)
{
    int r = me_prepare_tables(m, lambda, st);
    if (r) return r;
    MeFrameArgs a;
    memset(&a, 0, sizeof(a));
    a.org = d_org; a.i_org = i_org;
    for (int s = 0; s < m->n_refs; s++)
        for (int q = 0; q < 16; q++) a.planes[s][q] = me_plane_ptr(m, s, q);
    a.i_ref = m->stride; a.pad = m->pad;
    a.W = m->W; a.H = m->H; a.n_refs = m->n_refs; a.range = m->range; a.lambda_mv = lambda;
    a.out = d_out; a.q2tab = m->q2; a.rank2mv = m->r2m; a.sub_scratch = m->sub; a.shift_scratch = m->shift;
    a.shift_ready = true;             // kept current by me_interp_slot
    return launch_me_frame(a, m->tab, m->keys, st);
}

UAVS3E_CUDA_API int uavs3e_cuda_me_run(uavs3e_cuda_me *m, const uint8_t *org, int i_org, uint32_t lambda_mv,
                                       uavs3e_cuda_me_result_t *out)
{
    if (!m || !org || !out || i_org < m->W) return set_status(UC_ERR_ARG, "me_run: bad argument");
    if ((uint64_t)lambda_mv * 36u >= (1ull << 32)) return set_status(UC_ERR_ARG, "me_run: lambda_mv too large");
    if (ensure_init()) return uavs3e_cuda_status();
    UC_CHECK(cudaMemcpy2DAsync(m->org_buf, m->W, org, i_org, m->W, m->H, cudaMemcpyHostToDevice, m->st));
    int r = me_launch(m, m->org_buf, m->W, lambda_mv, m->out_buf, m->st);
    if (r) return r;
    UC_CHECK(cudaMemcpyAsync(out, m->out_buf, (size_t)uavs3e_cuda_me_num_results(m) * sizeof(MeResult),
                             cudaMemcpyDeviceToHost, m->st));
    UC_CHECK(cudaStreamSynchronize(m->st));
    return UC_OK;
}

UAVS3E_CUDA_API int uavs3e_cuda_me_run_device(uavs3e_cuda_me *m, const uint8_t *d_org, int i_org,
                                              uint32_t lambda_mv, uavs3e_cuda_me_result_t *d_out, void *stream)
{
    if (!m || !d_org || !d_out || i_org < m->W) return set_status(UC_ERR_ARG, "me_run_device: bad argument");
    if ((uint64_t)lambda_mv * 36u >= (1ull << 32)) return set_status(UC_ERR_ARG, "me_run_device: lambda_mv too large");
    if (ensure_init()) return uavs3e_cuda_status();
    return me_launch(m, d_org, i_org, lambda_mv, (MeResult *)d_out, (cudaStream_t)stream);
}

UAVS3E_CUDA_API int uavs3e_cuda_me_set_ref_chroma(uavs3e_cuda_me *m, int slot, const uint8_t *u, const uint8_t *v,
                                                  int stride)
{
    if (!m || !u || !v || slot < 0 || slot >= m->n_refs || stride < m->W / 2)
        return set_status(UC_ERR_ARG, "me_set_ref_chroma: bad argument");
    if (ensure_init()) return uavs3e_cuda_status();
    const int Wc = m->W / 2, Hc = m->H / 2;
    if (!m->chroma_buf) {
        m->stride_c = (Wc + 2 * kPadC + 15) & ~15;
        m->rows_c = Hc + 2 * kPadC;
        UC_CHECK(cudaMalloc(&m->chroma_buf, (size_t)m->n_refs * 2 * m->stride_c * m->rows_c));
    }
    for (int c = 0; c < 2; c++) {
        pel *d = me_chroma_ptr(m, slot, c);
        UC_CHECK(cudaMemcpy2DAsync(d, m->stride_c, c ? v : u, stride, Wc, Hc, cudaMemcpyHostToDevice, m->st));
        int r = launch_pad_plane(d, Wc, Hc, kPadC, m->stride_c, m->st);
        if (r) return r;
    }
    UC_CHECK(cudaStreamSynchronize(m->st));
    return UC_OK;
}

// the host entries of CU and affine motion compensation: requests up, predictions down
static int me_mc_host(uavs3e_cuda_me *m, bool affine, const void *reqs, size_t req_size, int n, uint8_t *out,
                      size_t out_bytes)
{
    if (!m || n < 0 || (n > 0 && (!reqs || !out))) return set_status(UC_ERR_ARG, "mc: bad argument");
    if (!m->chroma_buf) return set_status(UC_ERR_ARG, "mc: no chroma planes (uavs3e_cuda_me_set_ref_chroma)");
    if (ensure_init()) return uavs3e_cuda_status();
    if (n == 0) return UC_OK;
    const size_t rb = ((size_t)n * req_size + 255) & ~(size_t)255;
    if (m->mc_cap < rb + out_bytes) {
        if (m->mc_buf) UC_CHECK(cudaFree(m->mc_buf));
        m->mc_buf = nullptr;
        m->mc_cap = 0;
        UC_CHECK(cudaMalloc(&m->mc_buf, rb + out_bytes));
        m->mc_cap = rb + out_bytes;
    }
    const int slots = std::min(m->n_refs, UAVS3E_CUDA_TZ_MAX_SLOTS);
    const pel *planes[UAVS3E_CUDA_TZ_MAX_SLOTS * 16], *chroma[UAVS3E_CUDA_TZ_MAX_SLOTS * 2];
    for (int s = 0; s < slots; s++) {
        for (int ph = 0; ph < 16; ph++) planes[s * 16 + ph] = me_plane_ptr(m, s, ph);
        for (int c = 0; c < 2; c++) chroma[s * 2 + c] = me_chroma_ptr(m, s, c);
    }
    pel *d_out = (pel *)m->mc_buf + rb;
    UC_CHECK(cudaMemcpyAsync(m->mc_buf, reqs, (size_t)n * req_size, cudaMemcpyHostToDevice, m->st));
    int r = affine ? launch_mc_affine(m->W, m->H, planes, slots, m->stride, m->pad, chroma, m->stride_c, kPadC,
                                      m->mc_buf, n, d_out, (unsigned long long)out_bytes, m->st)
                   : launch_mc_cu(m->W, m->H, planes, slots, m->stride, m->pad, chroma, m->stride_c, kPadC,
                                  m->mc_buf, n, d_out, (unsigned long long)out_bytes, m->st);
    if (r) return r;
    UC_CHECK(cudaMemcpyAsync(out, d_out, out_bytes, cudaMemcpyDeviceToHost, m->st));
    UC_CHECK(cudaStreamSynchronize(m->st));
    return UC_OK;
}

UAVS3E_CUDA_API int uavs3e_cuda_mc_affine(uavs3e_cuda_me *m, const uavs3e_cuda_affine_req_t *reqs, int n,
                                          uint8_t *out, size_t out_bytes)
{
    return me_mc_host(m, true, reqs, sizeof(*reqs), n, out, out_bytes);
}

UAVS3E_CUDA_API int uavs3e_cuda_mc_cu(uavs3e_cuda_me *m, const uavs3e_cuda_mc_req_t *reqs, int n, uint8_t *out,
                                      size_t out_bytes)
{
    return me_mc_host(m, false, reqs, sizeof(*reqs), n, out, out_bytes);
}

UAVS3E_CUDA_API int uavs3e_cuda_me_tz(uavs3e_cuda_me *m, const uavs3e_cuda_tz_pic_t *pic, const uint8_t *org,
                                      int i_org, const uavs3e_cuda_tz_req_t *reqs, int n, uavs3e_cuda_tz_out_t *out)
{
    if (!m || !pic || !org || (n > 0 && (!reqs || !out)) || n < 0 || i_org < m->W || pic->width != m->W ||
        pic->height != m->H)
        return set_status(UC_ERR_ARG, "me_tz: bad argument");
    if (ensure_init()) return uavs3e_cuda_status();
    if (n == 0) return UC_OK;
    const size_t need = (size_t)n * (sizeof(uavs3e_cuda_tz_req_t) + sizeof(uavs3e_cuda_tz_out_t));
    if (m->tz_cap < need) {
        if (m->tz_buf) UC_CHECK(cudaFree(m->tz_buf));
        m->tz_buf = nullptr;
        m->tz_cap = 0;
        UC_CHECK(cudaMalloc(&m->tz_buf, need));
        m->tz_cap = need;
    }
    uavs3e_cuda_tz_req_t *d_req = (uavs3e_cuda_tz_req_t *)m->tz_buf;
    uavs3e_cuda_tz_out_t *d_out = (uavs3e_cuda_tz_out_t *)(d_req + n);
    const pel *planes[UAVS3E_CUDA_TZ_MAX_SLOTS * 16];
    const int slots = std::min(m->n_refs, UAVS3E_CUDA_TZ_MAX_SLOTS);
    for (int s = 0; s < slots; s++)
        for (int ph = 0; ph < 16; ph++) planes[s * 16 + ph] = me_plane_ptr(m, s, ph);
    for (int i = 0; i < n; i++)
        if (reqs[i].ref_slot >= slots || (reqs[i].bi && reqs[i].other_slot >= slots))
            return set_status(UC_ERR_ARG, "me_tz: reference slot");
    UC_CHECK(cudaMemcpy2DAsync(m->org_buf, m->W, org, i_org, m->W, m->H, cudaMemcpyHostToDevice, m->st));
    UC_CHECK(cudaMemcpyAsync(d_req, reqs, (size_t)n * sizeof(*reqs), cudaMemcpyHostToDevice, m->st));
    int r = launch_me_tz(pic, m->org_buf, m->W, planes, slots, m->stride, m->pad, d_req, n, d_out, m->st);
    if (r) return r;
    UC_CHECK(cudaMemcpyAsync(out, d_out, (size_t)n * sizeof(*out), cudaMemcpyDeviceToHost, m->st));
    UC_CHECK(cudaStreamSynchronize(m->st));
    return UC_OK;
}

UAVS3E_CUDA_API int uavs3e_cuda_me_affine(uavs3e_cuda_me *m, const uint8_t *org, int i_org,
                                          const uavs3e_cuda_affme_req_t *reqs, int n, uavs3e_cuda_affme_out_t *out)
{
    if (!m || !org || (n > 0 && (!reqs || !out)) || n < 0 || i_org < m->W)
        return set_status(UC_ERR_ARG, "me_affine: bad argument");
    if (ensure_init()) return uavs3e_cuda_status();
    if (n == 0) return UC_OK;
    const size_t need = (size_t)n * (sizeof(uavs3e_cuda_affme_req_t) + sizeof(uavs3e_cuda_affme_out_t));
    if (m->tz_cap < need) {
        if (m->tz_buf) UC_CHECK(cudaFree(m->tz_buf));
        m->tz_buf = nullptr;
        m->tz_cap = 0;
        UC_CHECK(cudaMalloc(&m->tz_buf, need));
        m->tz_cap = need;
    }
    uavs3e_cuda_affme_req_t *d_req = (uavs3e_cuda_affme_req_t *)m->tz_buf;
    uavs3e_cuda_affme_out_t *d_out = (uavs3e_cuda_affme_out_t *)(d_req + n);
    const pel *planes[UAVS3E_CUDA_TZ_MAX_SLOTS * 16];
    const int slots = std::min(m->n_refs, UAVS3E_CUDA_TZ_MAX_SLOTS);
    for (int s = 0; s < slots; s++)
        for (int ph = 0; ph < 16; ph++) planes[s * 16 + ph] = me_plane_ptr(m, s, ph);
    for (int i = 0; i < n; i++)
        if (reqs[i].ref_slot >= slots || ((reqs[i].flags & UAVS3E_CUDA_AFFME_BI) && reqs[i].other_slot >= slots))
            return set_status(UC_ERR_ARG, "me_affine: reference slot");
    UC_CHECK(cudaMemcpy2DAsync(m->org_buf, m->W, org, i_org, m->W, m->H, cudaMemcpyHostToDevice, m->st));
    UC_CHECK(cudaMemcpyAsync(d_req, reqs, (size_t)n * sizeof(*reqs), cudaMemcpyHostToDevice, m->st));
    int r = launch_me_affine(m->W, m->H, m->org_buf, m->W, planes, slots, m->stride, m->pad, d_req, n, d_out, m->st);
    if (r) return r;
    UC_CHECK(cudaMemcpyAsync(out, d_out, (size_t)n * sizeof(*out), cudaMemcpyDeviceToHost, m->st));
    UC_CHECK(cudaStreamSynchronize(m->st));
    return UC_OK;
}

UAVS3E_CUDA_API int uavs3e_cuda_me_frame_graph(uavs3e_cuda_me *m, int slot, const uint8_t *d_ref, int i_src,
                                               const uint8_t *d_org, int i_org, uint32_t lambda_mv,
                                               uavs3e_cuda_me_result_t *d_out, void *stream)
{
    if (!m || !d_ref || !d_org || !d_out || slot < 0 || slot >= m->n_refs || i_src < m->W || i_org < m->W)
        return set_status(UC_ERR_ARG, "me_frame_graph: bad argument");
    if ((uint64_t)lambda_mv * 36u >= (1ull << 32)) return set_status(UC_ERR_ARG, "me_frame_graph: lambda_mv too large");
    if (ensure_init()) return uavs3e_cuda_status();
    // the search tables follow lambda: graphs captured with other tables are dropped
    const bool new_tables = !(m->tab_ok && m->tab.lambda_mv == lambda_mv);
    int r = me_prepare_tables(m, lambda_mv, m->st);
    if (r) return r;
    if (new_tables) {
        for (auto &g : m->graphs) cudaGraphExecDestroy(g.exec);
        m->graphs.clear();
    }
    r = me_frame_once();
    if (r) return r;
    uavs3e_cuda_me::Graph *hit = nullptr;
    for (auto &g : m->graphs)
        if (g.slot == slot && g.ref == d_ref && g.i_src == i_src && g.org == d_org && g.i_org == i_org &&
            g.lambda == lambda_mv && g.out == d_out) { hit = &g; break; }
    if (!hit) {
        if (m->graphs.size() >= 32) {    // evict the least recently used
            auto lru = m->graphs.begin();
            for (auto it = m->graphs.begin(); it != m->graphs.end(); ++it) if (it->used < lru->used) lru = it;
            cudaGraphExecDestroy(lru->exec);
            m->graphs.erase(lru);
        }
        // capture on the session's stream the launches of set_ref_device + run_device
        UC_CHECK(cudaStreamSynchronize(m->st));
        UC_CHECK(cudaStreamBeginCapture(m->st, cudaStreamCaptureModeThreadLocal));
        const unsigned long long l0 = uavs3e_cuda_launch_count();
        cudaError_t ce = cudaMemcpy2DAsync(me_plane_ptr(m, slot, 0), m->stride, d_ref, i_src, m->W, m->H,
                                           cudaMemcpyDeviceToDevice, m->st);
        int rr = ce == cudaSuccess ? me_interp_slot(m, slot, m->st) : UC_ERR_CUDA;
        if (!rr) rr = me_launch(m, d_org, i_org, lambda_mv, (MeResult *)d_out, m->st);
        cudaGraph_t graph = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(m->st, &graph);
        if (rr || ce != cudaSuccess || ee != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            if (rr) return rr;
            return check_cuda(ce != cudaSuccess ? ce : ee, "me_frame_graph: capture");
        }
        uavs3e_cuda_me::Graph g;
        g.slot = slot; g.ref = d_ref; g.i_src = i_src; g.org = d_org; g.i_org = i_org; g.lambda = lambda_mv;
        g.out = d_out;
        g.launches = uavs3e_cuda_launch_count() - l0;
        const cudaError_t ie = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) return check_cuda(ie, "me_frame_graph: instantiate");
        m->graphs.push_back(g);
        hit = &m->graphs.back();
        // the capture counted its kernels once; replays count them below
        count_launch(-(int)hit->launches);
    }
    hit->used = ++m->graph_tick;
    UC_CHECK(cudaGraphLaunch(hit->exec, (cudaStream_t)stream));
    count_launch((int)hit->launches);
    return UC_OK;
}

UAVS3E_CUDA_API int uavs3e_cuda_me_frame(uavs3e_cuda_me *m, int slot, const uint8_t *ref, int i_ref,
                                         const uint8_t *org, int i_org, uint32_t lambda_mv,
                                         uavs3e_cuda_me_result_t *out)
{
    if (!m || !ref || !org || !out || slot < 0 || slot >= m->n_refs || i_ref < m->W || i_org < m->W)
        return set_status(UC_ERR_ARG, "me_frame: bad argument");
    if (ensure_init()) return uavs3e_cuda_status();
    if (!m->ref_stage) UC_CHECK(cudaMalloc(&m->ref_stage, (size_t)m->W * m->H));
    UC_CHECK(cudaMemcpy2DAsync(m->ref_stage, m->W, ref, i_ref, m->W, m->H, cudaMemcpyHostToDevice, m->st));
    UC_CHECK(cudaMemcpy2DAsync(m->org_buf, m->W, org, i_org, m->W, m->H, cudaMemcpyHostToDevice, m->st));
    int r = uavs3e_cuda_me_frame_graph(m, slot, m->ref_stage, m->W, m->org_buf, m->W, lambda_mv,
                                       (uavs3e_cuda_me_result_t *)m->out_buf, m->st);
    if (r) return r;
    UC_CHECK(cudaMemcpyAsync(out, m->out_buf, (size_t)uavs3e_cuda_me_num_results(m) * sizeof(MeResult),
                             cudaMemcpyDeviceToHost, m->st));
    UC_CHECK(cudaStreamSynchronize(m->st));
    return UC_OK;
}

UAVS3E_CUDA_API const uint8_t *uavs3e_cuda_me_plane(uavs3e_cuda_me *m, int slot, int phase)
{
    if (!m || slot < 0 || slot >= m->n_refs || phase < 0 || phase > 15) return nullptr;
    return me_plane_ptr(m, slot, phase);
}

UAVS3E_CUDA_API int uavs3e_cuda_me_plane_stride(const uavs3e_cuda_me *m) { return m ? m->stride : 0; }

UAVS3E_CUDA_API const uint8_t *uavs3e_cuda_me_chroma_plane(uavs3e_cuda_me *m, int slot, int c)
{
    if (!m || !m->chroma_buf || slot < 0 || slot >= m->n_refs || c < 0 || c > 1) return nullptr;
    return me_chroma_ptr(m, slot, c);
}

UAVS3E_CUDA_API int uavs3e_cuda_me_chroma_stride(const uavs3e_cuda_me *m) { return m ? m->stride_c : 0; }

}  // extern "C"
