// Batched motion search that allocates nothing (uavs3e_cuda_me_search_noalloc).
//
// Some callers cannot allocate device memory when they search a frame: an encoder thread that
// runs inside a fixed memory budget set up at start-up, code that must not call cudaMalloc /
// cudaFree because those synchronise the device and would stall other streams, or a host that
// hands this library only the buffers it owns.  This variant takes every input and output from
// the caller (original picture, the 16 planes of each reference -- e.g. from
// uavs3e_cuda_pad_plane + uavs3e_cuda_subpel_planes -- and the result array) and keeps its
// scratch -- the per-block integer winners, the per-candidate SATD sums of the refinement, the
// per-lambda search tables and the byte-shifted reference copies the integer search stages its
// windows from -- in one file-scope device array of fixed size, which every GPU
// that loads the library holds until the process exits.  The host-side search tables are built
// in static host arrays, so no heap allocation happens either.
#include "common.cuh"
#include "uavs3e_cuda_internal.h"
#include "../../include/uavs3e_cuda.h"

#include <algorithm>
#include <string.h>

namespace uc {

// limits of the static scratch: a 1920x1088 frame (510 CTUs of 64x64), 2 references,
// search range 64
constexpr int NA_MAX_CTUS = UAVS3E_CUDA_NOALLOC_MAX_CTUS;
constexpr int NA_MAX_REFS = UAVS3E_CUDA_NOALLOC_MAX_REFS;
constexpr int NA_MAX_RANGE = UAVS3E_CUDA_NOALLOC_MAX_RANGE;
constexpr int NA_NDY = ME_NDY;
constexpr size_t NA_KEYS = (size_t)NA_MAX_CTUS * NA_MAX_REFS * ME_BLOCKS_PER_CTU * sizeof(u64) + 2 * sizeof(u32);
// byte-shifted reference copies of the integer search: 4 per reference, each at most the
// padded geometry of a 1920x1088 frame (row pitch 2208, 1376 rows)
constexpr size_t NA_SHIFT_PLANE = (size_t)2208 * 1376;
constexpr size_t NA_SHIFT = (size_t)NA_MAX_REFS * 4 * NA_SHIFT_PLANE;
constexpr size_t NA_SUB = (size_t)NA_MAX_CTUS * NA_MAX_REFS * ME_BLOCKS_PER_CTU * 18 * sizeof(u32);
constexpr size_t NA_Q2_ENTRIES = me_q2_entries(NA_MAX_RANGE, NA_NDY);
constexpr size_t NA_Q2 = NA_Q2_ENTRIES * sizeof(u32);
constexpr size_t NA_R2M = (size_t)ME_R2M_ENTRIES * sizeof(u16);
constexpr size_t na_up(size_t v) { return (v + 255) & ~(size_t)255; }
constexpr size_t NA_OFF_SUB = na_up(NA_KEYS);
constexpr size_t NA_OFF_Q2 = na_up(NA_OFF_SUB + NA_SUB);
constexpr size_t NA_OFF_R2M = na_up(NA_OFF_Q2 + NA_Q2);
constexpr size_t NA_OFF_SHIFT = na_up(NA_OFF_R2M + NA_R2M);
constexpr size_t NA_BYTES = NA_OFF_SHIFT + NA_SHIFT;
static_assert(NA_BYTES == UAVS3E_CUDA_NOALLOC_SCRATCH_BYTES, "scratch size in the header");
static_assert(NA_OFF_SUB % 256 == 0 && NA_OFF_Q2 % 16 == 0 && NA_OFF_R2M % 16 == 0 && NA_OFF_SHIFT % 256 == 0,
              "scratch alignment");

// the scratch every call of this entry point uses
static __device__ __align__(256) unsigned char g_me_scratch[NA_BYTES];

// the scratch's device address on the library's device (looked up by the first call, with that
// device current) and the parameters of the search tables it currently holds; indexed by device
// ordinal, though every call runs on the device uavs3e_cuda_init selected
struct NaDevice {
    unsigned char *scratch = nullptr;
    bool tables = false;
    int W = 0, H = 0, range = 0;
    u32 lambda = 0;
    MeTables tab;
};
static NaDevice g_na[64];

// static host buffers for the table build (no heap use)
static u32 g_h_q2[NA_Q2_ENTRIES];
static u16 g_h_r2m[ME_R2M_ENTRIES];
static MeCand g_cand[ME_MAX_GROUP];

}  // namespace uc

using namespace uc;

extern "C" UAVS3E_CUDA_API int uavs3e_cuda_me_search_noalloc(const uint8_t *d_org, int i_org,
                                                             const uint8_t *const *d_planes, int i_ref, int pad,
                                                             int width, int height, int n_refs, int range,
                                                             uint32_t lambda_mv, uavs3e_cuda_me_result_t *d_out,
                                                             void *stream)
{
    // size limits of the static scratch first: a larger request is an argument error
    const long long n_ctu = (long long)((width + 63) / 64) * ((height + 63) / 64);
    if (width < 64 || height < 64 || n_ctu > NA_MAX_CTUS || n_refs < 1 || n_refs > NA_MAX_REFS || range < 1 ||
        range > NA_MAX_RANGE)
        return set_status(UC_ERR_ARG, "me_search_noalloc: frame, reference count or range exceeds the static scratch "
                                      "(at most 510 CTUs of 64x64, 2 references, range 64)");
    if ((size_t)((width + 2 * 144 + 15) & ~15) * (size_t)(height + 2 * 144) > NA_SHIFT_PLANE)
        return set_status(UC_ERR_ARG, "me_search_noalloc: frame exceeds the static scratch (the padded area of "
                                      "1920x1088)");
    if (!d_org || !d_planes || !d_out || i_org < width || pad < 144 || i_ref < width + 2 * pad)
        return set_status(UC_ERR_ARG, "me_search_noalloc: bad pointer or geometry");
    if ((uint64_t)lambda_mv * 36u >= (1ull << 32)) return set_status(UC_ERR_ARG, "me_search_noalloc: lambda_mv too large");
    for (int i = 0; i < n_refs * 16; i++)
        if (!d_planes[i]) return set_status(UC_ERR_ARG, "me_search_noalloc: null plane");
    // the caller's buffers must live on the library's device: ensure_init makes that device
    // current, so a caller on another device gets an argument error (and its device back)
    int caller_dev = 0;
    UC_CHECK(cudaGetDevice(&caller_dev));
    int r = ensure_init();
    if (r) return r;
    int dev = 0;
    UC_CHECK(cudaGetDevice(&dev));
    if (dev != caller_dev) {
        cudaSetDevice(caller_dev);
        return set_status(UC_ERR_ARG, "me_search_noalloc: the current device is not the library's device "
                                      "(uavs3e_cuda_init)");
    }
    if (dev < 0 || dev >= 64) return set_status(UC_ERR_UNSUPPORTED, "me_search_noalloc: device index");
    NaDevice &D = g_na[dev];
    cudaStream_t st = (cudaStream_t)stream;
    if (!D.scratch) {
        // once, with the library's device current: the array's device address (host code may
        // not use the symbol itself).  Under lazy module loading this lookup also loads this
        // file's module, which is when the array is created on the device.
        void *p = nullptr;
        UC_CHECK(cudaGetSymbolAddress(&p, g_me_scratch));
        D.scratch = (unsigned char *)p;
    }
    if (!D.tables || D.W != width || D.H != height || D.range != range || D.lambda != lambda_mv) {
        if (me_build_tables(width, height, range, lambda_mv, NA_NDY, &D.tab, g_h_q2, g_h_r2m, NA_Q2_ENTRIES, g_cand))
            return set_status(UC_ERR_ARG, "me_search_noalloc: cannot build search tables");
        D.tables = false;
        UC_CHECK(cudaMemcpyAsync(D.scratch + NA_OFF_Q2, g_h_q2, (size_t)D.tab.n_entries * sizeof(u32),
                                 cudaMemcpyHostToDevice, st));
        UC_CHECK(cudaMemcpyAsync(D.scratch + NA_OFF_R2M, g_h_r2m, NA_R2M, cudaMemcpyHostToDevice, st));
        // the host buffers are reused by the next build: wait until the copies have read them
        UC_CHECK(cudaStreamSynchronize(st));
        D.tables = true;
        D.W = width; D.H = height; D.range = range; D.lambda = lambda_mv;
    }
    MeFrameArgs a;
    memset(&a, 0, sizeof(a));
    a.org = d_org; a.i_org = i_org;
    for (int s = 0; s < n_refs; s++)
        for (int q = 0; q < 16; q++) a.planes[s][q] = d_planes[s * 16 + q];
    a.i_ref = i_ref; a.pad = pad;
    a.W = width; a.H = height; a.n_refs = n_refs; a.range = range; a.lambda_mv = lambda_mv;
    a.out = (MeResult *)d_out;
    a.q2tab = (const u32 *)(D.scratch + NA_OFF_Q2);
    a.rank2mv = (const u16 *)(D.scratch + NA_OFF_R2M);
    a.sub_scratch = (u32 *)(D.scratch + NA_OFF_SUB);      // zeroed by launch_me_frame before use
    a.shift_scratch = D.scratch + NA_OFF_SHIFT;           // rewritten by launch_me_frame from d_planes
    return launch_me_frame(a, D.tab, (u64 *)D.scratch, st);
}
