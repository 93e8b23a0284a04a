// Kernel-table entries with the exact signatures of funs_handle_t (include/uavs3e_cuda_table.h).
//
// Each entry evaluates one call on the GPU: the samples it reads are packed into a per-thread
// pinned staging buffer that is mapped into the device's address space, one kernel reads them
// there and writes its outputs there, and after the stream synchronises they are unpacked into
// the caller's memory with the caller's strides (one launch and one synchronisation per call,
// no copy calls).  Only outputs the reference function writes are written back.
#include "common.cuh"
#include "intra.cuh"
#include "tables.h"
#include "uavs3e_cuda_internal.h"
#include "../../include/uavs3e_cuda_table.h"

#include <string.h>

namespace uc {

// ------------------------------------------------------------------ per-thread staging
struct CallCtx {
    cudaStream_t st = nullptr;
    u8 *h = nullptr;      // pinned, mapped staging buffer (host address)
    u8 *d = nullptr;      // the same buffer's device address
    size_t cap = 0;
};
static thread_local CallCtx t_ctx;

class Call {
public:
    explicit Call(size_t need)
    {
        ok = ensure_init() == UC_OK && reserve_cap(need + 4096);
        used = 0;
    }
    bool ok;
    size_t used;
    CallCtx &c() { return t_ctx; }

    size_t take(size_t bytes)
    {
        size_t off = (used + 15) & ~(size_t)15;
        used = off + bytes;
        return off;
    }
    size_t put(const void *src, size_t bytes)
    {
        size_t off = take(bytes);
        if (bytes) memcpy(t_ctx.h + off, src, bytes);
        return off;
    }
    // rows of w elements with the caller's stride, packed densely
    template <class T> size_t put2d(const T *src, long long stride, int w, int h)
    {
        size_t off = take(sizeof(T) * (size_t)w * h);
        T *dst = (T *)(t_ctx.h + off);
        for (int y = 0; y < h; y++) memcpy(dst + (size_t)y * w, src + (long long)y * stride, sizeof(T) * w);
        return off;
    }
    template <class T> T *dev(size_t off) { return (T *)(t_ctx.d + off); }
    template <class T> T *host(size_t off) { return (T *)(t_ctx.h + off); }

    // the kernel reads the staged inputs in place (mapped host memory): nothing to copy
    bool upload() { return true; }
    bool launched() { return check(cudaGetLastError(), "entry kernel"); }
    // the kernel wrote its outputs in place: wait for it
    bool download(size_t, size_t) { return check(cudaStreamSynchronize(t_ctx.st), "entry sync"); }

private:
    static bool check(cudaError_t e, const char *what)
    {
        if (e == cudaSuccess) return true;
        check_cuda(e, what);
        return false;
    }
    static bool reserve_cap(size_t need)
    {
        CallCtx &x = t_ctx;
        if (!x.st && cudaStreamCreateWithFlags(&x.st, cudaStreamNonBlocking) != cudaSuccess) {
            set_status(UC_ERR_CUDA, "entry: stream creation failed");
            return false;
        }
        if (x.cap >= need) return true;
        size_t cap = std::max(need, (size_t)4 << 20);
        if (x.h) cudaFreeHost(x.h);
        x.h = nullptr; x.d = nullptr; x.cap = 0;
        if (cudaHostAlloc((void **)&x.h, cap, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess ||
            cudaHostGetDevicePointer((void **)&x.d, x.h, 0) != cudaSuccess) {
            set_status(UC_ERR_MEMORY, "entry: staging allocation failed");
            return false;
        }
        x.cap = cap;
        return true;
    }
};

static const DevTables *tabs()
{
    int dev = 0;
    cudaGetDevice(&dev);
    const DevTables *t = device_tables(dev);
    if (!t) set_status(UC_ERR_MEMORY, "entry: table upload failed");
    return t;
}

struct Taps8 { int c[8]; };
struct Taps3x8 { int c[3][8]; };

// ------------------------------------------------------------------ kernels

__device__ __forceinline__ u32 block_reduce_u32(u32 v)
{
    __shared__ u32 s[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
    __syncthreads();
    u32 t = 0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? s[threadIdx.x] : 0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xFFFFFFFFu, t, o);
    }
    __syncthreads();
    return t;
}

// SAD of org against n_pred predictions (cost_sad / _x3 / _x4), or SSD (cost_ssd)
__global__ void k_e_sad(const pel *o, const pel *p, int w, int h, int n_pred, int ssd, u64 *out)
{
    for (int k = 0; k < n_pred; k++) {
        u32 acc = 0;
        for (int i = threadIdx.x; i < w * h; i += blockDim.x) {
            int d = (int)o[i] - (int)p[(size_t)k * w * h + i];
            acc += ssd ? (u32)(d * d) : (u32)abs(d);
        }
        u32 t = block_reduce_u32(acc);
        if (threadIdx.x == 0) out[k] = t;
    }
}

__global__ void k_e_satd(int tw, int th, const pel *o, const pel *p, double sq32, double sq128, u32 *out)
{
    if (threadIdx.x == 0) out[0] = satd_tile(tw, th, o, tw, p, tw, sq32, sq128);
}

__global__ void k_e_copy(const pel *s, pel *d, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) d[i] = s[i];
}

// one-dimensional filters: src holds the block with `back` samples of halo before and
// taps-back-1 after, in the filtered direction (dense rows of sw samples)
__global__ void k_e_ipflt(const pel *src, int sw, pel *dst, int w, int h, int taps, int vert, Taps8 c, int max_val)
{
    const int back = taps / 2 - 1;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w * h; i += gridDim.x * blockDim.x) {
        int x = i % w, y = i / w;
        int sum = 0;
        for (int t = 0; t < taps; t++) {
            int sx = vert ? x : x + t, sy = vert ? y + t : y;
            sum += src[sy * sw + sx] * c.c[t];
        }
        dst[i] = (pel)min(max_val, max(0, (sum + 32) >> 6));
        (void)back;
    }
}

// two-pass filters (mc_if_hor_ver_luma / _chroma): src is the block with a full 2-D halo
__global__ void k_e_ipflt_ext(const pel *src, int sw, pel *dst, int w, int h, int taps, Taps8 cx, Taps8 cy, int max_val)
{
    const int shift1 = max_val == 255 ? 0 : 2, shift2 = max_val == 255 ? 12 : 10;
    const int add1 = (1 << shift1) >> 1, add2 = 1 << (shift2 - 1);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w * h; i += gridDim.x * blockDim.x) {
        int x = i % w, y = i / w;
        int sum = 0;
        for (int ty = 0; ty < taps; ty++) {
            int hs = 0;
            for (int tx = 0; tx < taps; tx++) hs += src[(y + ty) * sw + x + tx] * cx.c[tx];
            int tv = shift1 ? (hs + add1) >> shift1 : hs;
            sum += (int)(s16)tv * cy.c[ty];
        }
        dst[i] = (pel)min(max_val, max(0, (sum + add2) >> shift2));
    }
}

// frame-level passes of com_if_luma_frame (com_if_filter_hor_8 / _ver_8 /
// uavs3e_if_ver_luma_frame_ext, src/com_mc.c:668-758); src dense with halo
__global__ void k_e_flt_frame(int kind, const pel *src8, const s16 *src16, int sw, pel *d0, pel *d1, pel *d2, s16 *t0,
                              s16 *t1, s16 *t2, int w, int h, Taps3x8 c, int bd)
{
    const int mx = (1 << bd) - 1;
    pel *d[3] = { d0, d1, d2 };
    s16 *t[3] = { t0, t1, t2 };
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)w * h;
         i += (long long)gridDim.x * blockDim.x) {
        int x = (int)(i % w), y = (int)(i / w);
        for (int f = 0; f < 3; f++) {
            int sum = 0;
            for (int k = 0; k < 8; k++) {
                if (kind == 0) sum += src8[(long long)y * sw + x + k] * c.c[f][k];
                else if (kind == 1) sum += src8[(long long)(y + k) * sw + x] * c.c[f][k];
                else sum += src16[(long long)(y + k) * sw + x] * c.c[f][k];
            }
            if (kind == 0) {
                int sh = bd - 8, add = (1 << sh) >> 1;
                t[f][i] = (s16)((sum + add) >> sh);
                d[f][i] = (pel)min(mx, max(0, (sum + 32) >> 6));
            } else if (kind == 1) {
                d[f][i] = (pel)min(mx, max(0, (sum + 32) >> 6));
            } else {
                int sh = 20 - bd;
                d[f][i] = (pel)min(mx, max(0, (sum + (1 << (sh - 1))) >> sh));
            }
        }
    }
}

__global__ void k_e_recon(const s16 *resi, const pel *pred, pel *rec, int n, int cbf, int bd)
{
    const int mx = (1 << bd) - 1;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        rec[i] = cbf ? (pel)min(mx, max(0, resi[i] + pred[i])) : pred[i];
}

__global__ void k_e_diff(const pel *o, const pel *p, s16 *r, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) r[i] = (s16)(o[i] - p[i]);
}

__global__ void k_e_avrg(const pel *a, const pel *b, pel *d, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        d[i] = (pel)((a[i] + b[i] + 1) >> 1);
}

// intra entries.  nb: staged neighbour window whose centre is the array centre (index 288)
enum { IE_DC, IE_PLANE, IE_BI, IE_PLANE_S16, IE_BI_S16, IE_VER, IE_HOR, IE_ANG, IE_IPF, IE_IPF_S16 };

// angular sample of the algorithm class of table entry `entry` with mode `mode`
__device__ __forceinline__ int ang_entry_sample(const pel *s, int entry, int mode, int w, int h, int i, int j)
{
    if (entry < 12) {
        int off, idx = ang_ctx(mode, 0, j + 1, &off);
        int pw = entry == 10 ? w : min(w, 2 * w - idx + 1);
        const pel *p = pw <= 0 ? s + 2 * w : s + idx + min(i, pw - 1);
        return f4tap(p[0], p[1], p[2], p[3], off);
    }
    if (entry < 24) {
        int oy, xs = ang_ctx(mode, 1, i + 1, &oy);
        int yy = j - xs;
        if (yy <= -1) {
            int ox, ix = ang_ctx(mode, 0, j + 1, &ox);
            const pel *px = s - ix + i;
            return (px[2] * (32 - ox) + px[1] * (64 - ox) + px[0] * (32 + ox) + px[-1] * ox + 64) >> 7;
        }
        return (s[-yy - 2] * (32 - oy) + s[-yy - 1] * (64 - oy) + s[-yy] * (32 + oy) + s[-yy + 1] * oy + 64) >> 7;
    }
    if (entry == 32) return ang_sample(s, 32, w, h, i, j);
    int off, xs = ang_ctx(mode, 1, i + 1, &off);
    int idx = -j - xs;
    if (entry != 26) idx = max(-2 * h, idx);
    return f4tap(s[idx], s[idx - 1], s[idx - 2], s[idx - 3], off);
}

__global__ void k_e_intra(int kind, const pel *nb, pel *dst, s16 *dst16, const s16 *pred16, int w, int h, int avail,
                          int bd, int entry, int mode)
{
    __shared__ IpredBlock B;
    const pel *s = nb + 288;
    if (threadIdx.x == 0) ipred_block_setup(s, w, h, avail, bd, B);
    __syncthreads();
    const int mx = (1 << bd) - 1;
    for (int p = threadIdx.x; p < w * h; p += blockDim.x) {
        int i = p % w, j = p / w;
        int v;
        switch (kind) {
        case IE_DC: v = B.dc; break;
        case IE_PLANE: v = ipred_sample(s, B, 1, 0, i, j); break;
        case IE_BI: v = ipred_sample(s, B, 2, 0, i, j); break;
        case IE_PLANE_S16: dst16[p] = (s16)((B.pl_t + j * B.pl_c + i * B.pl_b) >> 5); continue;
        case IE_BI_S16: {
            int lxy = B.lw + B.lh + 1, offs = 1 << (B.lw + B.lh);
            int up = s[i + 1], le = s[-j - 1];
            int predx = (le << B.lw) + (i + 1) * (B.bi_a - le);
            int refup = (up << B.lh) + (j + 1) * (B.bi_b - up);
            dst16[p] = (s16)(((predx << B.lh) + (refup << B.lw) + i * j * B.bi_wt + offs) >> lxy);
            continue;
        }
        case IE_VER: v = s[1 + i]; break;
        case IE_HOR: v = s[-1 - j]; break;
        case IE_ANG: v = ang_entry_sample(s, entry, mode, w, h, i, j); break;
        default: {   // IPF on an existing prediction (dst in/out or pred16)
            int ih = B.lw - 2, iv = B.lh - 2;
            int vr = min(h, 10), hr = min(w, 10);
            if (ih > 4) { ih = 4; hr = 0; }
            if (iv > 4) { iv = 4; vr = 0; }
            if (mode >= 3 && mode <= 18) vr = 0;
            if (mode > 18) hr = 0;
            int cl = i < hr ? kIpfParam[ih][i] : 0;
            int ct = j < vr ? kIpfParam[iv][j] : 0;
            int base = kind == IE_IPF ? (int)dst[p] : (int)pred16[p];
            v = base;
            if (j < vr || i < hr) v = (cl * s[-j - 1] + ct * s[1 + i] + (64 - cl - ct) * base + 32) >> 6;
            if (kind == IE_IPF_S16) v = min(mx, max(0, v));
        }
        }
        dst[p] = (pel)v;
    }
}

// forward DCT2 of a dense w x h residual: dst dense w x h (only the kw x kh corner computed)
__global__ void k_e_fdct2(const s8 *FW, const s8 *FH, const s16 *src, s16 *dst, s16 *tmp, int w, int h, int bd)
{
    const int kw = min(w, 32), kh = min(h, 32);
    const int lw = 31 - __clz(w), lh = 31 - __clz(h);
    const int sh1 = lw + bd - 10, sh2 = lh + 5;
    const int r1 = sh1 > 0 ? 1 << (sh1 - 1) : 0, r2 = 1 << (sh2 - 1);
    for (int i = threadIdx.x; i < kw * h; i += blockDim.x) {
        int u = i / h, y = i % h;
        int acc = 0;
        for (int x = 0; x < w; x++) acc += FW[u * w + x] * src[y * w + x];
        tmp[u * h + y] = (s16)((acc + r1) >> sh1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kw * kh; i += blockDim.x) {
        int v = i / kw, u = i % kw;
        int acc = 0;
        for (int y = 0; y < h; y++) acc += FH[v * h + y] * tmp[u * h + y];
        dst[v * w + u] = (s16)((acc + r2) >> sh2);
    }
}

__global__ void k_e_idct2(const s8 *FW, const s8 *FH, const s16 *coef, s16 *resi, s16 *tmp, int w, int h, int bd)
{
    const int kw = min(w, 32), kh = min(h, 32);
    const int sh2 = 20 - bd, mx = (1 << bd) - 1, mn = -(1 << bd);
    for (int i = threadIdx.x; i < kw * h; i += blockDim.x) {
        int u = i % kw, y = i / kw;
        int acc = 0;
        for (int v = 0; v < kh; v++) acc += FH[v * h + y] * coef[v * w + u];
        tmp[y * kw + u] = (s16)min(32767, max(-32768, (acc + 16) >> 5));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < w * h; i += blockDim.x) {
        int x = i % w, y = i / w;
        int acc = 0;
        for (int u = 0; u < kw; u++) acc += FW[u * w + x] * tmp[y * kw + u];
        resi[i] = (s16)min(mx, max(mn, (acc + (1 << (sh2 - 1))) >> sh2));
    }
}

// one DCT8/DST7 pass: forward dst[k*line + i] = sum_n M[k][n] src[i*N + n];
// inverse blk[i*N + j] = clip(sum_k M[k][j] coef[k*line + i])
__global__ void k_e_d87(const s16 *M, int N, const s16 *src, s16 *dst, int shift, int line, int inv, int mx, int mn)
{
    const int rnd = shift > 0 ? 1 << (shift - 1) : 0;
    for (int t = threadIdx.x + blockIdx.x * blockDim.x; t < N * line; t += blockDim.x * gridDim.x) {
        int i = t / N, k = t % N;
        int acc = 0;
        if (!inv) {
            for (int n = 0; n < N; n++) acc += M[k * N + n] * src[i * N + n];
            dst[k * line + i] = (s16)((acc + rnd) >> shift);
        } else {
            for (int q = 0; q < N; q++) acc += src[q * line + i] * M[q * N + k];
            dst[i * N + k] = (s16)min(mx, max(mn, (acc + rnd) >> shift));
        }
    }
}

__global__ void k_e_dquant(int flat, const s16 *coef, s16 *out, const u8 *wq4, const u8 *wq8, int lw, int lh, int scale,
                           int shift)
{
    const int w = 1 << lw, h = 1 << lh;
    const int off = shift == 0 ? 0 : 1 << (shift - 1);
    const int refix = (lw + lh) & 1;
    const int n = flat ? min(h, 32) * w : w * h;
    for (int i = threadIdx.x + blockIdx.x * blockDim.x; i < n; i += blockDim.x * gridDim.x) {
        int lev;
        if (flat) {
            lev = (coef[i] * scale + off) >> shift;
            lev = min(32767, max(-32768, lev));
            out[i] = (s16)(refix ? (lev * 181 + 128) >> 8 : lev);
        } else {
            int r = i / w, c = i % w;
            int weight;
            if (lw == 2 && lh == 2) weight = ((r | c) & 0xE0) ? 0 : wq4[r * 4 + c];
            else {
                int ish = max(lw, lh) - 3;
                weight = ((r | c) & 0xE0) ? 0 : wq8[(r >> ish) * 8 + (c >> ish)];
            }
            lev = (int)((((((s64)((coef[i] * weight) >> 2)) * scale) >> 4) + off) >> shift);   // 64-bit, then truncated
            lev = min(32767, max(-32768, lev));
            if (refix) lev = (lev * 181 + 128) >> 8;
            out[i] = (s16)lev;
        }
    }
}

__global__ void k_e_quant(int mode, const s16 *coef, int num, int thr, int q_value, int q_bits, s32 err_scale, int pb,
                          u32 *abs_coef, s16 *abs_level, s64 *err, int *ret)
{
    __shared__ int s_ret;
    if (threadIdx.x == 0) s_ret = mode == 0 ? 1 : -1;
    __syncthreads();
    if (mode == 0) {   // quant_check: the first (num >> 2) * 4 coefficients within +-thr
        for (int i = threadIdx.x; i < (num >> 2) * 4; i += blockDim.x)
            if (coef[i] > thr || coef[i] < -thr) s_ret = 0;
    } else {           // quant_rdoq first pass
        const u32 add = 1u << (q_bits - 1);
        const int th = ((1 << (q_bits - 1)) - 1) / q_value + 1;
        for (int i = threadIdx.x; i < num; i += blockDim.x) {
            int a = coef[i] < 0 ? -(int)coef[i] : coef[i];
            if (a < th) { abs_level[i] = 0; continue; }
            u32 ld = (u32)a * (u32)q_value;
            s64 e = ((s64)ld * err_scale) >> pb;
            abs_level[i] = (s16)(u32)(((u64)ld + add) >> q_bits);
            abs_coef[i] = ld;
            err[i] = e * e;
            atomicMax(&s_ret, i);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) *ret = s_ret;
}

// ------------------------------------------------------------------ entry bodies

static u64 e_sad(int w, int h, const pel *o, int io, const pel *const *p, int n_pred, int ip, int ssd, u32 *outs)
{
    Call c((size_t)w * h * (n_pred + 1) + 64);
    if (!c.ok) return 0;
    size_t oo = c.put2d(o, io, w, h);
    size_t po = 0;
    for (int k = 0; k < n_pred; k++) {
        size_t q = c.put2d(p[k], ip, w, h);
        if (k == 0) po = q;
    }
    size_t ro = c.take(8 * 4);
    if (!c.upload()) return 0;
    k_e_sad<<<1, 256, 0, c.c().st>>>(c.dev<pel>(oo), c.dev<pel>(po), w, h, n_pred, ssd, c.dev<u64>(ro));
    count_launch(1);
    if (!c.launched() || !c.download(ro, 32)) return 0;
    const u64 *r = c.host<u64>(ro);
    if (outs)
        for (int k = 0; k < n_pred; k++) outs[k] = (u32)r[k];
    return r[0];
}

static u32 e_satd(int tw, int th, const pel *o, int io, const pel *p, int ip)
{
    Call c(2 * 256 + 64);
    if (!c.ok) return 0;
    size_t oo = c.put2d(o, io, tw, th), po = c.put2d(p, ip, tw, th), ro = c.take(4);
    if (!c.upload()) return 0;
    k_e_satd<<<1, 32, 0, c.c().st>>>(tw, th, c.dev<pel>(oo), c.dev<pel>(po), sqrt(32.0), sqrt(128.0), c.dev<u32>(ro));
    count_launch(1);
    if (!c.launched() || !c.download(ro, 4)) return 0;
    return *c.host<u32>(ro);
}

template <class T> static void unpack2d(T *dst, long long stride, const T *src, int w, int h)
{
    for (int y = 0; y < h; y++) memcpy(dst + (long long)y * stride, src + (size_t)y * w, sizeof(T) * w);
}

static void e_ipcpy(const pel *s, int is, pel *d, int id, int w, int h)
{
    Call c(2 * (size_t)w * h + 64);
    if (!c.ok) return;
    size_t so = c.put2d(s, is, w, h), dof = c.take((size_t)w * h);
    if (!c.upload()) return;
    k_e_copy<<<(w * h + 255) / 256, 256, 0, c.c().st>>>(c.dev<pel>(so), c.dev<pel>(dof), w * h);
    count_launch(1);
    if (!c.launched() || !c.download(dof, (size_t)w * h)) return;
    unpack2d(d, id, c.host<pel>(dof), w, h);
}

static void e_ipflt(int type, const pel *s, int is, pel *d, int id, int w, int h, const s8 *coef, int max_val)
{
    const int taps = (type == 0 || type == 2) ? 8 : 4, back = taps / 2 - 1, vert = type >= 2;
    const int sw = vert ? w : w + taps - 1, sh = vert ? h + taps - 1 : h;
    const pel *s0 = vert ? s - (long long)back * is : s - back;
    Call c((size_t)sw * sh + (size_t)w * h + 64);
    if (!c.ok) return;
    size_t so = c.put2d(s0, is, sw, sh), dof = c.take((size_t)w * h);
    Taps8 t = {};
    for (int k = 0; k < taps; k++) t.c[k] = coef[k];
    if (!c.upload()) return;
    k_e_ipflt<<<(w * h + 255) / 256, 256, 0, c.c().st>>>(c.dev<pel>(so), sw, c.dev<pel>(dof), w, h, taps, vert, t, max_val);
    count_launch(1);
    if (!c.launched() || !c.download(dof, (size_t)w * h)) return;
    unpack2d(d, id, c.host<pel>(dof), w, h);
}

static void e_ipflt_ext(int type, const pel *s, int is, pel *d, int id, int w, int h, const s8 *cx, const s8 *cy, int max_val)
{
    const int taps = type == 0 ? 8 : 4, back = taps / 2 - 1;
    const int sw = w + taps - 1, sh = h + taps - 1;
    Call c((size_t)sw * sh + (size_t)w * h + 64);
    if (!c.ok) return;
    size_t so = c.put2d(s - (long long)back * is - back, is, sw, sh), dof = c.take((size_t)w * h);
    Taps8 tx = {}, ty = {};
    for (int k = 0; k < taps; k++) { tx.c[k] = cx[k]; ty.c[k] = cy[k]; }
    if (!c.upload()) return;
    k_e_ipflt_ext<<<(w * h + 255) / 256, 256, 0, c.c().st>>>(c.dev<pel>(so), sw, c.dev<pel>(dof), w, h, taps, tx, ty, max_val);
    count_launch(1);
    if (!c.launched() || !c.download(dof, (size_t)w * h)) return;
    unpack2d(d, id, c.host<pel>(dof), w, h);
}

static void e_flt_frame(int kind, const pel *src8, const s16 *src16, int is, pel *dst[3], int id, s16 *tmp[3], int it,
                        int w, int h, s8 (*coeff)[8], int bd)
{
    const int sw = kind == 0 ? w + 7 : w, sh = kind == 0 ? h : h + 7;
    const size_t n = (size_t)w * h, esz = kind == 2 ? 2 : 1;
    Call c((size_t)sw * sh * esz + 3 * n * (kind == 0 ? 3 : 1) + 256);
    if (!c.ok) return;
    size_t so = kind == 2 ? c.put2d(src16 - 3LL * is, is, sw, sh)
                          : c.put2d(src8 - (kind == 0 ? 3 : 3LL * is), is, sw, sh);
    size_t dof = c.take(3 * n), tof = kind == 0 ? c.take(3 * n * 2) : 0;
    Taps3x8 t;
    for (int f = 0; f < 3; f++)
        for (int k = 0; k < 8; k++) t.c[f][k] = coeff[f][k];
    if (!c.upload()) return;
    pel *dd = c.dev<pel>(dof);
    s16 *td = kind == 0 ? c.dev<s16>(tof) : nullptr;
    int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
    k_e_flt_frame<<<blocks, 256, 0, c.c().st>>>(kind, kind == 2 ? nullptr : c.dev<pel>(so), kind == 2 ? c.dev<s16>(so) : nullptr,
                                               sw, dd, dd + n, dd + 2 * n, td, td ? td + n : nullptr, td ? td + 2 * n : nullptr,
                                               w, h, t, bd);
    count_launch(1);
    if (!c.launched()) return;
    size_t end = (kind == 0 ? tof + 3 * n * 2 : dof + 3 * n);
    if (!c.download(dof, end - dof)) return;
    for (int f = 0; f < 3; f++) {
        unpack2d(dst[f], id, c.host<pel>(dof) + f * n, w, h);
        if (kind == 0) unpack2d(tmp[f], it, c.host<s16>(tof) + f * n, w, h);
    }
}

static void e_recon(const s16 *resi, const pel *pred, int ip, int w, int h, pel *rec, int ir, int cbf, int bd)
{
    Call c((size_t)w * h * 4 + 64);
    if (!c.ok) return;
    size_t ro = cbf ? c.put(resi, sizeof(s16) * w * h) : c.take(0);
    size_t po = c.put2d(pred, ip, w, h), dof = c.take((size_t)w * h);
    if (!c.upload()) return;
    k_e_recon<<<(w * h + 255) / 256, 256, 0, c.c().st>>>(c.dev<s16>(ro), c.dev<pel>(po), c.dev<pel>(dof), w * h, cbf, bd);
    count_launch(1);
    if (!c.launched() || !c.download(dof, (size_t)w * h)) return;
    unpack2d(rec, ir, c.host<pel>(dof), w, h);
}

static void e_diff(int w, int h, const pel *o, int io, const pel *p, int ip, s16 *r, int ir)
{
    Call c((size_t)w * h * 4 + 64);
    if (!c.ok) return;
    size_t oo = c.put2d(o, io, w, h), po = c.put2d(p, ip, w, h), rof = c.take(sizeof(s16) * w * h);
    if (!c.upload()) return;
    k_e_diff<<<(w * h + 255) / 256, 256, 0, c.c().st>>>(c.dev<pel>(oo), c.dev<pel>(po), c.dev<s16>(rof), w * h);
    count_launch(1);
    if (!c.launched() || !c.download(rof, sizeof(s16) * w * h)) return;
    unpack2d(r, ir, c.host<s16>(rof), w, h);
}

static void e_avrg(int w, int h, pel *d, int id, const pel *s1, const pel *s2)
{
    Call c((size_t)w * h * 3 + 64);
    if (!c.ok) return;
    size_t a = c.put(s1, (size_t)w * h), b = c.put(s2, (size_t)w * h), dof = c.take((size_t)w * h);
    if (!c.upload()) return;
    k_e_avrg<<<(w * h + 255) / 256, 256, 0, c.c().st>>>(c.dev<pel>(a), c.dev<pel>(b), c.dev<pel>(dof), w * h);
    count_launch(1);
    if (!c.launched() || !c.download(dof, (size_t)w * h)) return;
    unpack2d(d, id, c.host<pel>(dof), w, h);
}

// stage the neighbour samples an intra entry can read: [src - R, src + R] with
// R = 4 * max(w, h) + 4 (the range com_intra_get_nbr fills around the array centre)
static void e_intra(int kind, const pel *src, pel *dst, int id, s16 *dst16, const s16 *pred16, int w, int h, int avail,
                    int bd, int entry, int mode)
{
    const int R = 4 * std::max(w, h) + 4;
    Call c(576 + (size_t)w * h * 5 + 64);
    if (!c.ok) return;
    size_t nbo = c.take(576);
    memcpy(c.host<pel>(nbo) + 288 - R, src - R, (size_t)(2 * R + 1));
    size_t dof = c.take((size_t)w * h);
    if (kind == IE_IPF) {
        for (int y = 0; y < h; y++) memcpy(c.host<pel>(dof) + (size_t)y * w, dst + (long long)y * id, w);
    }
    size_t po = kind == IE_IPF_S16 ? c.put(pred16, sizeof(s16) * w * h) : c.take(0);
    size_t d16 = (kind == IE_PLANE_S16 || kind == IE_BI_S16) ? c.take(sizeof(s16) * w * h) : c.take(0);
    if (!c.upload()) return;
    k_e_intra<<<1, 256, 0, c.c().st>>>(kind, c.dev<pel>(nbo), c.dev<pel>(dof), c.dev<s16>(d16), c.dev<s16>(po), w, h,
                                       avail, bd, entry, mode);
    count_launch(1);
    if (!c.launched()) return;
    if (kind == IE_PLANE_S16 || kind == IE_BI_S16) {
        if (!c.download(d16, sizeof(s16) * w * h)) return;
        memcpy(dst16, c.host<s16>(d16), sizeof(s16) * w * h);
        return;
    }
    if (!c.download(dof, (size_t)w * h)) return;
    unpack2d(dst, id, c.host<pel>(dof), w, h);
}

static void e_fdct2(int lw, int lh, const s16 *src, s16 *dst, int bd)
{
    const DevTables *t = tabs();
    if (!t) return;
    const int w = 1 << lw, h = 1 << lh, kw = std::min(w, 32), kh = std::min(h, 32);
    Call c(sizeof(s16) * (size_t)w * h * 3 + 64);
    if (!c.ok) return;
    size_t so = c.put(src, sizeof(s16) * w * h), dof = c.take(sizeof(s16) * w * h), tof = c.take(sizeof(s16) * w * h);
    if (!c.upload()) return;
    k_e_fdct2<<<1, 256, 0, c.c().st>>>(t->fold[lw], t->fold[lh], c.dev<s16>(so), c.dev<s16>(dof), c.dev<s16>(tof), w, h, bd);
    count_launch(1);
    if (!c.launched() || !c.download(dof, sizeof(s16) * w * h)) return;
    for (int v = 0; v < kh; v++) memcpy(dst + v * w, c.host<s16>(dof) + v * w, sizeof(s16) * kw);
}

static void e_idct2(int lh, int lw, const s16 *coef, s16 *resi, int bd)
{
    const DevTables *t = tabs();
    if (!t) return;
    const int w = 1 << lw, h = 1 << lh, kh = std::min(h, 32);
    Call c(sizeof(s16) * (size_t)w * h * 3 + 64);
    if (!c.ok) return;
    size_t co = c.take(sizeof(s16) * w * h);
    memcpy(c.host<s16>(co), coef, sizeof(s16) * w * kh);   // rows >= 32 are never read
    size_t dof = c.take(sizeof(s16) * w * h), tof = c.take(sizeof(s16) * w * h);
    if (!c.upload()) return;
    k_e_idct2<<<1, 256, 0, c.c().st>>>(t->fold[lw], t->fold[lh], c.dev<s16>(co), c.dev<s16>(dof), c.dev<s16>(tof), w, h, bd);
    count_launch(1);
    if (!c.launched() || !c.download(dof, sizeof(s16) * w * h)) return;
    memcpy(resi, c.host<s16>(dof), sizeof(s16) * w * h);
}

static void e_d87(int type, int ln, const s16 *src, s16 *dst, int shift, int line, int inv, int mx, int mn)
{
    const DevTables *t = tabs();
    if (!t) return;
    const int N = 1 << ln;
    Call c(sizeof(s16) * (size_t)N * line * 2 + 64);
    if (!c.ok) return;
    size_t so = c.put(src, sizeof(s16) * N * line), dof = c.take(sizeof(s16) * N * line);
    if (!c.upload()) return;
    k_e_d87<<<(N * line + 255) / 256, 256, 0, c.c().st>>>(t->d87[type][ln], N, c.dev<s16>(so), c.dev<s16>(dof), shift,
                                                          line, inv, mx, mn);
    count_launch(1);
    if (!c.launched() || !c.download(dof, sizeof(s16) * N * line)) return;
    memcpy(dst, c.host<s16>(dof), sizeof(s16) * N * line);
}

static void e_dquant(int flat, const s16 *coef, s16 *out, u8 *wq[2], int lw, int lh, int scale, int shift)
{
    const int w = 1 << lw, h = 1 << lh;
    const int n = flat ? std::min(h, 32) * w : w * h;
    Call c(sizeof(s16) * (size_t)w * h * 2 + 128);
    if (!c.ok) return;
    size_t co = c.put(coef, sizeof(s16) * n);
    size_t w4 = (!flat && wq[0]) ? c.put(wq[0], 16) : c.take(16);
    size_t w8 = (!flat && wq[1]) ? c.put(wq[1], 64) : c.take(64);
    size_t dof = c.take(sizeof(s16) * n);
    if (!c.upload()) return;
    k_e_dquant<<<(n + 255) / 256, 256, 0, c.c().st>>>(flat, c.dev<s16>(co), c.dev<s16>(dof), c.dev<u8>(w4), c.dev<u8>(w8),
                                                      lw, lh, scale, shift);
    count_launch(1);
    if (!c.launched() || !c.download(dof, sizeof(s16) * n)) return;
    memcpy(out, c.host<s16>(dof), sizeof(s16) * n);
}

static int e_quant(int mode, const s16 *coef, int num, int thr, int qv, int qb, s32 es, int pb, u32 *abs_coef,
                   s16 *abs_level, s64 *err)
{
    Call c((size_t)num * 16 + 128);
    if (!c.ok) return mode == 0 ? 0 : -1;
    size_t co = c.put(coef, sizeof(s16) * num);
    size_t ac = mode ? c.put(abs_coef, sizeof(u32) * num) : c.take(0);
    size_t ev = mode ? c.put(err, sizeof(s64) * num) : c.take(0);
    size_t al = mode ? c.take(sizeof(s16) * num) : c.take(0);
    size_t ro = c.take(4);
    if (!c.upload()) return mode == 0 ? 0 : -1;
    k_e_quant<<<1, 256, 0, c.c().st>>>(mode, c.dev<s16>(co), num, thr, qv, qb, es, pb, c.dev<u32>(ac), c.dev<s16>(al),
                                       c.dev<s64>(ev), c.dev<int>(ro));
    count_launch(1);
    if (!c.launched() || !c.download(ac, ro + 4 - ac)) return mode == 0 ? 0 : -1;
    if (mode) {
        memcpy(abs_coef, c.host<u32>(ac), sizeof(u32) * num);
        memcpy(err, c.host<s64>(ev), sizeof(s64) * num);
        memcpy(abs_level, c.host<s16>(al), sizeof(s16) * num);
    }
    return *c.host<int>(ro);
}

}  // namespace uc

using namespace uc;

// ------------------------------------------------------------------ exported entries
extern "C" {

UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_dc(uint8_t *src, uint8_t *dst, int i_dst, int w, int h, uint16_t avail, int bd)
{ e_intra(IE_DC, src, dst, i_dst, nullptr, nullptr, w, h, avail, bd, 0, 0); }
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_plane(uint8_t *src, uint8_t *dst, int i_dst, int w, int h, int bd)
{ e_intra(IE_PLANE, src, dst, i_dst, nullptr, nullptr, w, h, 0, bd, 0, 1); }
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_bi(uint8_t *src, uint8_t *dst, int i_dst, int w, int h, int bd)
{ e_intra(IE_BI, src, dst, i_dst, nullptr, nullptr, w, h, 0, bd, 0, 2); }
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_plane_ipf(uint8_t *src, int16_t *dst, int w, int h)
{ e_intra(IE_PLANE_S16, src, nullptr, w, dst, nullptr, w, h, 0, 8, 0, 1); }
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_bi_ipf(uint8_t *src, int16_t *dst, int w, int h)
{ e_intra(IE_BI_S16, src, nullptr, w, dst, nullptr, w, h, 0, 8, 0, 2); }
// ver / hor receive the array centre +1 / -1 (com_intra_pred, src/com_ipred.c:741-745)
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ver(uint8_t *src, uint8_t *dst, int i_dst, int w, int h)
{ e_intra(IE_VER, src - 1, dst, i_dst, nullptr, nullptr, w, h, 0, 8, 0, 12); }
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_hor(uint8_t *src, uint8_t *dst, int i_dst, int w, int h)
{ e_intra(IE_HOR, src + 1, dst, i_dst, nullptr, nullptr, w, h, 0, 8, 0, 24); }
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ipf_core(uint8_t *src, uint8_t *dst, int i_dst, int ipm, int w, int h, int bd)
{ e_intra(IE_IPF, src, dst, i_dst, nullptr, nullptr, w, h, 0, bd, 0, ipm); }
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ipf_core_s16(uint8_t *src, uint8_t *dst, int i_dst, int16_t *pred, int ipm, int w,
                                                         int h, int bd)
{ e_intra(IE_IPF_S16, src, dst, i_dst, nullptr, pred, w, h, 0, bd, 0, ipm); }

// intra_pred_ang[m]: the specialised entries (4, 6, 8, 10, 13..23, 26, 28, 30, 32) always
// predict their own mode; the generic ones use the mode argument
#define ANG_ENTRY(m, spec)                                                                                       \
    UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_##m(uint8_t *src, uint8_t *dst, int i_dst, int mode, int w, int h) \
    { e_intra(IE_ANG, src, dst, i_dst, nullptr, nullptr, w, h, 0, 8, m, spec ? m : mode); }
ANG_ENTRY(3, 0) ANG_ENTRY(4, 1) ANG_ENTRY(5, 0) ANG_ENTRY(6, 1) ANG_ENTRY(7, 0) ANG_ENTRY(8, 1) ANG_ENTRY(9, 0)
ANG_ENTRY(10, 1) ANG_ENTRY(11, 0) ANG_ENTRY(12, 0) ANG_ENTRY(13, 1) ANG_ENTRY(14, 1) ANG_ENTRY(15, 1)
ANG_ENTRY(16, 1) ANG_ENTRY(17, 1) ANG_ENTRY(18, 1) ANG_ENTRY(19, 1) ANG_ENTRY(20, 1) ANG_ENTRY(21, 1)
ANG_ENTRY(22, 1) ANG_ENTRY(23, 1) ANG_ENTRY(25, 0) ANG_ENTRY(26, 1) ANG_ENTRY(27, 0) ANG_ENTRY(28, 1)
ANG_ENTRY(29, 0) ANG_ENTRY(30, 1) ANG_ENTRY(31, 0) ANG_ENTRY(32, 1)
#undef ANG_ENTRY

UAVS3E_CUDA_API void uavs3e_cuda_ipcpy(const uint8_t *src, int i_src, uint8_t *dst, int i_dst, int w, int h)
{ e_ipcpy(src, i_src, dst, i_dst, w, h); }
UAVS3E_CUDA_API void uavs3e_cuda_ipflt_h8(const uint8_t *s, int is, uint8_t *d, int id, int w, int h, const int8_t *c, int mx)
{ e_ipflt(0, s, is, d, id, w, h, c, mx); }
UAVS3E_CUDA_API void uavs3e_cuda_ipflt_h4(const uint8_t *s, int is, uint8_t *d, int id, int w, int h, const int8_t *c, int mx)
{ e_ipflt(1, s, is, d, id, w, h, c, mx); }
UAVS3E_CUDA_API void uavs3e_cuda_ipflt_v8(const uint8_t *s, int is, uint8_t *d, int id, int w, int h, const int8_t *c, int mx)
{ e_ipflt(2, s, is, d, id, w, h, c, mx); }
UAVS3E_CUDA_API void uavs3e_cuda_ipflt_v4(const uint8_t *s, int is, uint8_t *d, int id, int w, int h, const int8_t *c, int mx)
{ e_ipflt(3, s, is, d, id, w, h, c, mx); }
UAVS3E_CUDA_API void uavs3e_cuda_ipflt_ext8(const uint8_t *s, int is, uint8_t *d, int id, int w, int h, const int8_t *cx,
                                            const int8_t *cy, int mx)
{ e_ipflt_ext(0, s, is, d, id, w, h, cx, cy, mx); }
UAVS3E_CUDA_API void uavs3e_cuda_ipflt_ext4(const uint8_t *s, int is, uint8_t *d, int id, int w, int h, const int8_t *cx,
                                            const int8_t *cy, int mx)
{ e_ipflt_ext(1, s, is, d, id, w, h, cx, cy, mx); }
UAVS3E_CUDA_API void uavs3e_cuda_ip_flt_y_hor(const uint8_t *src, int i_src, uint8_t *dst[3], int i_dst, int16_t *dst_tmp[3],
                                              int i_dst_tmp, int w, int h, int8_t (*coeff)[8], int bd)
{ e_flt_frame(0, src, nullptr, i_src, dst, i_dst, dst_tmp, i_dst_tmp, w, h, coeff, bd); }
UAVS3E_CUDA_API void uavs3e_cuda_ip_flt_y_ver(const uint8_t *src, int i_src, uint8_t *dst[3], int i_dst, int w, int h,
                                              int8_t (*coeff)[8], int bd)
{ e_flt_frame(1, src, nullptr, i_src, dst, i_dst, nullptr, 0, w, h, coeff, bd); }
UAVS3E_CUDA_API void uavs3e_cuda_ip_flt_y_ver_ext(const int16_t *src, int i_src, uint8_t *dst[3], int i_dst, int w, int h,
                                                  int8_t (*coeff)[8], int bd)
{ e_flt_frame(2, nullptr, src, i_src, dst, i_dst, nullptr, 0, w, h, coeff, bd); }

UAVS3E_CUDA_API void uavs3e_cuda_recon(int16_t *resi, uint8_t *pred, int i_pred, int w, int h, uint8_t *rec, int i_rec,
                                       int cbf, int bd)
{ e_recon(resi, pred, i_pred, w, h, rec, i_rec, cbf, bd); }
UAVS3E_CUDA_API void uavs3e_cuda_dquant(int16_t *coef, int16_t *out, uint8_t *wq[2], int lw, int lh, int scale, int shift, int bd)
{ (void)bd; e_dquant(1, coef, out, wq, lw, lh, scale, shift); }
UAVS3E_CUDA_API void uavs3e_cuda_dquant_wq(int16_t *coef, int16_t *out, uint8_t *wq[2], int lw, int lh, int scale, int shift,
                                           int bd)
{ (void)bd; e_dquant(0, coef, out, wq, lw, lh, scale, shift); }

#define TX_ENTRY(W, LW, H, LH)                                                                        \
    UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w##W##_h##H(int16_t *src, int16_t *dst, int bd)       \
    { e_fdct2(LW, LH, src, dst, bd); }                                                                \
    UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h##H##_w##W(int16_t *coef, int16_t *resi, int bd)    \
    { e_idct2(LH, LW, coef, resi, bd); }
TX_ENTRY(4, 2, 4, 2) TX_ENTRY(4, 2, 8, 3) TX_ENTRY(4, 2, 16, 4) TX_ENTRY(4, 2, 32, 5)
TX_ENTRY(8, 3, 4, 2) TX_ENTRY(8, 3, 8, 3) TX_ENTRY(8, 3, 16, 4) TX_ENTRY(8, 3, 32, 5) TX_ENTRY(8, 3, 64, 6)
TX_ENTRY(16, 4, 4, 2) TX_ENTRY(16, 4, 8, 3) TX_ENTRY(16, 4, 16, 4) TX_ENTRY(16, 4, 32, 5) TX_ENTRY(16, 4, 64, 6)
TX_ENTRY(32, 5, 4, 2) TX_ENTRY(32, 5, 8, 3) TX_ENTRY(32, 5, 16, 4) TX_ENTRY(32, 5, 32, 5) TX_ENTRY(32, 5, 64, 6)
TX_ENTRY(64, 6, 8, 3) TX_ENTRY(64, 6, 16, 4) TX_ENTRY(64, 6, 32, 5) TX_ENTRY(64, 6, 64, 6)
#undef TX_ENTRY

#define D87_ENTRY(N, LN)                                                                                         \
    UAVS3E_CUDA_API void uavs3e_cuda_tx_dct8_##N(int16_t *s, int16_t *d, int shift, int line)                    \
    { e_d87(0, LN, s, d, shift, line, 0, 0, 0); }                                                                \
    UAVS3E_CUDA_API void uavs3e_cuda_tx_dst7_##N(int16_t *s, int16_t *d, int shift, int line)                    \
    { e_d87(1, LN, s, d, shift, line, 0, 0, 0); }                                                                \
    UAVS3E_CUDA_API void uavs3e_cuda_itx_dct8_##N(int16_t *c, int16_t *b, int shift, int line, int mx, int mn)   \
    { e_d87(0, LN, c, b, shift, line, 1, mx, mn); }                                                              \
    UAVS3E_CUDA_API void uavs3e_cuda_itx_dst7_##N(int16_t *c, int16_t *b, int shift, int line, int mx, int mn)   \
    { e_d87(1, LN, c, b, shift, line, 1, mx, mn); }
D87_ENTRY(4, 2) D87_ENTRY(8, 3) D87_ENTRY(16, 4) D87_ENTRY(32, 5) D87_ENTRY(64, 6)
#undef D87_ENTRY

#define COST_ENTRY(W)                                                                                              \
    UAVS3E_CUDA_API uint32_t uavs3e_cuda_cost_sad_##W(uint8_t *o, int io, uint8_t *p, int ip, int h)               \
    { const pel *pp[1] = { p }; return (u32)e_sad(W, h, o, io, pp, 1, ip, 0, nullptr); }                          \
    UAVS3E_CUDA_API void uavs3e_cuda_cost_sad_x3_##W(uint8_t *o, int io, uint8_t *p0, uint8_t *p1, uint8_t *p2,     \
                                                     int ip, uint32_t sad[3], int h)                               \
    { const pel *pp[3] = { p0, p1, p2 }; e_sad(W, h, o, io, pp, 3, ip, 0, sad); }                                 \
    UAVS3E_CUDA_API void uavs3e_cuda_cost_sad_x4_##W(uint8_t *o, int io, uint8_t *p0, uint8_t *p1, uint8_t *p2,     \
                                                     uint8_t *p3, int ip, uint32_t sad[4], int h)                  \
    { const pel *pp[4] = { p0, p1, p2, p3 }; e_sad(W, h, o, io, pp, 4, ip, 0, sad); }                             \
    UAVS3E_CUDA_API uint64_t uavs3e_cuda_cost_ssd_##W(uint8_t *o, int io, uint8_t *p, int ip, int h)               \
    { const pel *pp[1] = { p }; return e_sad(W, h, o, io, pp, 1, ip, 1, nullptr); }                               \
    UAVS3E_CUDA_API void uavs3e_cuda_pel_diff_##W(uint8_t *o, int io, uint8_t *p, int ip, int16_t *r, int ir, int h) \
    { e_diff(W, h, o, io, p, ip, r, ir); }                                                                        \
    UAVS3E_CUDA_API void uavs3e_cuda_pel_avrg_##W(uint8_t *d, int id, uint8_t *s1, uint8_t *s2, int h)             \
    { e_avrg(W, h, d, id, s1, s2); }
COST_ENTRY(4) COST_ENTRY(8) COST_ENTRY(16) COST_ENTRY(32) COST_ENTRY(64) COST_ENTRY(128)
#undef COST_ENTRY

#define SATD_ENTRY(TW, TH)                                                                                     \
    UAVS3E_CUDA_API uint32_t uavs3e_cuda_cost_satd_##TW##x##TH(uint8_t *o, int io, uint8_t *p, int ip)         \
    { return e_satd(TW, TH, o, io, p, ip); }
SATD_ENTRY(4, 4) SATD_ENTRY(8, 4) SATD_ENTRY(4, 8) SATD_ENTRY(8, 8) SATD_ENTRY(16, 8) SATD_ENTRY(8, 16)
#undef SATD_ENTRY

UAVS3E_CUDA_API int uavs3e_cuda_quant_rdoq(int16_t *coef, int num, int q_value, int q_bits, int32_t err_scale,
                                           int precision_bits, uint32_t *abs_coef, int16_t *abs_level, int64_t *uncoded_err)
{ return e_quant(1, coef, num, 0, q_value, q_bits, err_scale, precision_bits, abs_coef, abs_level, uncoded_err); }
UAVS3E_CUDA_API int uavs3e_cuda_quant_check(int16_t *coef, int num, int threshold)
{ return e_quant(0, coef, num, threshold, 1, 1, 0, 0, nullptr, nullptr, nullptr); }

UAVS3E_CUDA_API int uavs3e_cuda_install(void *table)
{
    if (!table) return set_status(UC_ERR_ARG, "install: null table");
    int r = ensure_init();
    if (r) return r;
    uavs3e_cuda_funs_t *t = (uavs3e_cuda_funs_t *)table;
    t->intra_pred_dc = uavs3e_cuda_intra_pred_dc;
    t->intra_pred_plane = uavs3e_cuda_intra_pred_plane;
    t->intra_pred_bi = uavs3e_cuda_intra_pred_bi;
    t->intra_pred_plane_ipf = uavs3e_cuda_intra_pred_plane_ipf;
    t->intra_pred_bi_ipf = uavs3e_cuda_intra_pred_bi_ipf;
    t->intra_pred_ver = uavs3e_cuda_intra_pred_ver;
    t->intra_pred_hor = uavs3e_cuda_intra_pred_hor;
    typedef void (*ang_fn)(uint8_t *, uint8_t *, int, int, int, int);
    static const ang_fn ang[33] = {
        nullptr, nullptr, nullptr, uavs3e_cuda_intra_pred_ang_3, uavs3e_cuda_intra_pred_ang_4, uavs3e_cuda_intra_pred_ang_5,
        uavs3e_cuda_intra_pred_ang_6, uavs3e_cuda_intra_pred_ang_7, uavs3e_cuda_intra_pred_ang_8, uavs3e_cuda_intra_pred_ang_9,
        uavs3e_cuda_intra_pred_ang_10, uavs3e_cuda_intra_pred_ang_11, uavs3e_cuda_intra_pred_ang_12,
        uavs3e_cuda_intra_pred_ang_13, uavs3e_cuda_intra_pred_ang_14, uavs3e_cuda_intra_pred_ang_15,
        uavs3e_cuda_intra_pred_ang_16, uavs3e_cuda_intra_pred_ang_17, uavs3e_cuda_intra_pred_ang_18,
        uavs3e_cuda_intra_pred_ang_19, uavs3e_cuda_intra_pred_ang_20, uavs3e_cuda_intra_pred_ang_21,
        uavs3e_cuda_intra_pred_ang_22, uavs3e_cuda_intra_pred_ang_23, nullptr, uavs3e_cuda_intra_pred_ang_25,
        uavs3e_cuda_intra_pred_ang_26, uavs3e_cuda_intra_pred_ang_27, uavs3e_cuda_intra_pred_ang_28,
        uavs3e_cuda_intra_pred_ang_29, uavs3e_cuda_intra_pred_ang_30, uavs3e_cuda_intra_pred_ang_31,
        uavs3e_cuda_intra_pred_ang_32 };
    for (int m = 3; m < 33; m++)
        if (ang[m]) t->intra_pred_ang[m] = ang[m];
    t->intra_pred_ipf_core = uavs3e_cuda_intra_pred_ipf_core;
    t->intra_pred_ipf_core_s16 = uavs3e_cuda_intra_pred_ipf_core_s16;
    for (int i = 0; i < 6; i++) {
        t->ipcpy[i] = uavs3e_cuda_ipcpy;
        t->ipflt[0][i] = uavs3e_cuda_ipflt_h8;
        t->ipflt[1][i] = uavs3e_cuda_ipflt_h4;
        t->ipflt[2][i] = uavs3e_cuda_ipflt_v8;
        t->ipflt[3][i] = uavs3e_cuda_ipflt_v4;
        t->ipflt_ext[0][i] = uavs3e_cuda_ipflt_ext8;
        t->ipflt_ext[1][i] = uavs3e_cuda_ipflt_ext4;
        t->recon[i] = uavs3e_cuda_recon;
    }
    t->ip_flt_y_hor = uavs3e_cuda_ip_flt_y_hor;
    t->ip_flt_y_ver = uavs3e_cuda_ip_flt_y_ver;
    t->ip_flt_y_ver_ext = uavs3e_cuda_ip_flt_y_ver_ext;
    t->dquant[0] = uavs3e_cuda_dquant_wq;
    t->dquant[1] = uavs3e_cuda_dquant;
#define SETTX(W, LW, H, LH)                                                 \
    t->trans_dct2[LW - 1][LH - 1] = uavs3e_cuda_trans_dct2_w##W##_h##H;     \
    t->itrans_dct2[LH - 1][LW - 1] = uavs3e_cuda_itrans_dct2_h##H##_w##W;
    SETTX(4, 2, 4, 2) SETTX(4, 2, 8, 3) SETTX(4, 2, 16, 4) SETTX(4, 2, 32, 5)
    SETTX(8, 3, 4, 2) SETTX(8, 3, 8, 3) SETTX(8, 3, 16, 4) SETTX(8, 3, 32, 5) SETTX(8, 3, 64, 6)
    SETTX(16, 4, 4, 2) SETTX(16, 4, 8, 3) SETTX(16, 4, 16, 4) SETTX(16, 4, 32, 5) SETTX(16, 4, 64, 6)
    SETTX(32, 5, 4, 2) SETTX(32, 5, 8, 3) SETTX(32, 5, 16, 4) SETTX(32, 5, 32, 5) SETTX(32, 5, 64, 6)
    SETTX(64, 6, 8, 3) SETTX(64, 6, 16, 4) SETTX(64, 6, 32, 5) SETTX(64, 6, 64, 6)
#undef SETTX
#define SET87(N, LN)                                                 \
    t->trans_dct8_dst7[0][LN - 1] = uavs3e_cuda_tx_dct8_##N;         \
    t->trans_dct8_dst7[1][LN - 1] = uavs3e_cuda_tx_dst7_##N;         \
    t->itrans_dct8_dst7[0][LN - 1] = uavs3e_cuda_itx_dct8_##N;       \
    t->itrans_dct8_dst7[1][LN - 1] = uavs3e_cuda_itx_dst7_##N;
    SET87(4, 2) SET87(8, 3) SET87(16, 4) SET87(32, 5) SET87(64, 6)
#undef SET87
#define SETC(W, I)                                     \
    t->cost_sad[I] = uavs3e_cuda_cost_sad_##W;         \
    t->cost_sad_x3[I] = uavs3e_cuda_cost_sad_x3_##W;   \
    t->cost_sad_x4[I] = uavs3e_cuda_cost_sad_x4_##W;   \
    t->cost_ssd[I] = uavs3e_cuda_cost_ssd_##W;         \
    t->pel_diff[I] = uavs3e_cuda_pel_diff_##W;         \
    t->pel_avrg[I] = uavs3e_cuda_pel_avrg_##W;
    SETC(4, 0) SETC(8, 1) SETC(16, 2) SETC(32, 3) SETC(64, 4) SETC(128, 5)
#undef SETC
    t->cost_satd[0][0] = uavs3e_cuda_cost_satd_4x4;
    t->cost_satd[1][0] = uavs3e_cuda_cost_satd_8x4;
    t->cost_satd[0][1] = uavs3e_cuda_cost_satd_4x8;
    t->cost_satd[1][1] = uavs3e_cuda_cost_satd_8x8;
    t->cost_satd[2][1] = uavs3e_cuda_cost_satd_16x8;
    t->cost_satd[1][2] = uavs3e_cuda_cost_satd_8x16;
    t->quant_rdoq = uavs3e_cuda_quant_rdoq;
    t->quant_check = uavs3e_cuda_quant_check;
    return UC_OK;
}

}  // extern "C"
