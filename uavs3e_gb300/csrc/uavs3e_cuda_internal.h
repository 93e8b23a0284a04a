// Internal declarations shared between the .cu translation units of libuavs3e_cuda.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "common.cuh"
#include "../../include/uavs3e_cuda.h"

namespace uc {

struct PlaneSet15 { pel *p[15]; };

constexpr int ME_MAX_REFS = 4;
constexpr int ME_CTU = 64;
constexpr int ME_BLOCKS_PER_CTU = 169;
constexpr int ME_GROUPS = 16;          // lane groups (half-warps) per search CTA
constexpr int ME_RANK_BITS = 11;
constexpr int ME_NDY = 8;              // vertically adjacent candidates per search item
constexpr int ME_CLASSES = 4;          // horizontal offsets are split by residue mod 4 (one per CTA)
constexpr int ME_MAX_GROUP = 1 << ME_RANK_BITS;

// canonical per-CTU block list: shapes 8x8, 16x8, 8x16, 16x16, 32x16, 16x32, 32x32, 64x32,
// 32x64, 64x64, each in raster order of its positions inside the 64x64 CTU
struct CtuBlock { u8 x, y, w, h; };
void ctu_block_table(CtuBlock out[ME_BLOCKS_PER_CTU]);

// result record of one (block, reference), same layout as uavs3e_cuda_me_result_t
struct MeResult {
    s16 mv_int[2];
    s16 mv_sub[2];
    u32 sad_int;
    u32 satd_sub;
    u64 cost_int;
    u64 cost_sub;
};

// optional per-kernel timing with CUDA events on the launching stream
enum ProfKernel { PROF_PAD = 0, PROF_SUBPEL = 1, PROF_ME_INT = 2, PROF_ME_SUB = 3, PROF_LATTICE = 4, PROF_LOKA = 5, PROF_TZ = 6, PROF_MC = 7, PROF_RDOQ = 8, PROF_AFFME = 9, PROF_SHIFT = 10, PROF_N = 12 };
int ensure_init();   // selects the library's device (initialising device 0 on first use)
int me_frame_once(); // one-time per-device setup of the frame search (me.cu)
// per-call TZ motion searches (tz.cu); planes: n_slots * 16 sample-(0,0) pointers
// CU motion compensation (mc.cu); chroma: n_slots * 2 sample-(0,0) pointers (U, V)
int launch_mc_cu(int W, int H, const uint8_t *const *planes, int n_slots, int i_ref, int pad,
                 const uint8_t *const *chroma, int i_c, int pad_c, const void *reqs, int n, uint8_t *out,
                 unsigned long long out_bytes, cudaStream_t st);
int launch_mc_affine(int W, int H, const uint8_t *const *planes, int n_slots, int i_ref, int pad,
                     const uint8_t *const *chroma, int i_c, int pad_c, const void *reqs, int n, uint8_t *out,
                     unsigned long long out_bytes, cudaStream_t st);
int launch_coef_rate(const void *reqs, int n, const int16_t *levels, unsigned long long n_levels, void *out,
                     cudaStream_t st);
int launch_intra_rmd(const uint32_t *satd, unsigned long long n_rows, const void *reqs, int n, void *out,
                     cudaStream_t st);
int launch_me_affine(int W, int H, const uint8_t *org, int i_org, const uint8_t *const *planes, int n_slots,
                     int i_ref, int pad, const void *reqs, int n, void *out, cudaStream_t st);
int launch_me_tz(const uavs3e_cuda_tz_pic_t *pic, const uint8_t *org, int i_org, const uint8_t *const *planes,
                 int n_slots, int i_ref, int pad, const void *reqs, int n, void *out, cudaStream_t st);
void prof_begin(int k, cudaStream_t st);
void prof_end(int k, cudaStream_t st);
void count_launch(int n);

int launch_subpel_planes(const pel *src, int stride, int W, int H, int pad, const PlaneSet15 &out, cudaStream_t st);

// integer search + quarter-sample refinement over every CTU block of the frame
struct MeFrameArgs {
    const pel *org; int i_org;
    const pel *planes[ME_MAX_REFS][16]; int i_ref, pad;
    int W, H, n_refs, range;
    u32 lambda_mv;
    MeResult *out;                      // [n_ctu][169][n_refs]
    // device copies of the host-built search tables (me_build_tables)
    const u32 *q2tab; const u16 *rank2mv;
    u32 *sub_scratch;                   // me_sub_scratch_bytes(): per-candidate SATD sums
    pel *shift_scratch;                 // me_shift_scratch_bytes(): byte-shifted reference copies
    bool shift_ready;                   // the copies are current (else made from planes[r][0])
};
size_t me_sub_scratch_bytes(int W, int H, int n_refs);
// the four byte-shifted copies of every reference's integer plane read by the integer search
// (padding 144, row pitch a multiple of 16)
size_t me_shift_scratch_bytes(int W, int H, int n_refs);
struct MeShiftSrc { const pel *plane[ME_MAX_REFS]; int stride, n_refs; };
// writes the four shifted copies of each listed integer plane (padded by >= 144, stride i_ref)
// into dst, laid out [ref][shift] as me_shift_scratch_bytes() sizes them
int launch_shift_planes(const pel *const *planes, int n_refs, int i_ref, int W, int H, pel *dst, cudaStream_t st);

struct MeTables {
    int lo_x, hi_x, lo_y, hi_y, ndx, ndy, ndy_per_item;
    int nfull, rem;                     // full ndy_per_item-row chunks, rows left over
    int n_entries;                      // u32 entries of the table buffer in use
    // per alignment class (dx index mod 4): offsets, main and tail item counts, table offsets
    int n_dx[ME_CLASSES], n_main[ME_CLASSES], n_tail[ME_CLASSES];
    int q2_main[ME_CLASSES], q2_tail[ME_CLASSES], d_main[ME_CLASSES], d_tail[ME_CLASSES];
    u32 lambda_mv;
};
// one candidate of a lane group while its ranks are built
struct MeCand { u32 r, raster, pos; };
constexpr int ME_R2M_ENTRIES = ME_CLASSES * ME_GROUPS * ME_MAX_GROUP;   // rank -> raster map
// builds the packed (q << 11 | rank) table (me_q2_entries) and the rank -> raster map
// (ME_R2M_ENTRIES) on the host; cand is ME_MAX_GROUP entries of work space
int me_build_tables(int W, int H, int range, u32 lambda_mv, int ndy_per_item, MeTables *t,
                    u32 *q2tab, u16 *rank2mv, size_t q2cap, MeCand *cand);
// u32 entries of the search-table buffer (q2 entries, then item descriptors) for a search
// range: per class at most ceil(nd/4) horizontal offsets, ceil(nd/8) main chunks and 7 tail
// rows, each list padded to a multiple of ME_GROUPS items
constexpr size_t me_q2_entries(int range, int ndy_per_item)
{
    return ME_CLASSES * ((ndy_per_item + 1) * (((2 * (size_t)range + 1 + ME_CLASSES - 1) / ME_CLASSES) *
                                                   ((2 * (size_t)range + 1 + ndy_per_item - 1) / ndy_per_item) +
                                               ME_GROUPS) +
                         2 * (((2 * (size_t)range + 1 + ME_CLASSES - 1) / ME_CLASSES) * (ndy_per_item - 1) + ME_GROUPS));
}
// per-block integer winners ([ctu][ref][169] u64) followed by two control words (the search's
// status word is the second); all preset to 0xFF bytes by each frame's search
size_t me_key_scratch_bytes(int W, int H, int n_refs);
u32 me_mvbits(int v);   // MV bits of one quarter-sample component (host)
int launch_me_frame(const MeFrameArgs &a, const MeTables &t, u64 *keys, cudaStream_t st);

}  // namespace uc
