/*
 * oracle.h -- CPU restatement of uavs3e's mode-decision kernels (8-bit luma).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle for the GPU path: the parity tests,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg call it; the product library
 * (libuavs3e_cuda) never links, loads or falls back to it.
 *
 * Every function restates the algorithm of the reference function cited beside it
 * (paths relative to the uavs3e source tree).  The restatement is pinned against the
 * reference compiled from its own sources (oracle/Makefile "ref") by
 * tests/golden/make_golden.py, whose vectors are committed under tests/golden/.
 */
#ifndef UAVS3E_ORACLE_H
#define UAVS3E_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef uint8_t  pel;
typedef int8_t   s8;
typedef int16_t  s16;
typedef int32_t  s32;
typedef int64_t  s64;
typedef uint8_t  u8;
typedef uint16_t u16;
typedef uint32_t u32;
typedef uint64_t u64;

#define ORC_NEIB_SIZE 576           /* INTRA_NEIB_SIZE, inc/com_define.h:277 */
#define ORC_NEIB_MID  288

void orc_init(void);

/* tables */
const s8  *orc_dct_table(int log2n);                 /* [3][N][N]: DCT2, DCT8, DST7 */
const u16 *orc_scan(int log2w, int log2h);           /* zig-zag scan, src/com_util.c:1220 */
const s8  *orc_mc_luma_coef(void);                   /* [4][8] */
const s8  *orc_mc_chroma_coef(void);                 /* [8][4] */
u16        orc_quant_scale(int qp);
u32        orc_dq_scale(int qp);
u32        orc_dq_shift(int qp);
s32        orc_rdoq_err_scale(int qp, int log2_size_minus1);
double     orc_tbl_sqrt(int i);
void       orc_mvbits_table(u8 *tab, int offset);    /* fills tab[0 .. 2*offset], centre at tab[offset] */

/* costs, src/com_cost.c */
u32  orc_sad(int w, int h, const pel *o, int io, const pel *p, int ip);
u64  orc_ssd(int w, int h, const pel *o, int io, const pel *p, int ip);
u32  orc_satd_tile(int tw, int th, const pel *o, int io, const pel *p, int ip);  /* cost_satd[][] */
u32  orc_had(int w, int h, const pel *o, int io, const pel *p, int ip, int bd);  /* com_had */
u32  orc_satd_intra(int w, int h, const pel *o, const pel *p, int io, int ip, int bd);

/* motion compensation, src/com_mc.c */
void orc_ipcpy(const pel *s, int is, pel *d, int id, int w, int h);
void orc_ipflt(int type, const pel *s, int is, pel *d, int id, int w, int h, const s8 *c, int max_val);
void orc_ipflt_ext(int type, const pel *s, int is, pel *d, int id, int w, int h, const s8 *cx, const s8 *cy, int max_val);
void orc_if_luma_frame(pel *plane0, pel **planes15, int width, int height, int pad, int stride);

/* pel ops, src/com_util.c */
void orc_pel_diff(int w, int h, const pel *o, int io, const pel *p, int ip, s16 *r, int ir);
void orc_pel_avrg(int w, int h, pel *d, int id, const pel *s1, const pel *s2);
void orc_recon(const s16 *resi, const pel *pred, int ipred, int w, int h, pel *rec, int irec, int cbf, int bd);

/* intra, src/com_ipred.c */
void orc_intra_get_nbr(int x, int y, int w, int h, const pel *src, int s_src, const pel *top, int lcu_size, int avail,
                       pel *nb_out, int scup, const u8 *coded, int i_scu, int bd);
void orc_intra_pred(const pel *nb, pel *dst, int ipm, int w, int h, int bd, int avail, int ipf);
void orc_ipred_ang(const pel *nb, pel *dst, int i_dst, int mode, int w, int h);     /* intra_pred_ang[mode] */
void orc_ipred_dc(const pel *nb, pel *dst, int i_dst, int w, int h, int avail, int bd);
void orc_ipred_plane(const pel *nb, pel *dst, int i_dst, int w, int h, int bd);
void orc_ipred_bi(const pel *nb, pel *dst, int i_dst, int w, int h, int bd);
void orc_ipred_plane_ipf(const pel *nb, s16 *dst, int w, int h);
void orc_ipred_bi_ipf(const pel *nb, s16 *dst, int w, int h);
void orc_ipf_core(const pel *nb, pel *dst, int i_dst, int ipm, int w, int h, int bd);
void orc_ipf_core_s16(const pel *nb, pel *dst, int i_dst, const s16 *pred, int ipm, int w, int h, int bd);

/* transforms and quantisation, src/transform.c, src/com_itdq.c */
void orc_trans_dct2(int log2w, int log2h, const s16 *src, s16 *dst, int bd);
void orc_trans_dct8_dst7(int type, int log2n, const s16 *src, s16 *dst, int shift, int line);
void orc_transform(int tb_nxn, int blk_idx, s16 *coef, const s16 *resi, int log2w, int log2h, int bd, int sec, int alt4);
void orc_itrans_dct2(int log2h, int log2w, const s16 *coef, s16 *resi, int bd);
void orc_itrans_dct8_dst7(int type, int log2n, const s16 *coef, s16 *blk, int shift, int line, int max_v, int min_v);
void orc_dquant(int flat, const s16 *coef, s16 *out, const u8 *wq4, const u8 *wq8, int log2w, int log2h, int scale, int shift, int bd);
void orc_invqt(int tb_nxn, int blk_idx, const s16 *coef, s16 *resi, const u8 *wq4, const u8 *wq8, int log2w, int log2h, int qp, int bd, int sec, int alt4);
int  orc_quant_check(const s16 *coef, int num, int threshold);
int  orc_quant_rdoq(const s16 *coef, int num, int q_value, int q_bits, s32 err_scale, int precision_bits,
                    u32 *abs_coef, s16 *abs_level, s64 *uncoded_err);

/* ---------------- batched workloads (the GPU path's batch definitions) ---------------- */

/* one motion-search block: position and size in luma samples */
typedef struct { s16 x, y; u8 w, h; u16 pad; } orc_me_block_t;

/* per (block, reference) result of the batched motion search */
typedef struct {
    s16 mv_int[2];      /* best integer MV, integer-sample units            */
    s16 mv_sub[2];      /* best quarter-sample MV after hpel+qpel refinement  */
    u32 sad_int;        /* SAD at mv_int                                     */
    u32 satd_sub;       /* SATD (com_had) at mv_sub                          */
    u64 cost_int;       /* (SAD << 16) + mvbits * lambda_mv at mv_int        */
    u64 cost_sub;       /* (SATD << 16) + mvbits * lambda_mv at mv_sub       */
} orc_me_result_t;

/*
 * Full-search integer ME over [-range, range]^2 (clipped to the encoder's MV limits), then
 * hpel and qpel SATD refinement on the 15 fractional planes, for every block and reference.
 * planes[r*16 + dy*4 + dx] is the (dy,dx) quarter-sample plane of reference r (index 0 =
 * the integer plane), all with stride i_ref and a padding of at least 144 samples.
 * Results are written to out[b * n_refs + r].  Uses OpenMP over blocks when threads > 1.
 */
void orc_me_frame(const pel *org, int i_org, const pel *const *planes, int i_ref, int width, int height,
                  int n_refs, const orc_me_block_t *blocks, int n_blocks, int range, u32 lambda_mv,
                  orc_me_result_t *out, int threads);

/* one intra lattice CU */
typedef struct { s16 x, y; u8 w, h; u16 pad; } orc_cu_t;

/* per (CU, mode, QP) result of the intra lattice */
typedef struct {
    u32 ssd;            /* SSD(org, recon)                        */
    u32 coef_hash;      /* hash of the quantised levels (raster)  */
    u16 num_nz;         /* non-zero quantised levels              */
    s16 last_nz;        /* last non-zero position in scan order   */
    u32 sum_abs;        /* sum of |level|                         */
} orc_lat_q_t;

/*
 * Intra lattice: for each CU and each of the 33 luma modes: neighbours from `rec` (every
 * in-picture sample outside the CU counts as reconstructed), prediction (com_intra_pred,
 * ipf flag as given), SATD against org, residual, forward DCT2, then for each QP: first-pass
 * quantisation (quant_check + quant_rdoq level), dequantisation, inverse DCT2,
 * reconstruction and SSD.  satd_out[cu*33 + m]; q_out[(cu*33 + m)*n_qp + q].
 */
void orc_intra_lattice(const pel *org, int i_org, const pel *rec, int i_rec, int width, int height,
                       const orc_cu_t *cus, int n_cus, int ipf, const int *qps, int n_qp, int is_intra_slice,
                       u32 *satd_out, orc_lat_q_t *q_out, int threads);

/* level hash used by the lattice: sum over positions of level * ((pos * 0x9E3779B1 + 0x7F4A7C15) | 1),
 * mod 2^32 (pos = raster index in the w x h block) */
u32 orc_level_hash(const s16 *lev, int n);

/* ------------- lookahead cost estimation (loka_estimate_coding_cost, src/lookahead.c:82) ------------- */

#define ORC_LOKA_MAX_REFS 4             /* MAX_NUM_ACTIVE_REF_FRAME, inc/com_define.h:297 */

/* the picture-level inputs of one call: the inter_search_t fields its search reads
 * (inter_search_init, src/inter.c:2015) and the POCs that set the raster range */
typedef struct {
    int width, height;                  /* luma picture size                                   */
    int is_padding;                     /* 1: references padded by >= 144 samples (encoder);  */
                                        /* 0: MVs keep the unit inside the picture (lookahead) */
    int max_search_range;               /* 64 (low delay) or 384 (random access)               */
    int gop_size;
    int num_ref[2];                     /* references per list (<= ORC_LOKA_MAX_REFS)         */
    s64 ptr;                            /* POC of the current picture                          */
    s64 ref_ptr[2][ORC_LOKA_MAX_REFS];  /* POC of each reference                               */
} orc_loka_cfg_t;

/* per 16x16 unit (raster order over (width/16) x (height/16)) */
typedef struct {
    s16 mv[2][ORC_LOKA_MAX_REFS][2];    /* integer MV found by me_search_tz per list/ref       */
    u32 satd[2][ORC_LOKA_MAX_REFS];     /* com_had of the block at that MV                     */
    u32 bi_satd;                        /* average of the two list winners (bi pictures)       */
    u32 zero_satd;                      /* average of the (0,0) blocks of ref_l0[0], ref_l1[0] */
    u32 min_cost;                       /* min over the inter and intra costs                  */
    u32 min_icost;                      /* min over the 11 intra modes                         */
    u32 icost_u, icost_v;               /* 8x8 chroma SATD with the best luma mode             */
    u64 energy;                         /* cost_var of Y 16x16 + U 8x8 + V 8x8                 */
    u8  best_mode, pad[7];
} orc_loka_unit_t;

/* every unit's record; ref_l0/ref_l1 point at sample (0,0) of each reference luma plane
 * (stride i_ref).  Uses OpenMP over units when threads > 1. */
void orc_loka_units(const orc_loka_cfg_t *cfg, const pel *org_y, int i_org, const pel *org_u, const pel *org_v,
                    int i_org_c, const pel *const *ref_l0, const pel *const *ref_l1, int i_ref,
                    orc_loka_unit_t *units, int threads);
/* ----------------------- per-call TZ motion search (me_search_tz, src/me.c:529-568) ----------------------- */

/* one call of me_search_tz: the block, the reference (a slot of the planes array), and the
 * inter_search_t state the call reads */
typedef struct {
    s16 x, y;           /* block position (luma samples)                                  */
    u8  w, h;           /* block size, 4..64                                             */
    u8  ref_slot;       /* planes of pi->ref_pic: planes[ref_slot * 16 + phase]           */
    s8  refi;           /* reference index in its list (raster step, reference bits)      */
    u8  num_refp;       /* pi->num_refp                                                   */
    u8  mvr;            /* pi->curr_mvr, 0 (quarter) .. 4 (4 samples)                     */
    u8  bi;             /* 1: search against 2 org - the other list's prediction          */
    u8  flags;          /* bit 0: subpel_cost_type (SAD), bit 1: adaptive_raster_range    */
    s16 mvp[2];         /* predictor, quarter samples (a multiple of 1 << mvr)            */
    s16 mv[2];          /* bi: start MV (quarter samples, a multiple of 1 << mvr)         */
    s16 mv_ipel[2];     /* pi->mv_ipel[lidx][refi] (adaptive raster range), samples       */
    s16 other_mv[2];    /* bi: MV of the other list (quarter samples)                     */
    u8  other_slot;     /* bi: planes slot of the other list's reference                  */
    u8  pad0[3];
    s32 mot_bits_other; /* bi: pi->mot_bits of the other list                             */
    u32 lambda_mv;
    s32 dist;           /* |POC of the picture - POC of the reference|                    */
    s32 pad1;
} orc_tz_req_t;

typedef struct {
    s16 mv[2];          /* the MV me_search_tz writes (quarter samples)                   */
    s16 mv_ipel[2];     /* the integer winner it stores in pi->mv_ipel (uni searches)     */
    u64 cost;           /* its return value; UINT64_MAX when the MV range is empty        */
} orc_tz_out_t;

typedef struct { int width, height, is_padding, max_search_range, gop_size; } orc_tz_pic_t;

/* ------------------------- CU motion compensation (com_mc_cu, src/com_mc.c:140-200) ------------------------- */

typedef struct {
    s16 x, y;           /* CU position (luma samples)                                              */
    u8  w, h;           /* CU size, 8..64 (powers of two)                                          */
    s8  slot[2];        /* reference slot of list 0 / list 1, -1 when the list is unused           */
    s16 mv[2][2];       /* quarter-sample MVs                                                      */
    u8  channel;        /* channel_type_t: 0 luma and chroma, 1 luma, 2 chroma                     */
    u8  pad[3];
    u32 out_offset;     /* byte offset of the CU's prediction: Y (w x h), then U and V (w/2 x h/2) */
} orc_mc_req_t;

/* ------------- RDOQ of a transform block (quant_non_zero + rdoq_quant_block, src/quant.c:196-383) ------------- */

/* the bin-cost estimates rdoq_init_cu_est_bits (src/quant.c:139-156) derives from the entropy
 * coder's context state (core_t rdoq_bin_est_*, inc/define.h:335-339) */
typedef struct {
    s32 ctp[2];
    s32 cbf[3][2];
    s32 run[24][2];
    s32 lvl[24][2];
    s32 lst[2][6][12][2];
} orc_rdoq_est_t;

typedef struct {
    u32 coef_offset;    /* first coefficient (s16 index) of the w x h block (raster)            */
    u8  log2w, log2h;   /* 2..6                                                                 */
    u8  qp;             /* 0..79 (quantisation step index)                                      */
    u8  is_intra;
    u8  ch_type;        /* 0 Y, 1 U, 2 V                                                        */
    u8  slice_type;     /* 1 = SLICE_I                                                          */
    u16 est;            /* index of the estimate set                                            */
    u32 pad;
    s64 lambda;         /* (s64)(d_lambda * 2^15 + 0.5), as rdoq_quant_block forms it           */
} orc_rdoq_req_t;

/* quant_non_zero with flat quantisation for every block: levels written over the coefficients
 * (unchanged when quant_check finds no coefficient above the threshold), num_nz[i] returned */
void orc_rdoq(const orc_rdoq_req_t *reqs, int n, const orc_rdoq_est_t *ests, s16 *coefs, s32 *num_nz);

/* quant_non_zero with pic_wq_enable (src/quant.c:315-383): the zero-out past 32, then plain
 * quantisation with the weights of wq4 (4x4 blocks, 16) or wq8 (the others, 64; one weight per
 * block of samples); lambda and est of the requests are not used */
void orc_quant_wq(const orc_rdoq_req_t *reqs, int n, const u8 *wq4, const u8 *wq8, s16 *coefs, s32 *num_nz);

/* one affine CU (com_mc_cu_affine, src/com_mc.c:361-422) */
typedef struct {
    s16 x, y;           /* CU position                                                            */
    u8  w, h;           /* CU size, 16..64 (powers of two)                                        */
    s8  slot[2];        /* reference slot of list 0 / list 1, -1 when unused                      */
    u8  cp_num;         /* control points, 2 or 3                                                 */
    u8  sub8;           /* pichdr->affine_subblk_size_idx (1: 8x8 sub-blocks)                     */
    u8  pad[2];
    s32 cpmv[2][3][2];  /* control-point MVs per list, 1/16 samples                              */
    u32 out_offset;     /* Y (w x h), then U and V (w/2 x h/2)                                    */
} orc_affine_req_t;

/* affine CU predictions: luma by the 16-phase 8-tap filters from the integer planes
 * (planes[slot * 16]), chroma by the 32-phase 4-tap filters (chroma[slot * 2 + c]) */
void orc_mc_affine(int width, int height, const pel *const *planes, int i_ref, const pel *const *chroma, int i_c,
                   const orc_affine_req_t *reqs, int n, pel *out);

/* luma from the quarter-sample planes (planes[slot * 16 + phase], stride i_ref), chroma with the
 * 4-tap filters from chroma[slot * 2 + (0 U, 1 V)] (stride i_c, padded by >= 72) */
void orc_mc_cu(int width, int height, const pel *const *planes, int i_ref, const pel *const *chroma, int i_c,
               const orc_mc_req_t *reqs, int n, pel *out);

/* planes[slot * 16 + dy * 4 + dx]: the quarter-sample planes of each reference (0 = integer),
 * stride i_ref, padded by >= 144.  Uses OpenMP over requests when threads > 1. */
void orc_me_tz(const orc_tz_pic_t *pic, const pel *org, int i_org, const pel *const *planes, int i_ref,
               const orc_tz_req_t *reqs, int n, orc_tz_out_t *out, int threads);

/* ------------- coefficient rate (lbac_enc_run_length_cc_rdo, src/entropy.c:1688-1950) ------------- */

/* one transform block's levels coded in counting mode from a coder state: the context models of
 * its channel (luma or chroma half of run, run_rdoq, level, last1, last2) and the range */
typedef struct {
    s16 run[12], run_rdoq[12], level[12], last1[6], last2[12];
} orc_coef_ctx_t;

typedef struct {
    u32 coef_offset;    /* first level (s16 index) of the w x h block, raster order                */
    u8  log2w, log2h;   /* 2..6 (luma) / 2..5 (chroma)                                             */
    u8  ch_type;        /* 0 luma, 1 chroma                                                        */
    u8  pad;
    u16 num_sig;        /* non-zero levels of the block (>= 1)                                     */
    u16 range;          /* coder range before the block, 256..511                                  */
    orc_coef_ctx_t ctx; /* context models before the block                                         */
} orc_coef_rate_req_t;

typedef struct {
    u32 bits;           /* the bits the block adds (lbac bitcounter)                               */
    u16 range;          /* range after it                                                          */
    u16 pad;
    orc_coef_ctx_t ctx; /* context models after it                                                 */
} orc_coef_rate_out_t;

void orc_coef_rate(const s16 *levels, const orc_coef_rate_req_t *reqs, int n, orc_coef_rate_out_t *out);
/* one context-model update of the coder (the reference's tbl_plps / tbl_plps_ext, src/entropy.c:41) */
int orc_lbac_next(int model, int mps);

/* ------------- intra mode candidates (make_ipred_list, src/intra.c:236-367) ------------- */

/* one prediction block's candidate search: the SATD of each of its 33 modes comes from a
 * satd[satd_row * 33 + mode] array (the lattice's records), the rate of each mode from the
 * counting-mode LBAC coding of intra_dir (lbac_enc_intra_dir, src/entropy.c:2118) from the state
 * core->lbac_bakup holds: its range and the 7 intra_dir context models */
typedef struct {
    u32 satd_row;
    u8  pb_w, pb_h;     /* prediction block size                                                  */
    u8  mpm[2];         /* cur_info->mpm[part_idx] (33 = IPD_IPCM)                                */
    u8  skip_ipd;       /* skip DC, planar, bilinear                                              */
    u8  fast;           /* info->intra_fast_rmd                                                   */
    u16 range;          /* lbac_bakup.range, 256..511                                             */
    s16 ctx[7];         /* lbac_bakup.h.intra_dir[0..6]                                           */
    u8  pad[6];
    double sqrt_lambda; /* core->sqrt_lambda[0]                                                   */
    u64 inter_satd;     /* core->inter_satd (UINT64_MAX: no inter candidate yet)                  */
    double satd_threshold;
} orc_rmd_req_t;

typedef struct {
    s8 list[5];         /* ipred_list[0..4] as make_ipred_list leaves them                        */
    u8 count;           /* its return value (the candidates the RDO takes)                        */
    u8 pad[2];
} orc_rmd_out_t;

void orc_intra_rmd(const u32 *satd, const orc_rmd_req_t *reqs, int n, orc_rmd_out_t *out);
/* bits of intra prediction mode ipm (lbac_enc_intra_dir in counting mode) */
int orc_intra_dir_bits(int range, const s16 *ctx, int ipm, const u8 *mpm);

/* ------------- affine motion search (affine_me_gradient, src/inter.c:1339-1470) ------------- */

#define ORC_AFFME_BI        1   /* bi argument: org = 2 org - the other list's prediction (8x8 sub-blocks) */
#define ORC_AFFME_UNI_START 2   /* start CPMVs chosen as analyze_affine_uni does (src/inter.c:1607-1647)  */
#define ORC_AFFME_SUB8      4   /* affine_subblk_size_idx > 0: 8x8 sub-blocks in uni calls                */

typedef struct {
    s16 x, y;           /* CU position (luma samples), CU inside the picture                        */
    u8  w, h;           /* 16..64, powers of two                                                    */
    u8  ref_slot;       /* integer plane planes[ref_slot * 16] of pi->ref_pic                       */
    s8  refi;           /* reference index (reference bits), < num_refp                            */
    u8  num_refp;       /* pi->num_refp                                                             */
    u8  mvr;            /* pi->curr_mvr 0..2: CPMV step 1/4, 1, 1/16 sample (Tab_Affine_AMVR)       */
    u8  flags;          /* ORC_AFFME_*                                                              */
    u8  other_slot;     /* bi: integer plane of the other list's reference                          */
    u32 lambda_mv;      /* pi->lambda_mv                                                            */
    s32 mot_bits_other; /* bi: pi->mot_bits of the other list                                       */
    s32 pad;
    s32 mvp[2][2];      /* affine MVP of the two control points, 1/16 samples                      */
    s32 mv[2][2];       /* start CPMVs; with ORC_AFFME_UNI_START mv[0] is pi->best_mv_uni (1/4)     */
    s32 other_mv[2][2]; /* bi: the other list's CPMVs                                               */
} orc_affme_req_t;

typedef struct {
    s32 mv[2][2];       /* the CPMVs the call leaves in mv                                          */
    u32 satd;           /* affine_me_gradient's return value (com_had of the best, >> bi)          */
    s32 bits;           /* affine_mv_bits of the result (+ mot_bits_other for bi)                   */
    u64 cost;           /* satd + MV_COST(bits); UINT64_MAX for a request outside the domain        */
} orc_affme_out_t;

/* planes[slot * 16]: integer luma planes padded by >= 144 (stride i_ref); OpenMP over requests
 * when threads > 1 */
void orc_me_affine(int width, int height, const pel *org, int i_org, const pel *const *planes, int i_ref,
                   const orc_affme_req_t *reqs, int n, orc_affme_out_t *out, int threads);

/* one CU's affine MVP request (com_get_affine_mvp_scaling, src/com_util.c:1983-2058); the
 * motion field has the reference's layout: stride i_scu = pic_width_in_scu + 2, SCU (0, 0) at
 * index i_scu + 1 (one border row above, one border column on each side) */
typedef struct {
    s32 scup;           /* y_scu * i_scu + x_scu of the CU's top-left SCU                         */
    s16 cu_width;       /* luma samples                                                            */
    s8 lidx;            /* list 0 / 1                                                              */
    s8 cur_refi;        /* the CU's reference index in list lidx                                   */
    s8 mvr;             /* affine AMVR index (Tab_Affine_AMVR: 0 -> 2, 1 -> 4, 2 -> 0 bits)         */
    s8 pad[3];
} orc_affmvp_req_t;

typedef struct {
    s32 mvp[2][2];      /* (x, y) of the top-left and top-right control points, 1/16 samples       */
} orc_affmvp_out_t;

/* map_mv: s16 [rows * i_scu][2 lists][2]; map_refi: s8 [rows * i_scu][2]; ref_ptr: [n_ref][2]
 * (the POC of refp[i][lidx]).  Returns the number of requests outside the domain (a neighbour
 * outside the field, a reference index >= n_ref, a zero POC distance, mvr > 2); their output is
 * zero. */
int orc_affine_mvp(s64 ptr, const s64 *ref_ptr, int n_ref, const s16 *map_mv, const s8 *map_refi, int i_scu,
                   int rows, const orc_affmvp_req_t *reqs, int n, orc_affmvp_out_t *out);

/* Affine merge candidates (com_get_affine_merge_candidate, src/com_util.c:1761-1981, with
 * com_derive_affine_model_mv :1566-1654, com_derive_affine_constructed_candidate :1656-1758,
 * get_colocal_scup :303, get_col_mv / get_col_mv_from_list0 :977-1000, scaling_mv1 :322).  The
 * picture's maps have the reference's layout (stride i_scu = pic_width_in_scu + 2, SCU (0, 0) at
 * index i_scu + 1): map_mv s16 [rows * i_scu][2][2], map_refi s8 [rows * i_scu][2], map_scu u8
 * (com_scu_t: bit 0 coded, bit 1 intra, bits 4-5 affine), map_pos u32 (top-left SCU << 6 |
 * log2 h << 3 | log2 w of the CU covering the SCU); col_mv / col_refi are the colocated picture's
 * maps in the same layout (refp[0][REFP_1] in B slices, refp[0][REFP_0] otherwise). */
typedef struct {
    s64 ptr;                 /* POC of the current picture                                        */
    s64 ref0_ptr[2];         /* POC of refp[0][REFP_0] and refp[0][REFP_1]                         */
    s64 col_list_ptr[17];    /* the colocated picture's list_ptr (POC of its list-0 references)    */
    s32 i_scu, pic_width_in_scu, pic_height_in_scu, rows;
    s32 slice_type;          /* 3 = SLICE_B, else the P rule                                      */
    s32 log2_max_cuwh;
} orc_affmrg_pic_t;

typedef struct {
    s32 scup;                /* y_scu * i_scu + x_scu of the CU's top-left SCU                     */
    s16 cu_width, cu_height; /* luma samples, powers of two 16..128                                */
} orc_affmrg_req_t;

typedef struct {
    s32 num;                 /* candidates derived (the list is zero-padded to 5)                  */
    s8 cp_num[5];            /* control points of each candidate (2 or 3)                          */
    s8 refi[5][2];           /* reference index per list, -1 unused                                */
    s8 pad;
    s32 cpmv[5][2][3][2];    /* control-point MVs (1/16 samples); vertices past cp_num are 0       */
} orc_affmrg_out_t;

/* Returns the number of requests outside the domain (a map read outside the field, sizes not
 * powers of two in 16..128, a colocated reference index outside col_list_ptr, a zero POC
 * distance); their output is zero. */
int orc_affine_merge(const orc_affmrg_pic_t *pic, const s16 *map_mv, const s8 *map_refi, const u8 *map_scu,
                     const u32 *map_pos, const s16 *col_mv, const s8 *col_refi, const orc_affmrg_req_t *reqs, int n,
                     orc_affmrg_out_t *out);

/* the picture-level results from the records (src/lookahead.c:255-292): returns the picture
 * SATD cost; icost, icost_uv[2], map_dqp[units] are filled when non-NULL */
double orc_loka_finish(const orc_loka_cfg_t *cfg, const orc_loka_unit_t *units, double *icost, double *icost_uv,
                       float *map_dqp);

#ifdef __cplusplus
}
#endif
#endif
