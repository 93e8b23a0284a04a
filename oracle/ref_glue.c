/*
 * ref_glue.c -- test-side glue compiled together with the reference encoder's own C
 * sources (oracle/Makefile, target "ref").  TEST INFRASTRUCTURE ONLY: nothing in the
 * product library links or loads this.
 *
 * It does two things:
 *   1. supplies empty x86 SIMD initialisers, so uavs3e_create() (src/uavs3e.c:1332-1339)
 *      keeps the plain-C kernel table that uavs3e_funs_init_c() installs
 *      (src/com_util.c:3131); the C table and the SIMD table encode identical bitstreams;
 *   2. exports flat "refk_*" wrappers that call the reference's kernel-table entries
 *      (funs_handle_t, inc/com_util.h:278-341) and exported helpers with plain pointers,
 *      so the Python golden-vector generator and the CPU parity tests can call them
 *      through ctypes.
 */
#include "define.h"
#include "util.h"
#include <stddef.h>
#include <math.h>
#include "../include/uavs3e_cuda_table.h"

/* ---- 0. the GPU library's table twin must have funs_handle_t's layout, member by member ---- */
#define SAME_OFFSET(m) _Static_assert(offsetof(funs_handle_t, m) == offsetof(uavs3e_cuda_funs_t, m), #m)
SAME_OFFSET(intra_pred_dc); SAME_OFFSET(intra_pred_plane); SAME_OFFSET(intra_pred_bi);
SAME_OFFSET(intra_pred_plane_ipf); SAME_OFFSET(intra_pred_bi_ipf); SAME_OFFSET(intra_pred_ver);
SAME_OFFSET(intra_pred_hor); SAME_OFFSET(intra_pred_ang); SAME_OFFSET(intra_pred_ipf_core);
SAME_OFFSET(intra_pred_ipf_core_s16); SAME_OFFSET(deblock_luma); SAME_OFFSET(deblock_chroma); SAME_OFFSET(sao);
SAME_OFFSET(sao_stat); SAME_OFFSET(alf); SAME_OFFSET(alf_fix); SAME_OFFSET(alf_calc); SAME_OFFSET(ipcpy);
SAME_OFFSET(ipflt); SAME_OFFSET(ipflt_ext); SAME_OFFSET(ip_flt_y_hor); SAME_OFFSET(ip_flt_y_ver);
SAME_OFFSET(ip_flt_y_ver_ext); SAME_OFFSET(recon); SAME_OFFSET(dquant); SAME_OFFSET(itrans_dct2);
SAME_OFFSET(itrans_dct8_dst7); SAME_OFFSET(trans_dct2); SAME_OFFSET(trans_dct8_dst7); SAME_OFFSET(cost_sad);
SAME_OFFSET(cost_sad_x3); SAME_OFFSET(cost_sad_x4); SAME_OFFSET(cost_ssd); SAME_OFFSET(cost_satd);
SAME_OFFSET(cost_var); SAME_OFFSET(ssim_4x4x2_core); SAME_OFFSET(ssim_end4); SAME_OFFSET(pel_diff);
SAME_OFFSET(pel_avrg); SAME_OFFSET(affine_sobel_flt_hor); SAME_OFFSET(affine_sobel_flt_ver);
SAME_OFFSET(affine_coef_computer); SAME_OFFSET(quant_rdoq); SAME_OFFSET(quant_check); SAME_OFFSET(sobel_cost);
_Static_assert(sizeof(funs_handle_t) == sizeof(uavs3e_cuda_funs_t), "table size");
size_t refk_table_size(void) { return sizeof(funs_handle_t); }

/* ---- 1. SIMD initialisers left empty (their real bodies live in src/sse, src/avx2) ---- */
void uavs3e_funs_init_sse(void) {}
void uavs3e_funs_init_avx2(void) {}
int  uavs3e_simd_avx_level(int *phwavx) { if (phwavx) *phwavx = 0; return 0; }

/* ---- 2. flat wrappers ---------------------------------------------------------------- */
static int g_inited = 0;

void refk_init(void)
{
    if (g_inited) return;
    uavs3e_funs_init_c();           /* src/com_util.c:3131 */
    com_scan_tbl_init();            /* src/com_util.c:1254 */
    com_dct_coef_create();          /* src/com_tables.c:222 */
    rdoq_init_err_scale(8);         /* src/quant.c:69 */
    rdoq_init_prob_2_bits();        /* src/quant.c:85 */
    g_inited = 1;
}

#define H (&uavs3e_funs_handle)

u32  refk_sad(int widx, pel *o, int io, pel *p, int ip, int h) { return H->cost_sad[widx](o, io, p, ip, h); }
void refk_sad_x3(int widx, pel *o, int io, pel *p0, pel *p1, pel *p2, int ip, u32 *s, int h) { H->cost_sad_x3[widx](o, io, p0, p1, p2, ip, s, h); }
void refk_sad_x4(int widx, pel *o, int io, pel *p0, pel *p1, pel *p2, pel *p3, int ip, u32 *s, int h) { H->cost_sad_x4[widx](o, io, p0, p1, p2, p3, ip, s, h); }
u64  refk_ssd(int widx, pel *o, int io, pel *p, int ip, int h) { return H->cost_ssd[widx](o, io, p, ip, h); }
u32  refk_satd(int wi, int hi, pel *o, int io, pel *p, int ip) { return H->cost_satd[wi][hi](o, io, p, ip); }
u32  refk_had(int w, int h, pel *o, int io, pel *p, int ip, int bd) { return com_had(w, h, o, io, p, ip, bd); }
u32  refk_satd_intra(int w, int h, pel *o, pel *p, int io, int ip, int bd) { return calc_satd_intra(w, h, o, p, io, ip, bd); }

void refk_ipcpy(int widx, const pel *s, int is, pel *d, int id, int w, int h) { H->ipcpy[widx](s, is, d, id, w, h); }
void refk_ipflt(int t, int widx, const pel *s, int is, pel *d, int id, int w, int h, const s8 *c, int mx) { H->ipflt[t][widx](s, is, d, id, w, h, c, mx); }
void refk_ipflt_ext(int t, int widx, const pel *s, int is, pel *d, int id, int w, int h, const s8 *cx, const s8 *cy, int mx) { H->ipflt_ext[t][widx](s, is, d, id, w, h, cx, cy, mx); }

/* com_if_luma_frame (src/com_mc.c:760) on caller buffers: plane0 is the padded integer
 * plane, planes[15] the 15 fractional planes in [dy*4+dx-1] order, all width x height
 * with the same pad and stride (pels). */
void refk_if_luma_frame(pel *plane0, pel **planes, int width, int height, int pad, int stride)
{
    com_img_t imgs[16];
    com_img_t *list[4][4];
    s16 *tmp[3];
    int tmp_stride = width + 16;
    for (int i = 0; i < 16; i++) {
        memset(&imgs[i], 0, sizeof(com_img_t));
        imgs[i].num_planes = 1;
        imgs[i].width[0] = width;
        imgs[i].height[0] = height;
        imgs[i].stride[0] = stride * (int)sizeof(pel);
        imgs[i].pad[0] = pad;
        imgs[i].planes[0] = i == 0 ? plane0 : planes[i - 1];
        list[i >> 2][i & 3] = &imgs[i];
    }
    for (int i = 0; i < 3; i++) tmp[i] = (s16 *)malloc(sizeof(s16) * (size_t)tmp_stride * (height + 16));
    com_if_luma_frame(list, tmp, 8);
    for (int i = 0; i < 3; i++) free(tmp[i]);
}

void refk_pel_diff(int widx, pel *o, int io, pel *p, int ip, s16 *r, int ir, int h) { H->pel_diff[widx](o, io, p, ip, r, ir, h); }
void refk_pel_avrg(int widx, pel *d, int id, pel *s1, pel *s2, int h) { H->pel_avrg[widx](d, id, s1, s2, h); }
void refk_recon(int widx, s16 *resi, pel *pred, int ipred, int w, int h, pel *rec, int irec, int cbf, int bd) { H->recon[widx](resi, pred, ipred, w, h, rec, irec, cbf, bd); }

/* com_intra_get_nbr (src/com_ipred.c:40) with a plain byte map of "coded" flags of the
 * i_scu-wide SCU grid; scup indexes that grid.  nb_out receives INTRA_NEIB_SIZE pels. */
void refk_intra_get_nbr(int x, int y, int w, int h, pel *src, int s_src, pel *top, int lcu_size, int avail,
                        pel *nb_out, int scup, const u8 *coded, int n_scu, int i_scu, int bd)
{
    static pel nb[N_C][INTRA_NEIB_SIZE];
    com_scu_t *map = (com_scu_t *)calloc((size_t)n_scu, sizeof(com_scu_t));
    for (int i = 0; i < n_scu; i++) map[i].coded = coded[i] ? 1 : 0;
    memset(nb, 0, sizeof(nb));
    com_intra_get_nbr(x, y, w, h, src, s_src, top, lcu_size, (u16)avail, nb, scup, map, i_scu, bd, Y_C);
    memcpy(nb_out, nb[Y_C], sizeof(pel) * INTRA_NEIB_SIZE);
    free(map);
}

/* com_intra_pred (src/com_ipred.c:733); nb points at a full INTRA_NEIB_SIZE array */
void refk_intra_pred(pel *nb, pel *dst, int ipm, int w, int h, int bd, int avail, int ipf)
{
    com_intra_pred(nb + INTRA_NEIB_MID, dst, ipm, w, h, bd, (u16)avail, (u8)ipf);
}

/* one angular table entry called directly: lets the tests compare the specialised
 * entries (e.g. intra_pred_ang[4]) with the generic ones called for the same mode */
void refk_intra_ang_entry(int entry, pel *nb, pel *dst, int i_dst, int mode, int w, int h)
{
    H->intra_pred_ang[entry](nb + INTRA_NEIB_MID, dst, i_dst, mode, w, h);
}

void refk_trans_dct2(int log2w, int log2h, s16 *src, s16 *dst, int bd) { H->trans_dct2[log2w - 1][log2h - 1](src, dst, bd); }
void refk_trans_dct8_dst7(int t, int log2n, s16 *src, s16 *dst, int shift, int line) { H->trans_dct8_dst7[t][log2n - 1](src, dst, shift, line); }
void refk_itrans_dct2(int log2h, int log2w, s16 *coef, s16 *resi, int bd) { H->itrans_dct2[log2h - 1][log2w - 1](coef, resi, bd); }
void refk_itrans_dct8_dst7(int t, int log2n, s16 *coef, s16 *blk, int shift, int line, int mx, int mn) { H->itrans_dct8_dst7[t][log2n - 1](coef, blk, shift, line, mx, mn); }
void refk_dquant(int flat, s16 *coef, s16 *out, u8 *wq4, u8 *wq8, int log2w, int log2h, int scale, int shift, int bd)
{
    u8 *wq[2] = { wq4, wq8 };
    H->dquant[flat ? 1 : 0](coef, out, wq, log2w, log2h, scale, shift, bd);
}
int refk_quant_check(s16 *coef, int num, int thr) { return H->quant_check(coef, num, thr); }
int refk_quant_rdoq(s16 *coef, int num, int qv, int qb, int es, int pb, u32 *abs_coef, s16 *abs_level, s64 *err)
{
    return H->quant_rdoq(coef, num, qv, qb, es, pb, abs_coef, abs_level, err);
}

/* transform() (src/transform.c:772) and com_invqt() (src/com_itdq.c:873) for a luma TB */
void refk_transform(int tb_nxn, int blk_idx, s16 *coef, s16 *resi, int log2w, int log2h, int bd, int sec, int alt4)
{
    static com_mode_t mode;
    mode.tb_part = tb_nxn ? SIZE_NxN : SIZE_2Nx2N;
    transform(&mode, Y_C, blk_idx, coef, resi, log2w, log2h, bd, sec, alt4);
}
void refk_invqt(int tb_nxn, int blk_idx, s16 *coef, s16 *resi, u8 *wq4, u8 *wq8, int log2w, int log2h, int qp, int bd, int sec, int alt4)
{
    static com_mode_t mode;
    u8 *wq[2] = { wq4, wq8 };
    mode.tb_part = tb_nxn ? SIZE_NxN : SIZE_2Nx2N;
    com_invqt(&mode, Y_C, blk_idx, coef, resi, wq, log2w, log2h, qp, bd, sec, alt4);
}

const u16 *refk_scan(int log2w, int log2h) { return com_tbl_scan[log2w - 1][log2h - 1]; }
const s8 *refk_dct_table(int log2n)
{
    switch (log2n) {
    case 1: return &com_tbl_tm2[0][0][0];
    case 2: return &com_tbl_tm4[0][0][0];
    case 3: return &com_tbl_tm8[0][0][0];
    case 4: return &com_tbl_tm16[0][0][0];
    case 5: return &com_tbl_tm32[0][0][0];
    default: return &com_tbl_tm64[0][0][0];
    }
}
double refk_tbl_sqrt(int i) { return com_tbl_sqrt[i]; }

#undef H   /* the table shorthand of section 2 */

/* ---- 3. lookahead cost estimation -------------------------------------------------------
 * loka_estimate_coding_cost (src/lookahead.c:82) on caller planes.  The search context is set
 * up as inter_search_create/inter_search_init do (src/inter.c:2015-2057) for a picture of
 * W x H, with the low-delay search range when max_search_range is 64. */
static void loka_setup(com_info_t *info, inter_search_t *pi, int W, int H, int is_padding, int max_search_range,
                       int gop_size)
{
    memset(info, 0, sizeof(*info));
    info->pic_width = W;
    info->pic_height = H;
    info->bit_depth_internal = 8;
    info->gop_size = gop_size;
    info->sqh.low_delay = max_search_range == SEARCH_RANGE_IPEL_LD;
    inter_search_create(&info->tab_mvbits, info);
    memset(pi, 0, sizeof(*pi));
    inter_search_init(pi, info, is_padding);
}

static void loka_img(com_img_t *img, int W, int H, long long ptr, pel *y, int iy, pel *u, pel *v, int ic)
{
    memset(img, 0, sizeof(*img));
    img->num_planes = u ? 3 : 1;
    img->ptr = ptr;
    img->width[0] = W; img->height[0] = H; img->stride[0] = iy * (int)sizeof(pel); img->planes[0] = y;
    for (int i = 1; i < 3 && u; i++) {
        img->width[i] = W / 2; img->height[i] = H / 2; img->stride[i] = ic * (int)sizeof(pel);
        img->planes[i] = i == 1 ? u : v;
    }
}

double refk_loka_estimate(int W, int H, int is_padding, int max_search_range, int gop_size, long long ptr,
                          pel *org_y, int i_org, pel *org_u, pel *org_v, int i_org_c,
                          int n0, pel **ref0, long long *ptr0, int n1, pel **ref1, long long *ptr1, int i_ref,
                          double *icost, double *icost_uv, float *map_dqp)
{
    refk_init();
    static com_info_t info;
    inter_search_t *pi = (inter_search_t *)calloc(1, sizeof(inter_search_t));
    loka_setup(&info, pi, W, H, is_padding, max_search_range, gop_size);
    com_img_t org, r0[4], r1[4];
    com_img_t *l0[4], *l1[4];
    loka_img(&org, W, H, ptr, org_y, i_org, org_u, org_v, i_org_c);
    for (int i = 0; i < n0; i++) { loka_img(&r0[i], W, H, ptr0[i], ref0[i], i_ref, NULL, NULL, 0); l0[i] = &r0[i]; }
    for (int i = 0; i < n1; i++) { loka_img(&r1[i], W, H, ptr1[i], ref1[i], i_ref, NULL, NULL, 0); l1[i] = &r1[i]; }
    int num_ref[2] = { n0, n1 };
    double cost = loka_estimate_coding_cost(pi, &org, l0, l1, num_ref, 8, icost, icost_uv, map_dqp);
    inter_search_free(info.tab_mvbits, pi->tab_mvbits_offset);
    free(pi);
    return cost;
}

/* me_search_tz (src/me.c:529) for the 16x16 unit at (x, y) with the lookahead's settings
 * (src/lookahead.c:104-111): integer resolution, predictor (0,0), no bi-prediction.
 * Writes the integer MV; returns the search's cost. */
unsigned long long refk_loka_search(int W, int H, int is_padding, int max_search_range, int gop_size, long long ptr,
                                    pel *org_y, int i_org, pel *ref, int i_ref, long long ref_ptr, int refi, int num_refp,
                                    int x, int y, short *mv_out)
{
    refk_init();
    static com_info_t info;
    inter_search_t *pi = (inter_search_t *)calloc(1, sizeof(inter_search_t));
    loka_setup(&info, pi, W, H, is_padding, max_search_range, gop_size);
    com_img_t rimg;
    loka_img(&rimg, W, H, ref_ptr, ref, i_ref, NULL, NULL, 0);
    com_pic_t pic;
    com_subpel_t subpel;
    memset(&pic, 0, sizeof(pic));
    memset(&subpel, 0, sizeof(subpel));
    pic.subpel = &subpel;
    pic.ptr = ref_ptr;
    pic.img = &rimg;
    pic.stride_luma = i_ref;
    pic.y = ref;
    subpel.imgs[0][0] = &rimg;
    double base_lambda = 1.43631 * pow(2.0, (32 - 16.0) / 4.0);
    pi->ptr = ptr;
    pi->curr_mvr = 2;
    pi->lambda_mv = (u32)floor(65536.0 * sqrt(base_lambda));
    pi->i_org = i_org;
    pi->adaptive_raster_range = 0;
    pi->subpel_cost_type = 0;
    pi->org = org_y + y * i_org + x;
    pi->num_refp = (u8)num_refp;
    pi->ref_pic = &pic;
    s16 mv[2], mvp[2] = { 0, 0 };
    u64 cost = me_search_tz(pi, x, y, 16, 16, W, H, (s8)refi, 0, mvp, mv, 0);
    mv_out[0] = (short)(mv[0] >> 2);
    mv_out[1] = (short)(mv[1] >> 2);
    inter_search_free(info.tab_mvbits, pi->tab_mvbits_offset);
    free(pi);
    return cost;
}

/* ---- 4. per-call TZ motion search ---------------------------------------------------------
 * me_search_tz (src/me.c:529) for one request on caller planes: planes[slot * 16 + phase] are the
 * quarter-sample planes of each reference (0 = integer plane; stride i_ref; padded).  The
 * inter_search_t is set up as inter_search_init does, with the request's state; a bi request's
 * org is 2 org - (the other list's prediction by com_mc_blk_luma), clipped, as create_bi_org
 * (src/inter.c:55) forms it.  Layout of req/out: orc_tz_req_t / orc_tz_out_t (oracle.h). */
typedef struct {
    s16 x, y; u8 w, h; u8 ref_slot; s8 refi; u8 num_refp; u8 mvr; u8 bi; u8 flags;
    s16 mvp[2]; s16 mv[2]; s16 mv_ipel[2]; s16 other_mv[2]; u8 other_slot; u8 pad0[3];
    s32 mot_bits_other; u32 lambda_mv; s32 dist; s32 pad1;
} glue_tz_req_t;
typedef struct { s16 mv[2]; s16 mv_ipel[2]; u64 cost; } glue_tz_out_t;

static void tz_pic(com_pic_t *pic, com_subpel_t *sp, com_img_t imgs[16], pel **planes, int slot, int W, int H,
                   int i_ref, long long ptr)
{
    memset(pic, 0, sizeof(*pic));
    memset(sp, 0, sizeof(*sp));
    for (int i = 0; i < 16; i++) {
        loka_img(&imgs[i], W, H, ptr, planes[slot * 16 + i], i_ref, NULL, NULL, 0);
        sp->imgs[i >> 2][i & 3] = &imgs[i];
    }
    pic->subpel = sp;
    pic->ptr = ptr;
    pic->img = &imgs[0];
    pic->stride_luma = i_ref;
    pic->y = planes[slot * 16];
    pic->width_luma = W;
    pic->height_luma = H;
}

void refk_me_tz(int W, int H, int is_padding, int max_search_range, int gop_size, pel *org, int i_org,
                pel **planes, int i_ref, const glue_tz_req_t *rq, glue_tz_out_t *out)
{
    refk_init();
    static com_info_t info;
    inter_search_t *pi = (inter_search_t *)calloc(1, sizeof(inter_search_t));
    loka_setup(&info, pi, W, H, is_padding, max_search_range, gop_size);
    static com_pic_t pic, pic_o;
    static com_subpel_t sp, sp_o;
    static com_img_t imgs[16], imgs_o[16];
    tz_pic(&pic, &sp, imgs, planes, rq->ref_slot, W, H, i_ref, 0);
    ALIGNED_32(pel org_bi[MAX_CU_DIM]);
    const int x = rq->x, y = rq->y, w = rq->w, h = rq->h;
    pi->ptr = rq->dist;
    pi->curr_mvr = rq->mvr;
    pi->lambda_mv = rq->lambda_mv;
    pi->num_refp = rq->num_refp;
    pi->subpel_cost_type = rq->flags & 1;
    pi->adaptive_raster_range = (rq->flags >> 1) & 1;
    pi->mv_ipel[REFP_0][rq->refi][0] = rq->mv_ipel[0];
    pi->mv_ipel[REFP_0][rq->refi][1] = rq->mv_ipel[1];
    pi->mot_bits[REFP_1] = rq->mot_bits_other;
    pi->ref_pic = &pic;
    if (rq->bi) {
        ALIGNED_32(pel pred[MAX_CU_DIM]);
        tz_pic(&pic_o, &sp_o, imgs_o, planes, rq->other_slot, W, H, i_ref, 0);
        com_mc_blk_luma(&pic_o, pred, w, (x << 2) + rq->other_mv[0], (y << 2) + rq->other_mv[1], w, h,
                        CONV_LOG2(w) - MIN_CU_LOG2, pi->max_coord[MV_X], pi->max_coord[MV_Y], 255, 0);
        const pel *o = org + y * i_org + x;
        for (int j = 0; j < h; j++)
            for (int i = 0; i < w; i++) org_bi[j * w + i] = (pel)COM_CLIP3(0, 255, (o[j * i_org + i] << 1) - pred[j * w + i]);
        pi->org = org_bi;
        pi->i_org = w;
    } else {
        pi->org = org + y * i_org + x;
        pi->i_org = i_org;
    }
    s16 mvp[2] = { rq->mvp[0], rq->mvp[1] };
    s16 mv[2] = { rq->mv[0], rq->mv[1] };
    out->cost = me_search_tz(pi, x, y, w, h, W, H, rq->refi, REFP_0, mvp, mv, rq->bi);
    out->mv[0] = mv[0];
    out->mv[1] = mv[1];
    out->mv_ipel[0] = rq->bi ? rq->mv_ipel[0] : pi->mv_ipel[REFP_0][rq->refi][0];
    out->mv_ipel[1] = rq->bi ? rq->mv_ipel[1] : pi->mv_ipel[REFP_0][rq->refi][1];
    inter_search_free(info.tab_mvbits, pi->tab_mvbits_offset);
    free(pi);
}

/* ---- 5. CU motion compensation -------------------------------------------------------------
 * com_mc_cu (src/com_mc.c:140) for one request: planes[slot * 16 + phase] are each reference's
 * quarter-sample luma planes (stride i_ref), chroma[slot * 2 + (0 U, 1 V)] its chroma planes
 * (stride i_c); reference index = slot in both lists, POC = slot.  Layout of req:
 * orc_mc_req_t (oracle.h); the prediction goes to out as Y (w x h) then U, V (w/2 x h/2) for
 * the channels asked. */
typedef struct {
    s16 x, y; u8 w, h; s8 slot[2]; s16 mv[2][2]; u8 channel; u8 pad[3]; u32 out_offset;
} glue_mc_req_t;

void refk_mc_cu(int W, int H, pel **planes, int n_slots, int i_ref, pel **chroma, int i_c, const glue_mc_req_t *rq,
                pel *out)
{
    refk_init();
    static com_pic_t pics[8];
    static com_subpel_t sps[8];
    static com_img_t imgs[8][16];
    static com_ref_pic_t refp[8][REFP_NUM];
    static pel pred[N_C][MAX_CU_DIM];
    for (int s = 0; s < n_slots && s < 8; s++) {
        tz_pic(&pics[s], &sps[s], imgs[s], planes, s, W, H, i_ref, s);
        pics[s].u = chroma[s * 2];
        pics[s].v = chroma[s * 2 + 1];
        pics[s].stride_chroma = i_c;
        for (int l = 0; l < REFP_NUM; l++) { refp[s][l].pic = &pics[s]; refp[s][l].ptr = s; }
    }
    s8 refi[REFP_NUM] = { rq->slot[0], rq->slot[1] };
    s16 mv[REFP_NUM][MV_D] = { { rq->mv[0][0], rq->mv[0][1] }, { rq->mv[1][0], rq->mv[1][1] } };
    com_mc_cu(rq->x, rq->y, W, H, rq->w, rq->h, refi, mv, refp, pred, rq->w, (channel_type_t)rq->channel, 8);
    pel *o = out + rq->out_offset;
    const int w = rq->w, h = rq->h;
    if (rq->channel != CHANNEL_C) { memcpy(o, pred[Y_C], (size_t)w * h); o += w * h; }
    if (rq->channel != CHANNEL_L) {
        memcpy(o, pred[U_C], (size_t)w * h / 4);
        memcpy(o + w * h / 4, pred[V_C], (size_t)w * h / 4);
    }
}

/* ---- 6. affine CU motion compensation --------------------------------------------------------
 * com_mc_cu_affine (src/com_mc.c:361) for one request (layout orc_affine_req_t, oracle.h);
 * planes / chroma as in section 5.  The prediction goes to out as Y, then U, V. */
typedef struct {
    s16 x, y; u8 w, h; s8 slot[2]; u8 cp_num; u8 sub8; u8 pad[2]; s32 cpmv[2][3][2]; u32 out_offset;
} glue_affine_req_t;

void refk_mc_affine(int W, int H, pel **planes, int n_slots, int i_ref, pel **chroma, int i_c,
                    const glue_affine_req_t *rq, pel *out)
{
    refk_init();
    static com_pic_t pics[8];
    static com_subpel_t sps[8];
    static com_img_t imgs[8][16];
    static com_ref_pic_t refp[8][REFP_NUM];
    static pel pred[N_C][MAX_CU_DIM];
    static com_pic_header_t sh;
    for (int s = 0; s < n_slots && s < 8; s++) {
        tz_pic(&pics[s], &sps[s], imgs[s], planes, s, W, H, i_ref, s);
        pics[s].u = chroma[s * 2];
        pics[s].v = chroma[s * 2 + 1];
        pics[s].stride_chroma = i_c;
        for (int l = 0; l < REFP_NUM; l++) { refp[s][l].pic = &pics[s]; refp[s][l].ptr = s; }
    }
    sh.affine_subblk_size_idx = rq->sub8;
    s8 refi[REFP_NUM] = { rq->slot[0], rq->slot[1] };
    CPMV mv[REFP_NUM][VER_NUM][MV_D];
    memset(mv, 0, sizeof(mv));
    for (int l = 0; l < 2; l++)
        for (int v = 0; v < 3; v++) { mv[l][v][0] = rq->cpmv[l][v][0]; mv[l][v][1] = rq->cpmv[l][v][1]; }
    com_mc_cu_affine(rq->x, rq->y, W, H, rq->w, rq->h, refi, mv, refp, pred, rq->cp_num, &sh, 8);
    pel *o = out + rq->out_offset;
    const int n = rq->w * rq->h;
    memcpy(o, pred[Y_C], (size_t)n);
    memcpy(o + n, pred[U_C], (size_t)n / 4);
    memcpy(o + n + n / 4, pred[V_C], (size_t)n / 4);
}

/* ---- 7. RDOQ of a transform block ------------------------------------------------------------
 * quant_non_zero (src/quant.c:315) with flat quantisation, on a core_t whose bin-cost estimates
 * (rdoq_bin_est_*) are the request's; layouts orc_rdoq_req_t / orc_rdoq_est_t (oracle.h).  The
 * request's integer lambda L is passed as the double L / 2^15, which rdoq_quant_block turns back
 * into L exactly. */
typedef struct {
    s32 ctp[2]; s32 cbf[3][2]; s32 run[24][2]; s32 lvl[24][2]; s32 lst[2][6][12][2];
} glue_rdoq_est_t;
typedef struct {
    u32 coef_offset; u8 log2w, log2h; u8 qp, is_intra, ch_type, slice_type; u16 est; u32 pad; s64 lambda;
} glue_rdoq_req_t;

int refk_rdoq(const glue_rdoq_req_t *rq, const glue_rdoq_est_t *E, s16 *coef)
{
    refk_init();
    static core_t *core = NULL;
    static com_info_t info;
    static com_pic_header_t pichdr;
    if (!core) core = (core_t *)calloc(1, sizeof(core_t));
    memset(&info, 0, sizeof(info));
    memset(&pichdr, 0, sizeof(pichdr));
    info.bit_depth_internal = 8;
    pichdr.pic_wq_enable = 0;
    core->info = &info;
    core->pichdr = &pichdr;
    memcpy(core->rdoq_bin_est_ctp, E->ctp, sizeof(E->ctp));
    memcpy(core->rdoq_bin_est_cbf, E->cbf, sizeof(E->cbf));
    memcpy(core->rdoq_bin_est_run, E->run, sizeof(E->run));
    memcpy(core->rdoq_bin_est_lvl, E->lvl, sizeof(E->lvl));
    memcpy(core->rdoq_bin_est_lst, E->lst, sizeof(E->lst));
    return quant_non_zero(core, rq->qp, (double)rq->lambda / 32768.0, rq->is_intra, coef + rq->coef_offset,
                          rq->log2w, rq->log2h, rq->ch_type, rq->slice_type);
}

/* rdoq_init_cu_est_bits (src/quant.c:139) from raw context models, for realistic estimate sets:
 * ctx holds ctp_zero_flag, cbf[3], run_rdoq[24], level[24], last1[12], last2[22] (u16 models) */
void refk_rdoq_est_from_ctx(const u16 *ctx, glue_rdoq_est_t *E)
{
    refk_init();
    static core_t *core = NULL;
    static lbac_t lbac;
    if (!core) core = (core_t *)calloc(1, sizeof(core_t));
    memset(&lbac, 0, sizeof(lbac));
    int k = 0;
    lbac.h.ctp_zero_flag[0] = ctx[k++];
    for (int i = 0; i < LBAC_CTX_CBF; i++) lbac.h.cbf[i] = ctx[k++];
    for (int i = 0; i < LBAC_CTX_RUN_RDOQ; i++) lbac.h.run_rdoq[i] = ctx[k++];
    for (int i = 0; i < LBAC_CTX_LEVEL; i++) lbac.h.level[i] = ctx[k++];
    for (int i = 0; i < LBAC_CTX_LAST1 * 2; i++) lbac.h.last1[i] = ctx[k++];
    for (int i = 0; i < LBAC_CTX_LAST2 * 2 - 2; i++) lbac.h.last2[i] = ctx[k++];
    rdoq_init_cu_est_bits(core, &lbac);
    memcpy(E->ctp, core->rdoq_bin_est_ctp, sizeof(E->ctp));
    memcpy(E->cbf, core->rdoq_bin_est_cbf, sizeof(E->cbf));
    memcpy(E->run, core->rdoq_bin_est_run, sizeof(E->run));
    memcpy(E->lvl, core->rdoq_bin_est_lvl, sizeof(E->lvl));
    memcpy(E->lst, core->rdoq_bin_est_lst, sizeof(E->lst));
}

/* ---- 8. coefficient rate ------------------------------------------------------------------
 * lbac_enc_run_length_cc_rdo (src/entropy.c:1688) for one block: a reset coder (lbac_reset,
 * every context at PROB_INIT) takes the request's range and its channel's context models, codes
 * the block's levels, and the bits it counted, its range and those models come back.  Layout of
 * req / out: orc_coef_rate_req_t / orc_coef_rate_out_t (oracle.h). */
typedef struct { s16 run[12], run_rdoq[12], level[12], last1[6], last2[12]; } glue_coef_ctx_t;
typedef struct { u32 coef_offset; u8 log2w, log2h, ch_type, pad; u16 num_sig, range; glue_coef_ctx_t ctx; } glue_coef_rate_req_t;
typedef struct { u32 bits; u16 range, pad; glue_coef_ctx_t ctx; } glue_coef_rate_out_t;

void lbac_enc_run_length_cc_rdo(lbac_t *lbac, s16 *coef, int log2_w, int log2_h, int num_sig, int ch_type);
void lbac_encode_bin_for_rdoq(u32 bin, lbac_ctx_model_t *model);

void refk_coef_rate(s16 *levels, const glue_coef_rate_req_t *rq, glue_coef_rate_out_t *out)
{
    refk_init();
    static lbac_t lb;
    memset(&lb, 0, sizeof(lb));
    lbac_ctx_init(&lb.h);
    lbac_reset(&lb);
    lb.range = rq->range;
    const int c = rq->ch_type ? 1 : 0;
    for (int i = 0; i < 12; i++) {
        lb.h.run[c * 12 + i] = rq->ctx.run[i];
        lb.h.run_rdoq[c * 12 + i] = rq->ctx.run_rdoq[i];
        lb.h.level[c * 12 + i] = rq->ctx.level[i];
    }
    for (int i = 0; i < 6; i++) lb.h.last1[c * 6 + i] = rq->ctx.last1[i];
    for (int i = 0; i < (c ? 10 : 12); i++) lb.h.last2[c * 12 + i] = rq->ctx.last2[i];
    lbac_enc_run_length_cc_rdo(&lb, levels + rq->coef_offset, rq->log2w, rq->log2h, rq->num_sig, c);
    out->bits = lb.bitcounter;
    out->range = (u16)lb.range;
    out->pad = 0;
    for (int i = 0; i < 12; i++) {
        out->ctx.run[i] = lb.h.run[c * 12 + i];
        out->ctx.run_rdoq[i] = lb.h.run_rdoq[c * 12 + i];
        out->ctx.level[i] = lb.h.level[c * 12 + i];
    }
    for (int i = 0; i < 6; i++) out->ctx.last1[i] = lb.h.last1[c * 6 + i];
    for (int i = 0; i < 12; i++) out->ctx.last2[i] = (c && i >= 10) ? rq->ctx.last2[i] : lb.h.last2[c * 12 + i];
}

/* one entry of the reference's context-model transition table: MPS (mps = 1) or LPS */
int refk_lbac_next(int model, int mps)
{
    s16 m = (s16)model;
    lbac_encode_bin_for_rdoq(mps ? (u32)(m & 1) : (u32)!(m & 1), &m);
    return m;
}

/* ---- 9. weighted quantisation ----------------------------------------------------------------
 * quant_non_zero (src/quant.c:315) with pichdr->pic_wq_enable set: core->wq[0] = wq4 (4x4),
 * core->wq[1] = wq8 (8x8); the request as for refk_rdoq (lambda and estimates unused). */
int refk_quant_wq(const glue_rdoq_req_t *rq, u8 *wq4, u8 *wq8, s16 *coef)
{
    refk_init();
    static core_t *core = NULL;
    static com_info_t info;
    static com_pic_header_t pichdr;
    if (!core) core = (core_t *)calloc(1, sizeof(core_t));
    memset(&info, 0, sizeof(info));
    memset(&pichdr, 0, sizeof(pichdr));
    info.bit_depth_internal = 8;
    pichdr.pic_wq_enable = 1;
    core->info = &info;
    core->pichdr = &pichdr;
    core->wq[0] = wq4;
    core->wq[1] = wq8;
    return quant_non_zero(core, rq->qp, (double)rq->lambda / 32768.0, rq->is_intra, coef + rq->coef_offset,
                          rq->log2w, rq->log2h, rq->ch_type, rq->slice_type);
}

/* com_get_affine_mvp_scaling (src/com_util.c:1983) for one CU; map_mv / map_refi point at the
 * field's SCU (0, 0) (the border before it readable), ref_ptr[n_ref][2] the reference POCs */
void refk_affine_mvp(s64 ptr, const s64 *ref_ptr, int n_ref, s16 *map_mv, s8 *map_refi, int i_scu, int scup,
                     int lidx, int cur_refi, int cu_width, int mvr, s32 *mvp_out)
{
    static com_ref_pic_t refp[MAX_REFS][REFP_NUM];
    memset(refp, 0, sizeof(refp));
    for (int i = 0; i < n_ref && i < MAX_REFS; i++) {
        refp[i][0].ptr = ref_ptr[i * 2 + 0];
        refp[i][1].ptr = ref_ptr[i * 2 + 1];
    }
    CPMV mvp[VER_NUM][MV_D];
    com_get_affine_mvp_scaling(ptr, scup, lidx, (s8)cur_refi, (s16(*)[REFP_NUM][MV_D])map_mv,
                               (s8(*)[REFP_NUM])map_refi, refp, cu_width, cu_width, i_scu, mvp, NULL, NULL,
                               (u8)mvr);
    for (int g = 0; g < 2; g++)
        for (int d = 0; d < 2; d++) mvp_out[g * 2 + d] = mvp[g][d];
}

/* com_get_affine_merge_candidate (src/com_util.c:1761) for one CU.  The maps point at the
 * field's SCU (0, 0) (the border before it readable); the colocated picture's maps, POC and
 * list_ptr go into refp[0][REFP_1] for B slices and refp[0][REFP_0] otherwise, as the function
 * reads them.  out: num, cp_num[5], refi[5][2], cpmv[5][2][3][2] (vertices past cp_num zeroed). */
void refk_affine_merge(s64 ptr, const s64 *ref0_ptr, s64 *col_list_ptr, s16 *map_mv, s8 *map_refi, u8 *map_scu,
                       u32 *map_pos, s16 *col_mv, s8 *col_refi, int i_scu, int pic_w_scu, int pic_h_scu,
                       int slice_type, int log2_max_cuwh, int scup, int cu_width, int cu_height, s32 *num,
                       s8 *cp_num, s8 *refi, s32 *cpmv)
{
    static com_ref_pic_t refp[MAX_REFS][REFP_NUM];
    memset(refp, 0, sizeof(refp));
    refp[0][REFP_0].ptr = ref0_ptr[0];
    refp[0][REFP_1].ptr = ref0_ptr[1];
    com_ref_pic_t *col = &refp[0][slice_type == SLICE_B ? REFP_1 : REFP_0];
    col->map_mv = (s16(*)[REFP_NUM][MV_D])col_mv;
    col->map_refi = (s8(*)[REFP_NUM])col_refi;
    col->list_ptr = col_list_ptr;
    s8 mrg_refi[AFF_MAX_NUM_MRG][REFP_NUM];
    CPMV mrg_cpmv[AFF_MAX_NUM_MRG][REFP_NUM][VER_NUM][MV_D];
    int mrg_cp_num[AFF_MAX_NUM_MRG];
    memset(mrg_cpmv, 0, sizeof(mrg_cpmv));
    *num = com_get_affine_merge_candidate(ptr, scup, (s8(*)[REFP_NUM])map_refi, (s16(*)[REFP_NUM][MV_D])map_mv,
                                          (com_scu_t *)map_scu, map_pos, refp, cu_width, cu_height, i_scu, pic_w_scu,
                                          pic_h_scu, slice_type, mrg_refi, mrg_cpmv, mrg_cp_num, log2_max_cuwh);
    for (int k = 0; k < AFF_MAX_NUM_MRG; k++) {
        cp_num[k] = (s8)mrg_cp_num[k];
        for (int l = 0; l < REFP_NUM; l++) {
            refi[k * 2 + l] = mrg_refi[k][l];
            for (int i = 0; i < 3; i++)
                for (int d = 0; d < MV_D; d++)
                    cpmv[((k * 2 + l) * 3 + i) * 2 + d] = i < mrg_cp_num[k] ? mrg_cpmv[k][l][i][d] : 0;
        }
    }
}

/* ---- the encoder's final CU decisions (labels for the pruning network) ----
 * lbac_enc_unit (src/entropy.c:2461) codes each final CU of a picture into the bitstream; the
 * library is linked with --wrap=lbac_enc_unit, so the CU tree's calls (src/uavs3e.c:646) come
 * here first.  With UAVS3E_CU_LOG set, each call appends "x y w h intra ipm" (luma position and
 * size, 1 for an intra CU, its first luma prediction mode) to that file. */
int __real_lbac_enc_unit(lbac_t *lbac, bs_t *bs, core_t *core, enc_cu_t *cu_data, int x, int y, int cup, int cu_width,
                         int cu_height);

int __wrap_lbac_enc_unit(lbac_t *lbac, bs_t *bs, core_t *core, enc_cu_t *cu_data, int x, int y, int cup, int cu_width,
                         int cu_height)
{
    static FILE *log_file;
    static int log_init;
    const int r = __real_lbac_enc_unit(lbac, bs, core, cu_data, x, y, cup, cu_width, cu_height);
    if (!log_init) {
        const char *path = getenv("UAVS3E_CU_LOG");
        if (path) log_file = fopen(path, "a");
        log_init = 1;
    }
    if (log_file) {
        const com_mode_t *m = &core->mod_info_curr;
        fprintf(log_file, "%d %d %d %d %d %d\n", x, y, cu_width, cu_height, m->cu_mode == MODE_INTRA,
                (int)m->ipm[0][0]);
        fflush(log_file);
    }
    return r;
}
