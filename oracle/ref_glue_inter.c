/*
 * ref_glue_inter.c -- test-side glue that compiles the reference's src/inter.c a second time
 * (oracle/Makefile, target "ref") to call its file-local affine motion search.  TEST
 * INFRASTRUCTURE ONLY: nothing in the product library links or loads this.
 *
 * The functions src/inter.c exports are renamed before the include, so this translation unit
 * defines no symbol twice; everything it adds is the flat wrapper refk_affine_me below.
 */
#define analyze_inter_cu          refdup_analyze_inter_cu
#define inter_search_init         refdup_inter_search_init
#define inter_search_create       refdup_inter_search_create
#define inter_search_free         refdup_inter_search_free
#define pinter_residue_rdo_chroma refdup_pinter_residue_rdo_chroma
#include "inter.c"

void refk_init(void);

/* Layout of req/out: orc_affme_req_t / orc_affme_out_t (oracle.h). */
typedef struct {
    s16 x, y; u8 w, h; u8 ref_slot; s8 refi; u8 num_refp; u8 mvr; u8 flags; u8 other_slot;
    u32 lambda_mv; s32 mot_bits_other; s32 pad;
    s32 mvp[2][2]; s32 mv[2][2]; s32 other_mv[2][2];
} glue_affme_req_t;
typedef struct { s32 mv[2][2]; u32 satd; s32 bits; u64 cost; } glue_affme_out_t;

static void affme_pic(com_pic_t *pic, pel *plane, int i_ref, int W, int H)
{
    memset(pic, 0, sizeof(*pic));
    pic->y = plane;
    pic->stride_luma = i_ref;
    pic->width_luma = W;
    pic->height_luma = H;
}

/*
 * One affine_me_gradient call (src/inter.c:1339) as list 0 of a CU at (x, y): pi->ref_pic is
 * the integer plane planes[ref_slot * 16] (stride i_ref, padded by >= 144).  Flags (bit 0 bi,
 * bit 1 uni start, bit 2 8x8 sub-blocks):
 *   - bi: the org is create_bi_org (:55) of the other list's prediction by
 *     com_mc_blk_affine_luma with 8x8 sub-blocks, and the call runs with bi = 1 and 8x8
 *     sub-blocks, as analyze_affine_bi (:1730) makes it;
 *   - uni start: the start CPMVs are chosen as analyze_affine_uni (:1607-1647) chooses them,
 *     from the MVP and pi->best_mv_uni = req->mv[0] (quarter samples), by the reference's own
 *     mv_clip, com_mv_rounding_s32, com_mc_blk_affine_luma, com_had and affine_mv_bits.
 * out->cost is the call's return value + MV_COST(affine_mv_bits of the result (+ the other
 * list's bits for bi)), as both callers form it.
 */
void refk_affine_me(int W, int H, pel *org, int i_org, pel **planes, int i_ref, const glue_affme_req_t *rq,
                    glue_affme_out_t *out)
{
    refk_init();
    inter_search_t *pi = (inter_search_t *)calloc(1, sizeof(inter_search_t));
    com_pic_t pic, pic_o;
    ALIGNED_32(pel org_bi[MAX_CU_DIM]);
    ALIGNED_32(pel pred[MAX_CU_DIM]);
    const int x = rq->x, y = rq->y, w = rq->w, h = rq->h, bi = rq->flags & 1;
    const int sub = (bi || (rq->flags & 4)) ? 8 : 4;
    u32 lambda_mv = rq->lambda_mv;
    s8 refi = rq->refi;
    affme_pic(&pic, planes[rq->ref_slot * 16], i_ref, W, H);
    pi->bit_depth = 8;
    pi->ref_pic = &pic;
    pi->num_refp = rq->num_refp;
    pi->curr_mvr = rq->mvr;
    pi->lambda_mv = rq->lambda_mv;
    pi->mot_bits[REFP_1] = rq->mot_bits_other;
    pel *o = org + y * i_org + x;
    if (bi) {
        affme_pic(&pic_o, planes[rq->other_slot * 16], i_ref, W, H);
        CPMV omv[VER_NUM][MV_D] = { { rq->other_mv[0][0], rq->other_mv[0][1] }, { rq->other_mv[1][0], rq->other_mv[1][1] } };
        com_mc_blk_affine_luma(x, y, W, H, w, h, omv, &pic_o, pred, 8, 8, 8);
        create_bi_org(o, pred, i_org, w, h, org_bi, w, 8);
        pi->org = org_bi;
        pi->i_org = w;
    } else {
        pi->org = o;
        pi->i_org = i_org;
    }
    CPMV mvp[VER_NUM][MV_D] = { { rq->mvp[0][0], rq->mvp[0][1] }, { rq->mvp[1][0], rq->mvp[1][1] } };
    CPMV mv[VER_NUM][MV_D] = { { rq->mv[0][0], rq->mv[0][1] }, { rq->mv[1][0], rq->mv[1][1] } };
    if (!bi && (rq->flags & 2)) {
        com_mc_blk_affine_luma(x, y, W, H, w, h, mvp, &pic, pred, sub, sub, 8);
        u64 mvp_best = com_had(w, h, o, i_org, pred, w, 8);
        mvp_best += MV_COST(affine_mv_bits(mvp, mvp, rq->num_refp, refi, rq->mvr));
        s16 mv_cliped[REFP_NUM][MV_D];
        s8 refi_t[REFP_NUM] = { refi, -1 };
        mv_cliped[REFP_0][MV_X] = (s16)rq->mv[0][0];
        mv_cliped[REFP_0][MV_Y] = (s16)rq->mv[0][1];
        mv_clip(x, y, W, H, w, h, refi_t, mv_cliped, mv_cliped);
        CPMV tmp[VER_NUM][MV_D];
        for (int v = 0; v < 2; v++) {
            s32 tx = (s32)mv_cliped[REFP_0][MV_X] << 2, ty = (s32)mv_cliped[REFP_0][MV_Y] << 2;
            if (rq->mvr == 1) com_mv_rounding_s32(tx, ty, &tx, &ty, 4, 4);
            tmp[v][MV_X] = (CPMV)COM_CLIP3(COM_CPMV_MIN, COM_CPMV_MAX, tx);
            tmp[v][MV_Y] = (CPMV)COM_CLIP3(COM_CPMV_MIN, COM_CPMV_MAX, ty);
        }
        com_mc_blk_affine_luma(x, y, W, H, w, h, tmp, &pic, pred, sub, sub, 8);
        u64 mvp_temp = com_had(w, h, o, i_org, pred, w, 8);
        mvp_temp += MV_COST(affine_mv_bits(tmp, mvp, rq->num_refp, refi, rq->mvr));
        if (mvp_temp < mvp_best) CP128(mv, tmp);
        else CP128(mv, mvp);
    }
    u64 satd = affine_me_gradient(pi, x, y, CONV_LOG2(w), CONV_LOG2(h), &refi, REFP_0, mvp, mv, bi, sub, sub);
    int bits = affine_mv_bits(mv, mvp, rq->num_refp, refi, rq->mvr) + (bi ? rq->mot_bits_other : 0);
    for (int v = 0; v < 2; v++) { out->mv[v][0] = mv[v][MV_X]; out->mv[v][1] = mv[v][MV_Y]; }
    out->satd = (u32)satd;
    out->bits = bits;
    out->cost = satd + MV_COST(bits);
    free(pi);
}
