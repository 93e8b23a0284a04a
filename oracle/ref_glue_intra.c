/*
 * ref_glue_intra.c -- test-side glue that compiles the reference's src/intra.c a second time
 * (oracle/Makefile, target "ref") to call its file-local make_ipred_list.  TEST INFRASTRUCTURE
 * ONLY: nothing in the product library links or loads this.
 */
#define analyze_intra_cu refdup_analyze_intra_cu
#include "intra.c"

void refk_init(void);

/* Layout of req / out: orc_rmd_req_t / orc_rmd_out_t (oracle.h). */
typedef struct {
    u32 satd_row; u8 pb_w, pb_h; u8 mpm[2]; u8 skip_ipd; u8 fast; u16 range; s16 ctx[7]; u8 pad[6];
    double sqrt_lambda; u64 inter_satd; double satd_threshold;
} glue_rmd_req_t;
typedef struct { s8 list[5]; u8 count; u8 pad[2]; } glue_rmd_out_t;

/*
 * make_ipred_list (src/intra.c:226) for one prediction block: nb is its INTRA_NEIB_SIZE
 * neighbour array, org its samples (stride s_org), avail / ipf the com_intra_pred arguments; the
 * LBAC state core->lbac_bakup is a reset coder (lbac_reset) with the request's range and intra_dir
 * context models, the other request fields go where make_ipred_list reads them.  satd_out[33]
 * receives what check_one_mode computes for each mode (com_intra_pred + calc_satd_intra), the
 * input of the restatement.
 */
void refk_make_ipred_list(pel *nb, pel *org, int s_org, int avail, int ipf, const glue_rmd_req_t *rq,
                          glue_rmd_out_t *out, u32 *satd_out)
{
    refk_init();
    core_t *core = (core_t *)calloc(1, sizeof(core_t));
    com_info_t *info = (com_info_t *)calloc(1, sizeof(com_info_t));
    info->bit_depth_internal = 8;
    info->intra_fast_rmd = rq->fast;
    core->info = info;
    memcpy(core->nb[Y_C], nb, sizeof(pel) * INTRA_NEIB_SIZE);
    core->mod_info_curr.mpm[0][0] = rq->mpm[0];
    core->mod_info_curr.mpm[0][1] = rq->mpm[1];
    core->mod_info_curr.ipf_flag = (u8)ipf;
    lbac_reset(&core->lbac_bakup);
    core->lbac_bakup.range = rq->range;
    for (int i = 0; i < 7; i++) core->lbac_bakup.h.intra_dir[i] = rq->ctx[i];
    core->sqrt_lambda[0] = rq->sqrt_lambda;
    core->inter_satd = rq->inter_satd;
    core->satd_threshold = rq->satd_threshold;
    const int w = rq->pb_w, h = rq->pb_h;
    int list[IPD_CNT];
    const int cnt = make_ipred_list(core, w, h, CONV_LOG2(w), CONV_LOG2(h), org, s_org, list, 0, (u16)avail,
                                    rq->skip_ipd);
    for (int k = 0; k < 5; k++) out->list[k] = (s8)list[k];
    out->count = (u8)cnt;
    out->pad[0] = out->pad[1] = 0;
    ALIGNED_32(pel pred[MAX_CU_DIM]);
    for (int m = 0; m < IPD_CNT; m++) {
        com_intra_pred(core->nb[Y_C] + INTRA_NEIB_MID, pred, m, w, h, 8, (u16)avail, (u8)ipf);
        satd_out[m] = calc_satd_intra(w, h, org, pred, s_org, w, 8);
    }
    free(info);
    free(core);
}
