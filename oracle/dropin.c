/*
 * dropin.c -- TEST INFRASTRUCTURE: a drop-in check of the kernel-table boundary on the CPU.
 *
 * Loaded with LD_PRELOAD into the reference encoder binary (oracle/_ref/uavs3enc, built by
 * `make -C oracle ref`), it wraps uavs3e_create() (src/uavs3e.c:1266): after the encoder has
 * filled its kernel table (uavs3e_funs_init_c, src/com_util.c:3131), every hot-path member of
 * funs_handle_t (inc/com_util.h:278-341) -- the members the GPU library installs -- is replaced
 * by an adapter onto the oracle restatement (oracle.c), which the GPU entries are checked
 * against bit for bit.  An encode through the restated kernels must give the reference's
 * bitstream md5.  The layout of the table is uavs3e_cuda_funs_t (include/uavs3e_cuda_table.h,
 * checked member by member against funs_handle_t in ref_glue.c).
 *
 * UAVS3E_DROPIN_SKIP (environment) lists member families to leave as the reference's:
 * "intra,mc,frame,recon,dquant,itx,tx,sad,ssd,satd,pel,quant".  UAVS3E_DROPIN_PLANT=satd adds
 * 1 to every 8x8 SATD (a planted mistake: the check must then see a different bitstream).
 * UAVS3E_DROPIN_COSTLOG=1 records every cost call of the table as installed
 * (uavs3e_gb300/dropin/costlog.h): with every family skipped, that is the reference's own
 * functions, the record the GPU entries' record is compared with.
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"
#include "../include/uavs3e_cuda_table.h"
#include "../uavs3e_gb300/dropin/costlog.h"

#define CLIP8(v) ((v) < 0 ? 0 : (v) > 255 ? 255 : (v))

/* ---- intra prediction: the table passes src = nb + INTRA_NEIB_MID ---- */
static void a_dc(u8 *s, u8 *d, int id, int w, int h, uint16_t av, int bd) { orc_ipred_dc(s - ORC_NEIB_MID, d, id, w, h, av, bd); }
static void a_plane(u8 *s, u8 *d, int id, int w, int h, int bd) { orc_ipred_plane(s - ORC_NEIB_MID, d, id, w, h, bd); }
static void a_bi(u8 *s, u8 *d, int id, int w, int h, int bd) { orc_ipred_bi(s - ORC_NEIB_MID, d, id, w, h, bd); }
static void a_plane_ipf(u8 *s, s16 *d, int w, int h) { orc_ipred_plane_ipf(s - ORC_NEIB_MID, d, w, h); }
static void a_bi_ipf(u8 *s, s16 *d, int w, int h) { orc_ipred_bi_ipf(s - ORC_NEIB_MID, d, w, h); }
/* ipred_vert / ipred_hor (src/com_ipred.c:114-128): called with the top row / the first left
 * sample, the left column running towards lower addresses */
static void a_ver(u8 *s, u8 *d, int id, int w, int h) { for (int y = 0; y < h; y++) memcpy(d + y * id, s, (size_t)w); }
static void a_hor(u8 *s, u8 *d, int id, int w, int h) { for (int y = 0; y < h; y++) memset(d + y * id, s[-y], (size_t)w); }
static void a_ang(u8 *s, u8 *d, int id, int mode, int w, int h) { orc_ipred_ang(s - ORC_NEIB_MID, d, id, mode, w, h); }
static void a_ipf(u8 *s, u8 *d, int id, int ipm, int w, int h, int bd) { orc_ipf_core(s - ORC_NEIB_MID, d, id, ipm, w, h, bd); }
static void a_ipf16(u8 *s, u8 *d, int id, s16 *p, int ipm, int w, int h, int bd) { orc_ipf_core_s16(s - ORC_NEIB_MID, d, id, p, ipm, w, h, bd); }

/* ---- block MC ---- */
static void a_ipcpy(const u8 *s, int is, u8 *d, int id, int w, int h) { orc_ipcpy(s, is, d, id, w, h); }
#define IPFLT(t) static void a_ipflt##t(const u8 *s, int is, u8 *d, int id, int w, int h, const s8 *c, int mx) { orc_ipflt(t, s, is, d, id, w, h, c, mx); }
IPFLT(0) IPFLT(1) IPFLT(2) IPFLT(3)
#define IPFLTX(t) static void a_ipfltx##t(const u8 *s, int is, u8 *d, int id, int w, int h, const s8 *cx, const s8 *cy, int mx) { orc_ipflt_ext(t, s, is, d, id, w, h, cx, cy, mx); }
IPFLTX(0) IPFLTX(1)

/* ---- frame interpolation passes (com_if_filter_hor_8 / ver_8 / if_ver_luma_frame_ext,
 * src/com_mc.c:668-758): 8-tap sums, (t + 32) >> 6 for the planes, the raw horizontal sums
 * kept in s16 for the diagonal pass, (t + 2048) >> 12 there (8-bit) ---- */
static void a_flt_hor(const u8 *s, int is, u8 *d[3], int id, s16 *dt[3], int idt, int w, int h, int8_t (*c)[8], int bd)
{
    (void)bd;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++)
            for (int f = 0; f < 3; f++) {
                int t = 0;
                for (int k = 0; k < 8; k++) t += s[y * is + x + k - 3] * c[f][k];
                dt[f][y * idt + x] = (s16)t;
                d[f][y * id + x] = (u8)CLIP8((t + 32) >> 6);
            }
}
static void a_flt_ver(const u8 *s, int is, u8 *d[3], int id, int w, int h, int8_t (*c)[8], int bd)
{
    (void)bd;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++)
            for (int f = 0; f < 3; f++) {
                int t = 0;
                for (int k = 0; k < 8; k++) t += s[(y + k - 3) * is + x] * c[f][k];
                d[f][y * id + x] = (u8)CLIP8((t + 32) >> 6);
            }
}
static void a_flt_ver_ext(const s16 *s, int is, u8 *d[3], int id, int w, int h, int8_t (*c)[8], int bd)
{
    (void)bd;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++)
            for (int f = 0; f < 3; f++) {
                int t = 0;
                for (int k = 0; k < 8; k++) t += s[(y + k - 3) * is + x] * c[f][k];
                d[f][y * id + x] = (u8)CLIP8((t + 2048) >> 12);
            }
}

/* ---- recon, dequant, transforms ---- */
static void a_recon(s16 *r, u8 *p, int ip, int w, int h, u8 *rec, int ir, int cbf, int bd) { orc_recon(r, p, ip, w, h, rec, ir, cbf, bd); }
static void a_dq0(s16 *c, s16 *o, u8 *wq[2], int lw, int lh, int sc, int sh, int bd) { orc_dquant(0, c, o, wq[0], wq[1], lw, lh, sc, sh, bd); }
static void a_dq1(s16 *c, s16 *o, u8 *wq[2], int lw, int lh, int sc, int sh, int bd) { orc_dquant(1, c, o, wq ? wq[0] : NULL, wq ? wq[1] : NULL, lw, lh, sc, sh, bd); }
#define ITX2(a, b) static void a_itx2_##a##_##b(s16 *c, s16 *r, int bd) { orc_itrans_dct2(a, b, c, r, bd); }
#define TX2(a, b) static void a_tx2_##a##_##b(s16 *s, s16 *d, int bd) { orc_trans_dct2(a, b, s, d, bd); }
#define ROW(M, a) M(a, 1) M(a, 2) M(a, 3) M(a, 4) M(a, 5) M(a, 6)
ROW(ITX2, 1) ROW(ITX2, 2) ROW(ITX2, 3) ROW(ITX2, 4) ROW(ITX2, 5) ROW(ITX2, 6)
ROW(TX2, 1) ROW(TX2, 2) ROW(TX2, 3) ROW(TX2, 4) ROW(TX2, 5) ROW(TX2, 6)
#define ITX87(t, n) static void a_itx87_##t##_##n(s16 *c, s16 *b, int sh, int line, int mx, int mn) { orc_itrans_dct8_dst7(t, n, c, b, sh, line, mx, mn); }
#define TX87(t, n) static void a_tx87_##t##_##n(s16 *s, s16 *d, int sh, int line) { orc_trans_dct8_dst7(t, n, s, d, sh, line); }
ROW(ITX87, 0) ROW(ITX87, 1) ROW(TX87, 0) ROW(TX87, 1)

/* ---- costs and pel ops, one instance per width index (w = 4 << widx) ---- */
#define WIDX(M) M(0, 4) M(1, 8) M(2, 16) M(3, 32) M(4, 64) M(5, 128)
#define SAD(i, w) static u32 a_sad##i(u8 *o, int io, u8 *p, int ip, int h) { return orc_sad(w, h, o, io, p, ip); }
#define SADX3(i, w) static void a_sadx3_##i(u8 *o, int io, u8 *p0, u8 *p1, u8 *p2, int ip, u32 s[3], int h) \
    { s[0] = orc_sad(w, h, o, io, p0, ip); s[1] = orc_sad(w, h, o, io, p1, ip); s[2] = orc_sad(w, h, o, io, p2, ip); }
#define SADX4(i, w) static void a_sadx4_##i(u8 *o, int io, u8 *p0, u8 *p1, u8 *p2, u8 *p3, int ip, u32 s[4], int h) \
    { s[0] = orc_sad(w, h, o, io, p0, ip); s[1] = orc_sad(w, h, o, io, p1, ip); s[2] = orc_sad(w, h, o, io, p2, ip); s[3] = orc_sad(w, h, o, io, p3, ip); }
#define SSD(i, w) static u64 a_ssd##i(u8 *o, int io, u8 *p, int ip, int h) { return orc_ssd(w, h, o, io, p, ip); }
#define DIFF(i, w) static void a_diff##i(u8 *o, int io, u8 *p, int ip, s16 *r, int ir, int h) { orc_pel_diff(w, h, o, io, p, ip, r, ir); }
#define AVRG(i, w) static void a_avrg##i(u8 *d, int id, u8 *s1, u8 *s2, int h) { orc_pel_avrg(w, h, d, id, s1, s2); }
WIDX(SAD) WIDX(SADX3) WIDX(SADX4) WIDX(SSD) WIDX(DIFF) WIDX(AVRG)
static int g_plant;
#define SATD(a, b) static u32 a_satd_##a##_##b(u8 *o, int io, u8 *p, int ip) \
    { return orc_satd_tile(4 << a, 4 << b, o, io, p, ip) + (u32)(g_plant && a == 1 && b == 1); }
SATD(0, 0) SATD(0, 1) SATD(1, 0) SATD(1, 1) SATD(2, 1) SATD(1, 2)

static int a_rdoq(s16 *c, int n, int qv, int qb, int32_t es, int pb, u32 *ac, s16 *al, int64_t *ue)
{
    return orc_quant_rdoq(c, n, qv, qb, es, pb, ac, al, ue);
}
static int a_qcheck(s16 *c, int n, int thr) { return orc_quant_check(c, n, thr); }

static int skip(const char *fam)
{
    const char *e = getenv("UAVS3E_DROPIN_SKIP");
    return e && strstr(e, fam) != NULL;
}

static void install(uavs3e_cuda_funs_t *t)
{
    orc_init();
    g_plant = getenv("UAVS3E_DROPIN_PLANT") && strstr(getenv("UAVS3E_DROPIN_PLANT"), "satd");
    if (!skip("intra")) {
        t->intra_pred_dc = a_dc; t->intra_pred_plane = a_plane; t->intra_pred_bi = a_bi;
        t->intra_pred_plane_ipf = a_plane_ipf; t->intra_pred_bi_ipf = a_bi_ipf;
        t->intra_pred_ver = a_ver; t->intra_pred_hor = a_hor;
        for (int m = 0; m < UAVS3E_CUDA_IPD_CNT; m++)
            if (t->intra_pred_ang[m]) t->intra_pred_ang[m] = a_ang;   /* the members the reference sets */
        t->intra_pred_ipf_core = a_ipf; t->intra_pred_ipf_core_s16 = a_ipf16;
    }
    if (!skip("mc")) {
        for (int i = 0; i < UAVS3E_CUDA_CU_SIZE_NUM; i++) {
            t->ipcpy[i] = a_ipcpy;
            t->ipflt[0][i] = a_ipflt0; t->ipflt[1][i] = a_ipflt1; t->ipflt[2][i] = a_ipflt2; t->ipflt[3][i] = a_ipflt3;
            t->ipflt_ext[0][i] = a_ipfltx0; t->ipflt_ext[1][i] = a_ipfltx1;
        }
    }
    if (!skip("frame")) {
        t->ip_flt_y_hor = a_flt_hor; t->ip_flt_y_ver = a_flt_ver; t->ip_flt_y_ver_ext = a_flt_ver_ext;
    }
    if (!skip("recon"))
        for (int i = 0; i < UAVS3E_CUDA_CU_SIZE_NUM; i++) t->recon[i] = a_recon;
    if (!skip("dquant")) { t->dquant[0] = a_dq0; t->dquant[1] = a_dq1; }
#define SET2(arr, M, a) arr[a - 1][0] = M##_##a##_1; arr[a - 1][1] = M##_##a##_2; arr[a - 1][2] = M##_##a##_3; \
    arr[a - 1][3] = M##_##a##_4; arr[a - 1][4] = M##_##a##_5; arr[a - 1][5] = M##_##a##_6;
    if (!skip("itx")) {
        SET2(t->itrans_dct2, a_itx2, 1) SET2(t->itrans_dct2, a_itx2, 2) SET2(t->itrans_dct2, a_itx2, 3)
        SET2(t->itrans_dct2, a_itx2, 4) SET2(t->itrans_dct2, a_itx2, 5) SET2(t->itrans_dct2, a_itx2, 6)
        for (int ty = 0; ty < 2; ty++) {
            void (*const f0[6])(s16 *, s16 *, int, int, int, int) = { a_itx87_0_1, a_itx87_0_2, a_itx87_0_3, a_itx87_0_4, a_itx87_0_5, a_itx87_0_6 };
            void (*const f1[6])(s16 *, s16 *, int, int, int, int) = { a_itx87_1_1, a_itx87_1_2, a_itx87_1_3, a_itx87_1_4, a_itx87_1_5, a_itx87_1_6 };
            for (int n = 0; n < 6; n++) t->itrans_dct8_dst7[ty][n] = ty ? f1[n] : f0[n];
        }
    }
    if (!skip("tx")) {
        SET2(t->trans_dct2, a_tx2, 1) SET2(t->trans_dct2, a_tx2, 2) SET2(t->trans_dct2, a_tx2, 3)
        SET2(t->trans_dct2, a_tx2, 4) SET2(t->trans_dct2, a_tx2, 5) SET2(t->trans_dct2, a_tx2, 6)
        void (*const g0[6])(s16 *, s16 *, int, int) = { a_tx87_0_1, a_tx87_0_2, a_tx87_0_3, a_tx87_0_4, a_tx87_0_5, a_tx87_0_6 };
        void (*const g1[6])(s16 *, s16 *, int, int) = { a_tx87_1_1, a_tx87_1_2, a_tx87_1_3, a_tx87_1_4, a_tx87_1_5, a_tx87_1_6 };
        for (int n = 0; n < 6; n++) { t->trans_dct8_dst7[0][n] = g0[n]; t->trans_dct8_dst7[1][n] = g1[n]; }
    }
    if (!skip("sad")) {
        u32 (*const s[6])(u8 *, int, u8 *, int, int) = { a_sad0, a_sad1, a_sad2, a_sad3, a_sad4, a_sad5 };
        void (*const s3[6])(u8 *, int, u8 *, u8 *, u8 *, int, u32 *, int) = { a_sadx3_0, a_sadx3_1, a_sadx3_2, a_sadx3_3, a_sadx3_4, a_sadx3_5 };
        void (*const s4[6])(u8 *, int, u8 *, u8 *, u8 *, u8 *, int, u32 *, int) = { a_sadx4_0, a_sadx4_1, a_sadx4_2, a_sadx4_3, a_sadx4_4, a_sadx4_5 };
        for (int i = 0; i < 6; i++) { t->cost_sad[i] = s[i]; t->cost_sad_x3[i] = s3[i]; t->cost_sad_x4[i] = s4[i]; }
    }
    if (!skip("ssd")) {
        u64 (*const s[6])(u8 *, int, u8 *, int, int) = { a_ssd0, a_ssd1, a_ssd2, a_ssd3, a_ssd4, a_ssd5 };
        for (int i = 0; i < 6; i++) t->cost_ssd[i] = s[i];
    }
    if (!skip("satd")) {
        t->cost_satd[0][0] = a_satd_0_0; t->cost_satd[0][1] = a_satd_0_1; t->cost_satd[1][0] = a_satd_1_0;
        t->cost_satd[1][1] = a_satd_1_1; t->cost_satd[2][1] = a_satd_2_1; t->cost_satd[1][2] = a_satd_1_2;
    }
    if (!skip("pel")) {
        void (*const d[6])(u8 *, int, u8 *, int, s16 *, int, int) = { a_diff0, a_diff1, a_diff2, a_diff3, a_diff4, a_diff5 };
        void (*const a[6])(u8 *, int, u8 *, u8 *, int) = { a_avrg0, a_avrg1, a_avrg2, a_avrg3, a_avrg4, a_avrg5 };
        for (int i = 0; i < 6; i++) { t->pel_diff[i] = d[i]; t->pel_avrg[i] = a[i]; }
    }
    if (!skip("quant")) { t->quant_rdoq = a_rdoq; t->quant_check = a_qcheck; }
}

/* the wrapped encoder constructor */
void *uavs3e_create(void *cfg, int *err)
{
    void *(*real)(void *, int *) = (void *(*)(void *, int *))dlsym(RTLD_NEXT, "uavs3e_create");
    if (!real) {
        fprintf(stderr, "dropin: uavs3e_create not found\n");
        exit(3);
    }
    void *h = real(cfg, err);
    uavs3e_cuda_funs_t *t = (uavs3e_cuda_funs_t *)dlsym(RTLD_DEFAULT, "uavs3e_funs_handle");
    if (!t) {
        fprintf(stderr, "dropin: uavs3e_funs_handle not found\n");
        exit(3);
    }
    install(t);
    if (getenv("UAVS3E_DROPIN_COSTLOG") && getenv("UAVS3E_DROPIN_COSTLOG")[0] == '1') costlog_install(t);
    fprintf(stderr, "dropin: kernel table replaced by the oracle restatement\n");
    return h;
}
