/*
 * uavs3e_cuda_table.h -- kernel-table entry points of libuavs3e_cuda.
 *
 * The reference encoder dispatches its hot kernels through one global struct of function
 * pointers, funs_handle_t uavs3e_funs_handle (inc/com_util.h:278-341, src/com_util.c:40),
 * filled by uavs3e_funs_init_c/_sse/_avx2 from uavs3e_create (src/uavs3e.c:1332-1339).
 * uavs3e_cuda_funs_t below has the same layout, and every function declared here has the exact
 * C signature of the table member it replaces.  uavs3e_cuda_install() writes them into a
 * caller's table (call it after uavs3e_create returns); members outside the hot path
 * (deblock, SAO, ALF, variance, SSIM, affine, sobel) keep the caller's pointers.
 *
 * Each entry evaluates its one call on the GPU: the inputs it reads are staged through a
 * per-thread pinned buffer, one kernel runs, the outputs are copied back, and the call
 * returns when they are in place (a synchronous "miss" path; the batched entry points of
 * uavs3e_cuda.h are the throughput path).  Entries are thread-safe (per-thread stream and
 * staging).  Errors are recorded in uavs3e_cuda_status(); the table signatures have no error
 * channel, and on error outputs are left unchanged (u32/u64 entries return 0).
 *
 * Types: pel = uint8_t, s8 = int8_t, s16 = int16_t, u8 = uint8_t, u32 = uint32_t,
 * s32 = int32_t, u64 = uint64_t, s64 = int64_t (8-bit build, inc/com_api.h:46).
 */
#ifndef UAVS3E_CUDA_TABLE_H
#define UAVS3E_CUDA_TABLE_H

#include <stdint.h>
#include "uavs3e_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

#define UAVS3E_CUDA_IPD_CNT        33   /* IPD_CNT, inc/com_define.h:377 */
#define UAVS3E_CUDA_CU_SIZE_NUM     6   /* CU_SIZE_NUM, inc/com_define.h:284 */
#define UAVS3E_CUDA_MAX_TR_LOG2     6   /* MAX_TR_LOG2, inc/com_define.h:273 */

/* Layout twin of funs_handle_t (inc/com_util.h:278-341), same member order and types.  The
 * pointer types of members outside the hot path are written as void * (same size). */
typedef struct uavs3e_cuda_funs_t {
    void (*intra_pred_dc)(uint8_t *src, uint8_t *dst, int i_dst, int width, int height, uint16_t cu_avail, int bit_depth);
    void (*intra_pred_plane)(uint8_t *src, uint8_t *dst, int i_dst, int width, int height, int bit_depth);
    void (*intra_pred_bi)(uint8_t *src, uint8_t *dst, int i_dst, int width, int height, int bit_depth);
    void (*intra_pred_plane_ipf)(uint8_t *src, int16_t *dst, int width, int height);
    void (*intra_pred_bi_ipf)(uint8_t *src, int16_t *dst, int width, int height);
    void (*intra_pred_ver)(uint8_t *src, uint8_t *dst, int i_dst, int width, int height);
    void (*intra_pred_hor)(uint8_t *src, uint8_t *dst, int i_dst, int width, int height);
    void (*intra_pred_ang[UAVS3E_CUDA_IPD_CNT])(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
    void (*intra_pred_ipf_core)(uint8_t *src, uint8_t *dst, int i_dst, int ipm, int w, int h, int bit_depth);
    void (*intra_pred_ipf_core_s16)(uint8_t *src, uint8_t *dst, int i_dst, int16_t *pred, int ipm, int w, int h, int bit_depth);

    void *deblock_luma[2];
    void *deblock_chroma[2];
    void *sao;
    void *sao_stat;
    void *alf;
    void *alf_fix;
    void *alf_calc;

    void (*ipcpy[UAVS3E_CUDA_CU_SIZE_NUM])(const uint8_t *src, int i_src, uint8_t *dst, int i_dst, int width, int height);
    void (*ipflt[4][UAVS3E_CUDA_CU_SIZE_NUM])(const uint8_t *src, int i_src, uint8_t *dst, int i_dst, int width, int height, const int8_t *coeff, int max_val);
    void (*ipflt_ext[2][UAVS3E_CUDA_CU_SIZE_NUM])(const uint8_t *src, int i_src, uint8_t *dst, int i_dst, int width, int height, const int8_t *coef_x, const int8_t *coef_y, int max_val);

    void (*ip_flt_y_hor)(const uint8_t *src, int i_src, uint8_t *dst[3], int i_dst, int16_t *dst_tmp[3], int i_dst_tmp, int width, int height, int8_t (*coeff)[8], int bit_depth);
    void (*ip_flt_y_ver)(const uint8_t *src, int i_src, uint8_t *dst[3], int i_dst, int width, int height, int8_t (*coeff)[8], int bit_depth);
    void (*ip_flt_y_ver_ext)(const int16_t *src, int i_src, uint8_t *dst[3], int i_dst, int width, int height, int8_t (*coeff)[8], int bit_depth);

    void (*recon[UAVS3E_CUDA_CU_SIZE_NUM])(int16_t *resi, uint8_t *pred, int i_pred, int width, int height, uint8_t *rec, int i_rec, int cbf, int bit_depth);
    void (*dquant[2])(int16_t *coef, int16_t *coef_out, uint8_t *wq_matrix[2], int log2_w, int log2_h, int scale, int shift, int bit_depth);

    void (*itrans_dct2[UAVS3E_CUDA_MAX_TR_LOG2][UAVS3E_CUDA_MAX_TR_LOG2])(int16_t *coef, int16_t *resi, int bit_depth);
    void (*itrans_dct8_dst7[2][UAVS3E_CUDA_MAX_TR_LOG2])(int16_t *coeff, int16_t *block, int shift, int line, int max_tr_val, int min_tr_val);
    void (*trans_dct2[UAVS3E_CUDA_MAX_TR_LOG2][UAVS3E_CUDA_MAX_TR_LOG2])(int16_t *coef, int16_t *resi, int bit_depth);
    void (*trans_dct8_dst7[2][UAVS3E_CUDA_MAX_TR_LOG2])(int16_t *src, int16_t *dst, int shift, int line);

    uint32_t (*cost_sad[UAVS3E_CUDA_CU_SIZE_NUM])(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred, int height);
    void (*cost_sad_x3[UAVS3E_CUDA_CU_SIZE_NUM])(uint8_t *p_org, int i_org, uint8_t *pred0, uint8_t *pred1, uint8_t *pred2, int i_pred, uint32_t sad[3], int height);
    void (*cost_sad_x4[UAVS3E_CUDA_CU_SIZE_NUM])(uint8_t *p_org, int i_org, uint8_t *pred0, uint8_t *pred1, uint8_t *pred2, uint8_t *pred3, int i_pred, uint32_t sad[4], int height);
    uint64_t (*cost_ssd[UAVS3E_CUDA_CU_SIZE_NUM])(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred, int height);
    uint32_t (*cost_satd[3][3])(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred);

    void *cost_var[UAVS3E_CUDA_CU_SIZE_NUM];
    void *ssim_4x4x2_core;
    void *ssim_end4;

    void (*pel_diff[UAVS3E_CUDA_CU_SIZE_NUM])(uint8_t *org, int i_org, uint8_t *pred, int i_pred, int16_t *resi, int i_resi, int height);
    void (*pel_avrg[UAVS3E_CUDA_CU_SIZE_NUM])(uint8_t *dst, int i_dst, uint8_t *src1, uint8_t *src2, int height);

    void *affine_sobel_flt_hor;
    void *affine_sobel_flt_ver;
    void *affine_coef_computer;

    int (*quant_rdoq)(int16_t *coef, int num, int q_value, int q_bits, int32_t err_scale, int precision_bits, uint32_t *abs_coef, int16_t *abs_level, int64_t *uncoded_err);
    int (*quant_check)(int16_t *coef, int num, int threshold);

    void *sobel_cost;
} uavs3e_cuda_funs_t;

/* Write every hot-path entry of this library into *table (a funs_handle_t, e.g.
 * &uavs3e_funs_handle) and initialise the library on device 0 if needed.  Returns 0 or an
 * error code. */
UAVS3E_CUDA_API int uavs3e_cuda_install(void *table);

/* ---- intra prediction: intra_pred_* members, src/com_ipred.c:114-368, 607-731, 844-1645 */
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_dc(uint8_t *src, uint8_t *dst, int i_dst, int width, int height, uint16_t cu_avail, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_plane(uint8_t *src, uint8_t *dst, int i_dst, int width, int height, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_bi(uint8_t *src, uint8_t *dst, int i_dst, int width, int height, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_plane_ipf(uint8_t *src, int16_t *dst, int width, int height);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_bi_ipf(uint8_t *src, int16_t *dst, int width, int height);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ver(uint8_t *src, uint8_t *dst, int i_dst, int width, int height);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_hor(uint8_t *src, uint8_t *dst, int i_dst, int width, int height);
/* intra_pred_ang[m], m = 3..32 except 12 and 24 (the reference leaves 0..2, 12 is set but 24 is not) */
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_3(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_4(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_5(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_6(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_7(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_8(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_9(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_10(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_11(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_12(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_13(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_14(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_15(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_16(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_17(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_18(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_19(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_20(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_21(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_22(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_23(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_25(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_26(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_27(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_28(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_29(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_30(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_31(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ang_32(uint8_t *src, uint8_t *dst, int i_dst, int uiDirMode, int iWidth, int iHeight);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ipf_core(uint8_t *src, uint8_t *dst, int i_dst, int ipm, int w, int h, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_intra_pred_ipf_core_s16(uint8_t *src, uint8_t *dst, int i_dst, int16_t *pred, int ipm, int w, int h, int bit_depth);

/* ---- motion compensation: ipcpy / ipflt / ipflt_ext / ip_flt_y_*, src/com_mc.c:461-758 */
UAVS3E_CUDA_API void uavs3e_cuda_ipcpy(const uint8_t *src, int i_src, uint8_t *dst, int i_dst, int width, int height);
UAVS3E_CUDA_API void uavs3e_cuda_ipflt_h8(const uint8_t *src, int i_src, uint8_t *dst, int i_dst, int width, int height, const int8_t *coeff, int max_val);
UAVS3E_CUDA_API void uavs3e_cuda_ipflt_h4(const uint8_t *src, int i_src, uint8_t *dst, int i_dst, int width, int height, const int8_t *coeff, int max_val);
UAVS3E_CUDA_API void uavs3e_cuda_ipflt_v8(const uint8_t *src, int i_src, uint8_t *dst, int i_dst, int width, int height, const int8_t *coeff, int max_val);
UAVS3E_CUDA_API void uavs3e_cuda_ipflt_v4(const uint8_t *src, int i_src, uint8_t *dst, int i_dst, int width, int height, const int8_t *coeff, int max_val);
UAVS3E_CUDA_API void uavs3e_cuda_ipflt_ext8(const uint8_t *src, int i_src, uint8_t *dst, int i_dst, int width, int height, const int8_t *coef_x, const int8_t *coef_y, int max_val);
UAVS3E_CUDA_API void uavs3e_cuda_ipflt_ext4(const uint8_t *src, int i_src, uint8_t *dst, int i_dst, int width, int height, const int8_t *coef_x, const int8_t *coef_y, int max_val);
UAVS3E_CUDA_API void uavs3e_cuda_ip_flt_y_hor(const uint8_t *src, int i_src, uint8_t *dst[3], int i_dst, int16_t *dst_tmp[3], int i_dst_tmp, int width, int height, int8_t (*coeff)[8], int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_ip_flt_y_ver(const uint8_t *src, int i_src, uint8_t *dst[3], int i_dst, int width, int height, int8_t (*coeff)[8], int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_ip_flt_y_ver_ext(const int16_t *src, int i_src, uint8_t *dst[3], int i_dst, int width, int height, int8_t (*coeff)[8], int bit_depth);

/* ---- reconstruction, dequantisation, transforms: src/com_util.c:3107, src/com_itdq.c, src/transform.c */
UAVS3E_CUDA_API void uavs3e_cuda_recon(int16_t *resi, uint8_t *pred, int i_pred, int width, int height, uint8_t *rec, int i_rec, int cbf, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_dquant(int16_t *coef, int16_t *coef_out, uint8_t *wq_matrix[2], int log2_w, int log2_h, int scale, int shift, int bit_depth);     /* dquant[1] */
UAVS3E_CUDA_API void uavs3e_cuda_dquant_wq(int16_t *coef, int16_t *coef_out, uint8_t *wq_matrix[2], int log2_w, int log2_h, int scale, int shift, int bit_depth);  /* dquant[0] */
/* trans_dct2[log2w-1][log2h-1] (src/transform.c:253-412) and itrans_dct2[log2h-1][log2w-1] (src/com_itdq.c:264-423) */
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w4_h4(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w4_h8(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w4_h16(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w4_h32(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w8_h4(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w8_h8(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w8_h16(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w8_h32(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w8_h64(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w16_h4(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w16_h8(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w16_h16(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w16_h32(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w16_h64(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w32_h4(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w32_h8(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w32_h16(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w32_h32(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w32_h64(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w64_h8(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w64_h16(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w64_h32(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_trans_dct2_w64_h64(int16_t *src, int16_t *dst, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h4_w4(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h8_w4(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h16_w4(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h32_w4(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h4_w8(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h8_w8(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h16_w8(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h32_w8(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h64_w8(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h4_w16(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h8_w16(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h16_w16(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h32_w16(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h64_w16(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h4_w32(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h8_w32(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h16_w32(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h32_w32(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h64_w32(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h8_w64(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h16_w64(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h32_w64(int16_t *coef, int16_t *resi, int bit_depth);
UAVS3E_CUDA_API void uavs3e_cuda_itrans_dct2_h64_w64(int16_t *coef, int16_t *resi, int bit_depth);
/* trans_dct8_dst7[0 DCT8 / 1 DST7][log2n-1] (src/transform.c:416-671), itrans_dct8_dst7 (src/com_itdq.c:428-653) */
UAVS3E_CUDA_API void uavs3e_cuda_tx_dct8_4(int16_t *src, int16_t *dst, int shift, int line);
UAVS3E_CUDA_API void uavs3e_cuda_tx_dct8_8(int16_t *src, int16_t *dst, int shift, int line);
UAVS3E_CUDA_API void uavs3e_cuda_tx_dct8_16(int16_t *src, int16_t *dst, int shift, int line);
UAVS3E_CUDA_API void uavs3e_cuda_tx_dct8_32(int16_t *src, int16_t *dst, int shift, int line);
UAVS3E_CUDA_API void uavs3e_cuda_tx_dct8_64(int16_t *src, int16_t *dst, int shift, int line);
UAVS3E_CUDA_API void uavs3e_cuda_tx_dst7_4(int16_t *src, int16_t *dst, int shift, int line);
UAVS3E_CUDA_API void uavs3e_cuda_tx_dst7_8(int16_t *src, int16_t *dst, int shift, int line);
UAVS3E_CUDA_API void uavs3e_cuda_tx_dst7_16(int16_t *src, int16_t *dst, int shift, int line);
UAVS3E_CUDA_API void uavs3e_cuda_tx_dst7_32(int16_t *src, int16_t *dst, int shift, int line);
UAVS3E_CUDA_API void uavs3e_cuda_tx_dst7_64(int16_t *src, int16_t *dst, int shift, int line);
UAVS3E_CUDA_API void uavs3e_cuda_itx_dct8_4(int16_t *coeff, int16_t *block, int shift, int line, int max_tr_val, int min_tr_val);
UAVS3E_CUDA_API void uavs3e_cuda_itx_dct8_8(int16_t *coeff, int16_t *block, int shift, int line, int max_tr_val, int min_tr_val);
UAVS3E_CUDA_API void uavs3e_cuda_itx_dct8_16(int16_t *coeff, int16_t *block, int shift, int line, int max_tr_val, int min_tr_val);
UAVS3E_CUDA_API void uavs3e_cuda_itx_dct8_32(int16_t *coeff, int16_t *block, int shift, int line, int max_tr_val, int min_tr_val);
UAVS3E_CUDA_API void uavs3e_cuda_itx_dct8_64(int16_t *coeff, int16_t *block, int shift, int line, int max_tr_val, int min_tr_val);
UAVS3E_CUDA_API void uavs3e_cuda_itx_dst7_4(int16_t *coeff, int16_t *block, int shift, int line, int max_tr_val, int min_tr_val);
UAVS3E_CUDA_API void uavs3e_cuda_itx_dst7_8(int16_t *coeff, int16_t *block, int shift, int line, int max_tr_val, int min_tr_val);
UAVS3E_CUDA_API void uavs3e_cuda_itx_dst7_16(int16_t *coeff, int16_t *block, int shift, int line, int max_tr_val, int min_tr_val);
UAVS3E_CUDA_API void uavs3e_cuda_itx_dst7_32(int16_t *coeff, int16_t *block, int shift, int line, int max_tr_val, int min_tr_val);
UAVS3E_CUDA_API void uavs3e_cuda_itx_dst7_64(int16_t *coeff, int16_t *block, int shift, int line, int max_tr_val, int min_tr_val);

/* ---- costs: cost_sad / _x3 / _x4 / cost_ssd [log2w-2], cost_satd[log2w-2][log2h-2], src/com_cost.c:40-710 */
UAVS3E_CUDA_API uint32_t uavs3e_cuda_cost_sad_4(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred, int height);
UAVS3E_CUDA_API uint32_t uavs3e_cuda_cost_sad_8(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred, int height);
UAVS3E_CUDA_API uint32_t uavs3e_cuda_cost_sad_16(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred, int height);
UAVS3E_CUDA_API uint32_t uavs3e_cuda_cost_sad_32(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred, int height);
UAVS3E_CUDA_API uint32_t uavs3e_cuda_cost_sad_64(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred, int height);
UAVS3E_CUDA_API uint32_t uavs3e_cuda_cost_sad_128(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred, int height);
UAVS3E_CUDA_API void uavs3e_cuda_cost_sad_x3_4(uint8_t *p_org, int i_org, uint8_t *pred0, uint8_t *pred1, uint8_t *pred2, int i_pred, uint32_t sad[3], int height);
UAVS3E_CUDA_API void uavs3e_cuda_cost_sad_x3_8(uint8_t *p_org, int i_org, uint8_t *pred0, uint8_t *pred1, uint8_t *pred2, int i_pred, uint32_t sad[3], int height);
UAVS3E_CUDA_API void uavs3e_cuda_cost_sad_x3_16(uint8_t *p_org, int i_org, uint8_t *pred0, uint8_t *pred1, uint8_t *pred2, int i_pred, uint32_t sad[3], int height);
UAVS3E_CUDA_API void uavs3e_cuda_cost_sad_x3_32(uint8_t *p_org, int i_org, uint8_t *pred0, uint8_t *pred1, uint8_t *pred2, int i_pred, uint32_t sad[3], int height);
UAVS3E_CUDA_API void uavs3e_cuda_cost_sad_x3_64(uint8_t *p_org, int i_org, uint8_t *pred0, uint8_t *pred1, uint8_t *pred2, int i_pred, uint32_t sad[3], int height);
UAVS3E_CUDA_API void uavs3e_cuda_cost_sad_x3_128(uint8_t *p_org, int i_org, uint8_t *pred0, uint8_t *pred1, uint8_t *pred2, int i_pred, uint32_t sad[3], int height);
UAVS3E_CUDA_API void uavs3e_cuda_cost_sad_x4_4(uint8_t *p_org, int i_org, uint8_t *pred0, uint8_t *pred1, uint8_t *pred2, uint8_t *pred3, int i_pred, uint32_t sad[4], int height);
UAVS3E_CUDA_API void uavs3e_cuda_cost_sad_x4_8(uint8_t *p_org, int i_org, uint8_t *pred0, uint8_t *pred1, uint8_t *pred2, uint8_t *pred3, int i_pred, uint32_t sad[4], int height);
UAVS3E_CUDA_API void uavs3e_cuda_cost_sad_x4_16(uint8_t *p_org, int i_org, uint8_t *pred0, uint8_t *pred1, uint8_t *pred2, uint8_t *pred3, int i_pred, uint32_t sad[4], int height);
UAVS3E_CUDA_API void uavs3e_cuda_cost_sad_x4_32(uint8_t *p_org, int i_org, uint8_t *pred0, uint8_t *pred1, uint8_t *pred2, uint8_t *pred3, int i_pred, uint32_t sad[4], int height);
UAVS3E_CUDA_API void uavs3e_cuda_cost_sad_x4_64(uint8_t *p_org, int i_org, uint8_t *pred0, uint8_t *pred1, uint8_t *pred2, uint8_t *pred3, int i_pred, uint32_t sad[4], int height);
UAVS3E_CUDA_API void uavs3e_cuda_cost_sad_x4_128(uint8_t *p_org, int i_org, uint8_t *pred0, uint8_t *pred1, uint8_t *pred2, uint8_t *pred3, int i_pred, uint32_t sad[4], int height);
UAVS3E_CUDA_API uint64_t uavs3e_cuda_cost_ssd_4(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred, int height);
UAVS3E_CUDA_API uint64_t uavs3e_cuda_cost_ssd_8(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred, int height);
UAVS3E_CUDA_API uint64_t uavs3e_cuda_cost_ssd_16(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred, int height);
UAVS3E_CUDA_API uint64_t uavs3e_cuda_cost_ssd_32(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred, int height);
UAVS3E_CUDA_API uint64_t uavs3e_cuda_cost_ssd_64(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred, int height);
UAVS3E_CUDA_API uint64_t uavs3e_cuda_cost_ssd_128(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred, int height);
UAVS3E_CUDA_API uint32_t uavs3e_cuda_cost_satd_4x4(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred);
UAVS3E_CUDA_API uint32_t uavs3e_cuda_cost_satd_8x4(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred);
UAVS3E_CUDA_API uint32_t uavs3e_cuda_cost_satd_4x8(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred);
UAVS3E_CUDA_API uint32_t uavs3e_cuda_cost_satd_8x8(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred);
UAVS3E_CUDA_API uint32_t uavs3e_cuda_cost_satd_16x8(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred);
UAVS3E_CUDA_API uint32_t uavs3e_cuda_cost_satd_8x16(uint8_t *p_org, int i_org, uint8_t *p_pred, int i_pred);

/* ---- residual and bi-prediction average: pel_diff / pel_avrg [log2w-2], src/com_util.c:3068-3105 */
UAVS3E_CUDA_API void uavs3e_cuda_pel_diff_4(uint8_t *org, int i_org, uint8_t *pred, int i_pred, int16_t *resi, int i_resi, int height);
UAVS3E_CUDA_API void uavs3e_cuda_pel_diff_8(uint8_t *org, int i_org, uint8_t *pred, int i_pred, int16_t *resi, int i_resi, int height);
UAVS3E_CUDA_API void uavs3e_cuda_pel_diff_16(uint8_t *org, int i_org, uint8_t *pred, int i_pred, int16_t *resi, int i_resi, int height);
UAVS3E_CUDA_API void uavs3e_cuda_pel_diff_32(uint8_t *org, int i_org, uint8_t *pred, int i_pred, int16_t *resi, int i_resi, int height);
UAVS3E_CUDA_API void uavs3e_cuda_pel_diff_64(uint8_t *org, int i_org, uint8_t *pred, int i_pred, int16_t *resi, int i_resi, int height);
UAVS3E_CUDA_API void uavs3e_cuda_pel_diff_128(uint8_t *org, int i_org, uint8_t *pred, int i_pred, int16_t *resi, int i_resi, int height);
UAVS3E_CUDA_API void uavs3e_cuda_pel_avrg_4(uint8_t *dst, int i_dst, uint8_t *src1, uint8_t *src2, int height);
UAVS3E_CUDA_API void uavs3e_cuda_pel_avrg_8(uint8_t *dst, int i_dst, uint8_t *src1, uint8_t *src2, int height);
UAVS3E_CUDA_API void uavs3e_cuda_pel_avrg_16(uint8_t *dst, int i_dst, uint8_t *src1, uint8_t *src2, int height);
UAVS3E_CUDA_API void uavs3e_cuda_pel_avrg_32(uint8_t *dst, int i_dst, uint8_t *src1, uint8_t *src2, int height);
UAVS3E_CUDA_API void uavs3e_cuda_pel_avrg_64(uint8_t *dst, int i_dst, uint8_t *src1, uint8_t *src2, int height);
UAVS3E_CUDA_API void uavs3e_cuda_pel_avrg_128(uint8_t *dst, int i_dst, uint8_t *src1, uint8_t *src2, int height);

/* ---- quantisation first pass: quant_rdoq / quant_check, src/com_itdq.c:910-954 */
UAVS3E_CUDA_API int uavs3e_cuda_quant_rdoq(int16_t *coef, int num, int q_value, int q_bits, int32_t err_scale, int precision_bits, uint32_t *abs_coef, int16_t *abs_level, int64_t *uncoded_err);
UAVS3E_CUDA_API int uavs3e_cuda_quant_check(int16_t *coef, int num, int threshold);

#ifdef __cplusplus
}
#endif
#endif
