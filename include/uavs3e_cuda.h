/*
 * uavs3e_cuda.h -- C ABI of libuavs3e_cuda, the GB300 (sm_103a) implementation of uavs3e's
 * mode-decision hot path (8-bit luma).
 *
 * Two layers:
 *   1. Batched entry points (this file): one call per frame does the work the encoder's
 *      search loops would otherwise ask for one block at a time -- frame interpolation,
 *      the full motion-search cost table, the intra/transform lattice, the lookahead's
 *      per-picture cost estimate.  Inputs and outputs
 *      are plain pointers and sizes; "d_" pointers are device memory, others host memory.
 *   2. Kernel-table entries (uavs3e_cuda_table.h): functions with the exact C signatures of
 *      the reference's function-pointer table funs_handle_t (inc/com_util.h:278-341), and an
 *      installer that writes them into a caller's table.
 *
 * Types: the reference's pel/s16/u32/u64 (inc/com_api.h:48, inc/com_system.h) are written
 * here as uint8_t/int16_t/uint32_t/uint64_t, which is the same ABI for an 8-bit build.
 *
 * Errors: every int-returning call returns 0 or a negative UAVS3E_CUDA_ERR_* code, and the
 * first failure is also kept as a sticky status (uavs3e_cuda_status).  The library never
 * computes on the CPU: without a usable GPU the calls fail.
 */
#ifndef UAVS3E_CUDA_H
#define UAVS3E_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define UAVS3E_CUDA_API __declspec(dllexport)
#else
#define UAVS3E_CUDA_API __attribute__((visibility("default")))
#endif

#define UAVS3E_CUDA_OK                 0
#define UAVS3E_CUDA_ERR_ARG         (-101)   /* mirrors COM_ERR_INVALID_ARGUMENT, inc/com_api.h:61 */
#define UAVS3E_CUDA_ERR_MEMORY      (-102)   /* mirrors COM_ERR_OUT_OF_MEMORY */
#define UAVS3E_CUDA_ERR_UNSUPPORTED (-103)   /* mirrors COM_ERR_UNSUPPORTED */
#define UAVS3E_CUDA_ERR_CUDA        (-110)   /* a CUDA runtime call failed */
#define UAVS3E_CUDA_ERR_NOT_INIT    (-111)   /* no device selected / no GPU */
#define UAVS3E_CUDA_ERR_TIMEOUT     (-112)   /* a bounded device wait gave up */

/* ------------------------------------------------------------------ library state */

/* Select the CUDA device used by this process and upload constant tables.  Must be called
 * before the first other call (kernel-table entries call it lazily with device 0). */
UAVS3E_CUDA_API int uavs3e_cuda_init(int device);

/* First error since the last clear (0 if none), its text, and reset. */
UAVS3E_CUDA_API int uavs3e_cuda_status(void);
UAVS3E_CUDA_API const char *uavs3e_cuda_status_string(void);
UAVS3E_CUDA_API void uavs3e_cuda_clear_status(void);

/* Library version string. */
UAVS3E_CUDA_API const char *uavs3e_cuda_version(void);

/* Kernel timing (observability; the reference has none): while enabled, every launch of the
 * batched kernels is bracketed by CUDA events on its stream.  collect() waits for them and
 * returns, per kernel id (0 pad, 1 frame interpolation, 2 integer search, 3 fractional
 * refinement, 4 intra lattice, 5 lookahead estimate, 6 TZ requests, 7 CU motion compensation,
 * 8 RDOQ, 9 affine motion search), the summed milliseconds and launch counts,
 * then forgets them. */
UAVS3E_CUDA_API void uavs3e_cuda_profile_enable(int on);
/* Measured issue rate of the 4-sample SAD instruction (vabsdiff4 with accumulate) on the current
 * device: operations per second and per clock per SM.  The integer motion search's roofline
 * denominator (about 1.3 ms of GPU time). */
UAVS3E_CUDA_API int uavs3e_cuda_measure_sad4_rate(double *ops_per_s, double *ops_per_clk_sm);
/* The same for the 2-way halfword-by-byte dot product (dp2a), which carries the intra lattice's
 * transforms (2 multiply-adds per instruction). */
UAVS3E_CUDA_API int uavs3e_cuda_measure_dp2a_rate(double *ops_per_s, double *ops_per_clk_sm);

/* Number of kernels this library has launched in this process. */
UAVS3E_CUDA_API unsigned long long uavs3e_cuda_launch_count(void);
UAVS3E_CUDA_API int uavs3e_cuda_profile_collect(double ms[], int counts[], int n);

/* ------------------------------------------------------------ frame interpolation */

/*
 * The 15 quarter-sample luma planes of a padded reference picture, identical to
 * com_if_luma_frame (src/com_mc.c:760-800) followed by its padding of each plane
 * (com_img_padding(img, 1, 4), src/com_util.c:148).  Replaces the per-frame call of the
 * ip_flt_y_hor / ip_flt_y_ver / ip_flt_y_ver_ext entries (inc/com_util.h:304-306).
 *   d_plane0   : device pointer to sample (0,0) of the integer plane, padded by >= pad
 *                (pad >= 8) with its edges replicated (com_img_padding(img, 3, 0));
 *   d_planes   : 15 device pointers to sample (0,0) of the output planes, index
 *                dy*4 + dx - 1 for quarter-sample phase (dx, dy); every sample of the padded
 *                plane [-pad, width+pad) x [-pad, height+pad) is written;
 *   stride     : samples per row of all 16 planes;
 *   stream     : cudaStream_t (NULL = legacy default stream); the call does not synchronise.
 */
UAVS3E_CUDA_API int uavs3e_cuda_subpel_planes(const uint8_t *d_plane0, uint8_t *const d_planes[15], int width,
                                              int height, int pad, int stride, void *stream);

/* Replicate the edge samples of a picture into its padding (com_img_padding with ext 0,
 * src/com_util.c:148, one luma plane). */
UAVS3E_CUDA_API int uavs3e_cuda_pad_plane(uint8_t *d_plane0, int width, int height, int pad, int stride, void *stream);

/* ------------------------------------------------------------ batched motion search */

/*
 * A motion-search session holds, resident in HBM, the reference pictures (integer plane plus
 * the 15 fractional planes each) and the search tables of one picture size.  One call per
 * frame computes, for every block of the ten shapes 8x8, 16x8, 8x16, 16x16, 32x16, 16x32,
 * 32x32, 64x32, 32x64, 64x64 on the 64x64 CTU grid and every reference:
 *   - the integer full search over [-range, range]^2 (range <= 64; clipped as
 *     get_max_search_range, src/me.c:502-527, with is_padding = 1), cost
 *     (SAD << 16) + (mvbits(4dx) + mvbits(4dy)) * lambda_mv, predictor (0,0), first minimum
 *     in raster order (dy outer, dx inner) -- the costs the encoder's search_raster /
 *     search_diamond (src/me.c:103-355) evaluate with cost_sad;
 *   - the quarter-sample refinement of me_sub_pel_search (src/me.c:366-500) with the SATD
 *     cost (com_had): centre, 8 half-sample, then 8 quarter-sample neighbours.
 * Results are indexed [ctu][block][ref], ctu in raster order of the CTU grid, block as
 * uavs3e_cuda_me_block_table; blocks that do not fit inside the picture have cost fields
 * set to UINT64_MAX.
 */
typedef struct uavs3e_cuda_me uavs3e_cuda_me;

typedef struct {
    int16_t  mv_int[2];   /* best integer MV (integer samples)                    */
    int16_t  mv_sub[2];   /* best MV after refinement (quarter samples)           */
    uint32_t sad_int;     /* SAD at mv_int                                        */
    uint32_t satd_sub;    /* com_had SATD at mv_sub                               */
    uint64_t cost_int;    /* (sad_int << 16) + mvbits * lambda_mv                 */
    uint64_t cost_sub;    /* (satd_sub << 16) + mvbits * lambda_mv                */
} uavs3e_cuda_me_result_t;

/* (x, y, w, h) inside the CTU of the 169 blocks, in result order */
UAVS3E_CUDA_API int uavs3e_cuda_me_block_table(int out[169][4]);

/* pad: reference padding in samples (>= 144, the encoder's PIC_PAD_SIZE_L); n_refs <= 4 */
UAVS3E_CUDA_API uavs3e_cuda_me *uavs3e_cuda_me_open(int width, int height, int n_refs, int range, int pad);
UAVS3E_CUDA_API void uavs3e_cuda_me_close(uavs3e_cuda_me *me);
UAVS3E_CUDA_API int uavs3e_cuda_me_num_results(const uavs3e_cuda_me *me);

/* Make picture `plane` (host, width x height, row stride in samples) reference `slot`:
 * upload, pad and interpolate it on the GPU.  The hook point in the encoder is the
 * per-reference com_if_luma_frame call (src/uavs3e.c:1088). */
UAVS3E_CUDA_API int uavs3e_cuda_me_set_ref(uavs3e_cuda_me *me, int slot, const uint8_t *plane, int stride);
/* same from a device picture, enqueued on `stream` */
UAVS3E_CUDA_API int uavs3e_cuda_me_set_ref_device(uavs3e_cuda_me *me, int slot, const uint8_t *d_plane, int stride,
                                                  void *stream);

/* Search one frame: host org in, host results out (num_results records); synchronous. */
UAVS3E_CUDA_API int uavs3e_cuda_me_run(uavs3e_cuda_me *me, const uint8_t *org, int i_org, uint32_t lambda_mv,
                                       uavs3e_cuda_me_result_t *out);
/* Search one frame from device org into device results, enqueued on `stream`. */
UAVS3E_CUDA_API int uavs3e_cuda_me_run_device(uavs3e_cuda_me *me, const uint8_t *d_org, int i_org,
                                              uint32_t lambda_mv, uavs3e_cuda_me_result_t *d_out, void *stream);

/* One call per frame from host buffers: reference `slot` becomes `ref` (as uavs3e_cuda_me_set_ref)
 * and the frame `org` is searched (as uavs3e_cuda_me_run), the work replayed as the session's
 * captured graph (uavs3e_cuda_me_frame_graph) with one synchronisation at the end. */
UAVS3E_CUDA_API int uavs3e_cuda_me_frame(uavs3e_cuda_me *me, int slot, const uint8_t *ref, int i_ref,
                                         const uint8_t *org, int i_org, uint32_t lambda_mv,
                                         uavs3e_cuda_me_result_t *out);
/* One frame as a CUDA graph: refresh reference `slot` from the device picture d_ref (stride
 * i_src; padding and the 15 quarter-sample planes) and search d_org into d_out -- the launches of
 * uavs3e_cuda_me_set_ref_device + uavs3e_cuda_me_run_device, captured once per distinct set of
 * arguments (up to 32 kept, least recently used dropped; all dropped when lambda_mv changes the
 * search tables) and replayed with one graph launch on `stream`.  The first call with a new set
 * synchronises the session's stream to capture. */
UAVS3E_CUDA_API int uavs3e_cuda_me_frame_graph(uavs3e_cuda_me *me, int slot, const uint8_t *d_ref, int i_src,
                                               const uint8_t *d_org, int i_org, uint32_t lambda_mv,
                                               uavs3e_cuda_me_result_t *d_out, void *stream);

/*
 * The same search without any allocation -- no cudaMalloc/cudaFree, no allocating library call,
 * and no host heap while kernel timing (uavs3e_cuda_profile_enable) is off.  It has no counterpart in the reference; it exists for callers that cannot
 * allocate when they search a frame (an encoder thread working inside a fixed memory budget set
 * up at start-up, or code that must not call cudaMalloc/cudaFree because they synchronise the
 * device).  The caller passes every buffer: d_org (W x H, row stride i_org), d_planes
 * (n_refs * 16 device pointers to sample (0,0) of each reference's planes, index
 * ref*16 + dy*4 + dx, 0 = integer plane; padded by `pad` >= 144 with stride i_ref, e.g. filled
 * by uavs3e_cuda_pad_plane + uavs3e_cuda_subpel_planes) and d_out (uavs3e_cuda_me_block_table
 * order, (W+63)/64 * (H+63)/64 * 169 * n_refs records).  The scratch lives in one static device
 * array of UAVS3E_CUDA_NOALLOC_SCRATCH_BYTES (about 38 MB: the search's keys, refinement sums and
 * tables, and the byte-shifted reference copies its windows are staged from) that every GPU
 * loading this library holds until the process exits; frames beyond UAVS3E_CUDA_NOALLOC_MAX_CTUS
 * CTUs or the padded area of 1920x1088, more than UAVS3E_CUDA_NOALLOC_MAX_REFS references or a
 * range above UAVS3E_CUDA_NOALLOC_MAX_RANGE are rejected with UAVS3E_CUDA_ERR_ARG.  The call runs on the device uavs3e_cuda_init selected
 * (device 0 if none): the caller's current device must be that device and the buffers must live
 * on it, else UAVS3E_CUDA_ERR_ARG.  The first call looks up the array's device address; with lazy
 * module loading (the CUDA default) that lookup is also when the array is created on the device,
 * so make the first call at start-up, inside the budget it is meant for, and before any stream
 * capture.  Every call with a new size, range or lambda uploads search tables and waits for that
 * upload.  All calls share
 * the one array and the call leaves its contents behind: calls whose GPU work overlaps (other
 * streams, other host threads) race and must be serialised by the caller.
 */
#define UAVS3E_CUDA_NOALLOC_MAX_CTUS      510
#define UAVS3E_CUDA_NOALLOC_MAX_REFS      2
#define UAVS3E_CUDA_NOALLOC_MAX_RANGE     64
#define UAVS3E_CUDA_NOALLOC_SCRATCH_BYTES 38449408u
UAVS3E_CUDA_API int uavs3e_cuda_me_search_noalloc(const uint8_t *d_org, int i_org, const uint8_t *const *d_planes,
                                                  int i_ref, int pad, int width, int height, int n_refs, int range,
                                                  uint32_t lambda_mv, uavs3e_cuda_me_result_t *d_out, void *stream);

/* ------------------------------------------------------------ per-call TZ motion search */

/*
 * me_search_tz (src/me.c:529-568, declared inc/analyze.h:60) for a list of independent calls,
 * each with the inter_search_t state it reads: integer search (search_diamond :199, and for
 * uni-prediction search_raster :103 + a refinement diamond), the fractional refinement of
 * me_sub_pel_search (:366) at quarter/half resolution, every AMVR resolution (curr_mvr 0..4),
 * bi-prediction (the org replaced by 2 org - the other list's prediction, create_bi_org
 * src/inter.c:55).  Each result equals that call of the reference: the MV it writes, the integer
 * MV it stores in pi->mv_ipel (uni), and its return value.
 */
#define UAVS3E_CUDA_TZ_SAD             1   /* flags: pi->subpel_cost_type = 1 (SAD refinement) */
#define UAVS3E_CUDA_TZ_ADAPTIVE_RANGE  2   /* flags: pi->adaptive_raster_range                 */
#define UAVS3E_CUDA_TZ_MAX_SLOTS       8

typedef struct {
    int16_t  x, y;            /* block position (luma samples)                                 */
    uint8_t  w, h;            /* block size, 4..64 (powers of two)                             */
    uint8_t  ref_slot;        /* planes of pi->ref_pic                                         */
    int8_t   refi;            /* reference index in its list (raster step, reference bits)     */
    uint8_t  num_refp;        /* pi->num_refp                                                  */
    uint8_t  mvr;             /* pi->curr_mvr 0..4                                             */
    uint8_t  bi;              /* the bi argument                                               */
    uint8_t  flags;           /* UAVS3E_CUDA_TZ_*                                              */
    int16_t  mvp[2];          /* predictor, quarter samples, a multiple of 1 << mvr            */
    int16_t  mv[2];           /* bi: start MV (pi->mv_scale), quarter samples, same grid        */
    int16_t  mv_ipel[2];      /* pi->mv_ipel[lidx][refi] (adaptive raster range), samples      */
    int16_t  other_mv[2];     /* bi: the other list's MV, quarter samples                      */
    uint8_t  other_slot;      /* bi: planes of the other list's reference                      */
    uint8_t  pad0[3];
    int32_t  mot_bits_other;  /* bi: pi->mot_bits of the other list                            */
    uint32_t lambda_mv;       /* pi->lambda_mv                                                 */
    int32_t  dist;            /* |pi->ptr - ref_pic->ptr|                                      */
    int32_t  pad1;
} uavs3e_cuda_tz_req_t;

typedef struct {
    int16_t  mv[2];           /* the MV the call writes (quarter samples)                      */
    int16_t  mv_ipel[2];      /* pi->mv_ipel[lidx][refi] after the call                        */
    uint64_t cost;            /* return value; UINT64_MAX when the MV range is empty or the    */
                              /* request is outside the supported domain (MVs left unchanged)  */
} uavs3e_cuda_tz_out_t;

/* picture-level inter_search_t fields (inter_search_init, src/inter.c:2015) */
typedef struct { int width, height, is_padding, max_search_range, gop_size; } uavs3e_cuda_tz_pic_t;

/* Requests against a motion-search session's references (slot = session slot), host buffers,
 * synchronous: org is the current picture (row stride i_org). */
UAVS3E_CUDA_API int uavs3e_cuda_me_tz(uavs3e_cuda_me *me, const uavs3e_cuda_tz_pic_t *pic, const uint8_t *org,
                                      int i_org, const uavs3e_cuda_tz_req_t *reqs, int n, uavs3e_cuda_tz_out_t *out);
/* Device form: d_planes is a host array of n_slots * 16 device pointers (slot-major, phase
 * dy*4 + dx, 0 = integer plane) to sample (0,0) of planes padded by pad >= 144 with stride i_ref
 * (a multiple of 4); max_search_range <= 1024. */
UAVS3E_CUDA_API int uavs3e_cuda_me_tz_device(const uavs3e_cuda_tz_pic_t *pic, const uint8_t *d_org, int i_org,
                                             const uint8_t *const *d_planes, int n_slots, int i_ref, int pad,
                                             const uavs3e_cuda_tz_req_t *d_reqs, int n, uavs3e_cuda_tz_out_t *d_out,
                                             void *stream);

/* ------------------------------------------------------------ CU motion compensation */

/*
 * com_mc_cu (src/com_mc.c:140-200, declared inc/com_modules.h:71) for a list of CUs: the luma
 * prediction copied from the reference's quarter-sample plane (com_mc_blk_luma), the chroma
 * predictions by the 4-tap filters at eighth-sample positions (com_mc_blk_chroma: ipcpy,
 * ipflt H_4 / V_4, ipflt_ext EXT_4), the two lists averaged (pel_avrg).  Each CU's prediction
 * is written at out + out_offset: Y (w x h) then U and V (w/2 x h/2), for the channels asked.
 */
#define UAVS3E_CUDA_MC_LUMA_CHROMA 0   /* channel_type_t CHANNEL_LC */
#define UAVS3E_CUDA_MC_LUMA        1   /* CHANNEL_L */
#define UAVS3E_CUDA_MC_CHROMA      2   /* CHANNEL_C */

typedef struct {
    int16_t  x, y;            /* CU position (luma samples), CU inside the picture             */
    uint8_t  w, h;            /* 8..64, powers of two                                          */
    int8_t   slot[2];         /* reference slot of list 0 / 1 (refi), -1 = list not used       */
    int16_t  mv[2][2];        /* quarter-sample MVs                                            */
    uint8_t  channel;         /* UAVS3E_CUDA_MC_*                                              */
    uint8_t  pad[3];
    uint32_t out_offset;      /* byte offset of this CU's prediction                           */
} uavs3e_cuda_mc_req_t;

/* Chroma planes of reference `slot` of a motion-search session (host, W/2 x H/2, stride in
 * samples): uploaded and padded by 72 samples (PIC_PAD_SIZE_C) with the edges replicated. */
UAVS3E_CUDA_API int uavs3e_cuda_me_set_ref_chroma(uavs3e_cuda_me *me, int slot, const uint8_t *u, const uint8_t *v,
                                                  int stride);
/* CU predictions from the session's references (luma planes and chroma planes), host buffers,
 * synchronous; out holds out_bytes (CUs whose prediction would not fit are skipped). */
UAVS3E_CUDA_API int uavs3e_cuda_mc_cu(uavs3e_cuda_me *me, const uavs3e_cuda_mc_req_t *reqs, int n, uint8_t *out,
                                      size_t out_bytes);
/* Device form: d_planes = n_slots * 16 luma plane pointers (as uavs3e_cuda_me_tz_device, padded by
 * pad >= 144), d_chroma = n_slots * 2 pointers to sample (0,0) of U and V (stride i_c, padded by
 * pad_c >= 72); host pointer arrays of device pointers. */
UAVS3E_CUDA_API int uavs3e_cuda_mc_cu_device(int width, int height, const uint8_t *const *d_planes, int n_slots,
                                             int i_ref, int pad, const uint8_t *const *d_chroma, int i_c, int pad_c,
                                             const uavs3e_cuda_mc_req_t *d_reqs, int n, uint8_t *d_out,
                                             size_t out_bytes, void *stream);

/*
 * Affine CUs: com_mc_cu_affine (src/com_mc.c:361-422, declared inc/com_modules.h:72): each list's
 * sub-block MVs from its 2 or 3 control-point MVs (4x4 sub-blocks, 8x8 with
 * affine_subblk_size_idx 1 or both lists), luma by the 16-phase 8-tap filters of the integer
 * plane, chroma 4x4 blocks at the rounded mean MV of their four luma units by the 32-phase 4-tap
 * filters, the lists averaged.  Output Y (w x h), U, V (w/2 x h/2) at out + out_offset.
 */
typedef struct {
    int16_t  x, y;            /* CU position, CU inside the picture                            */
    uint8_t  w, h;            /* 16..64, powers of two                                         */
    int8_t   slot[2];         /* reference slot of list 0 / 1, -1 = unused                     */
    uint8_t  cp_num;          /* 2 or 3 control points                                         */
    uint8_t  sub8;            /* pichdr->affine_subblk_size_idx                                */
    uint8_t  pad[2];
    int32_t  cpmv[2][3][2];   /* control-point MVs per list, 1/16 samples                      */
    uint32_t out_offset;
} uavs3e_cuda_affine_req_t;

UAVS3E_CUDA_API int uavs3e_cuda_mc_affine(uavs3e_cuda_me *me, const uavs3e_cuda_affine_req_t *reqs, int n,
                                          uint8_t *out, size_t out_bytes);
UAVS3E_CUDA_API int uavs3e_cuda_mc_affine_device(int width, int height, const uint8_t *const *d_planes, int n_slots,
                                                 int i_ref, int pad, const uint8_t *const *d_chroma, int i_c,
                                                 int pad_c, const uavs3e_cuda_affine_req_t *d_reqs, int n,
                                                 uint8_t *d_out, size_t out_bytes, void *stream);

/* ------------------------------------------------------------ coefficient rate */

/*
 * lbac_enc_run_length_cc_rdo (src/entropy.c:1688-1950): the bits the encoder's RDO counts for a
 * transform block's levels, for a list of blocks each with the coder state it starts from -- the
 * range and its channel's context models (the luma or chroma half of lbac->h.run, run_rdoq,
 * level, last1, last2).  Each result holds the bits counted (the bitcounter increase), the range
 * and the models after the block, so the caller can go on from that state.  Levels are int16 in
 * raster order (w x h from coef_offset), e.g. the output of uavs3e_cuda_rdoq.  The blocks of one
 * call may repeat a level range (the same block from several coder states) but not overlap one
 * partially.
 */
typedef struct {
    int16_t run[12], run_rdoq[12], level[12], last1[6], last2[12];   /* chroma: last2[0..9] */
} uavs3e_cuda_coef_ctx_t;

typedef struct {
    uint32_t coef_offset;     /* first level of the block                                      */
    uint8_t  log2w, log2h;    /* 2..6 luma, 2..5 chroma                                        */
    uint8_t  ch_type;         /* 0 luma, 1 chroma                                              */
    uint8_t  pad;
    uint16_t num_sig;         /* non-zero levels of the block (>= 1)                           */
    uint16_t range;           /* coder range, 256..511                                         */
    uavs3e_cuda_coef_ctx_t ctx;
} uavs3e_cuda_coef_rate_req_t;

typedef struct {
    uint32_t bits;            /* bits counted; UINT32_MAX for a request outside the domain     */
    uint16_t range;           /* (invalid: num_sig above the block's non-zero levels, shapes,  */
    uint16_t pad;             /* ranges, models with a zero LPS range); state unchanged then   */
    uavs3e_cuda_coef_ctx_t ctx;
} uavs3e_cuda_coef_rate_out_t;

UAVS3E_CUDA_API int uavs3e_cuda_coef_rate(const uavs3e_cuda_coef_rate_req_t *reqs, int n, const int16_t *levels,
                                          size_t n_levels, uavs3e_cuda_coef_rate_out_t *out);
UAVS3E_CUDA_API int uavs3e_cuda_coef_rate_device(const uavs3e_cuda_coef_rate_req_t *d_reqs, int n,
                                                 const int16_t *d_levels, size_t n_levels,
                                                 uavs3e_cuda_coef_rate_out_t *d_out, void *stream);

/* ------------------------------------------------------------ affine motion search */

/*
 * affine_me_gradient (src/inter.c:1339-1470, file-local in the reference) for a list of
 * independent calls: up to 7 (uni) / 5 (bi) gradient steps of the 4-parameter affine model from
 * the start CPMVs, each step's CPMV change from the normal equations of the residual and the
 * Sobel gradients of the prediction (affine_sobel_flt_hor / _ver, affine_coef_computer,
 * solve_equal in double precision), rounded to the AMVR step, kept when SATD + MV cost drops.
 * Flags add what the callers do around the call:
 *   UAVS3E_CUDA_AFFME_UNI_START: the start CPMVs of analyze_affine_uni (:1607-1647), the cheaper
 *     of the MVP and pi->best_mv_uni (req mv[0], quarter samples) clipped by mv_clip and scaled;
 *   UAVS3E_CUDA_AFFME_BI: the org of analyze_affine_bi (:1730-1790), 2 org - the other list's
 *     prediction (8x8 sub-blocks), the call with bi = 1 and 8x8 sub-blocks;
 *   UAVS3E_CUDA_AFFME_SUB8: pichdr->affine_subblk_size_idx > 0 (8x8 sub-blocks in uni calls).
 * Results equal the reference's: the CPMVs left in mv, the return value, and the callers' cost
 * (return value + MV_COST of affine_mv_bits, + pi->mot_bits of the other list for bi).
 * The reference asserts that mvp and the start CPMVs lie on the AMVR step's grid.
 */
#define UAVS3E_CUDA_AFFME_BI        1
#define UAVS3E_CUDA_AFFME_UNI_START 2
#define UAVS3E_CUDA_AFFME_SUB8      4

typedef struct {
    int16_t  x, y;            /* CU position (luma samples), CU inside the picture             */
    uint8_t  w, h;            /* 16..64, powers of two                                         */
    uint8_t  ref_slot;        /* planes of pi->ref_pic (only the integer plane is read)        */
    int8_t   refi;            /* reference index, < num_refp (reference bits)                  */
    uint8_t  num_refp;        /* pi->num_refp                                                  */
    uint8_t  mvr;             /* pi->curr_mvr 0..2: CPMV step 1/4, 1, 1/16 sample              */
    uint8_t  flags;           /* UAVS3E_CUDA_AFFME_*                                           */
    uint8_t  other_slot;      /* bi: planes of the other list's reference                      */
    uint32_t lambda_mv;       /* pi->lambda_mv                                                 */
    int32_t  mot_bits_other;  /* bi: pi->mot_bits of the other list                            */
    int32_t  pad;
    int32_t  mvp[2][2];       /* affine MVP of the two control points, 1/16 samples            */
    int32_t  mv[2][2];        /* start CPMVs; UNI_START: mv[0] = pi->best_mv_uni (1/4 samples) */
    int32_t  other_mv[2][2];  /* bi: the other list's CPMVs                                    */
} uavs3e_cuda_affme_req_t;

typedef struct {
    int32_t  mv[2][2];        /* the CPMVs the call leaves in mv                               */
    uint32_t satd;            /* return value (com_had of the best prediction, >> bi)          */
    int32_t  bits;            /* affine_mv_bits of the result (+ mot_bits_other for bi)        */
    uint64_t cost;            /* satd + MV_COST(bits); UINT64_MAX for a request outside the    */
                              /* supported domain (sides 16..64, CU inside the picture,        */
                              /* CPMVs within 18 bits), mv = the start CPMVs                   */
} uavs3e_cuda_affme_out_t;

/* Requests against a motion-search session's references (slot = session slot), host buffers,
 * synchronous: org is the current picture (row stride i_org). */
UAVS3E_CUDA_API int uavs3e_cuda_me_affine(uavs3e_cuda_me *me, const uint8_t *org, int i_org,
                                          const uavs3e_cuda_affme_req_t *reqs, int n, uavs3e_cuda_affme_out_t *out);
/* Device form: d_planes as uavs3e_cuda_me_tz_device (n_slots * 16 pointers, padded by >= 144). */
UAVS3E_CUDA_API int uavs3e_cuda_me_affine_device(int width, int height, const uint8_t *d_org, int i_org,
                                                 const uint8_t *const *d_planes, int n_slots, int i_ref, int pad,
                                                 const uavs3e_cuda_affme_req_t *d_reqs, int n,
                                                 uavs3e_cuda_affme_out_t *d_out, void *stream);

/* Affine control-point MVP (com_get_affine_mvp_scaling, src/com_util.c:1983-2058, with
 * scaling_mv1 src/com_util.c:322 and com_mv_rounding_s32 inc/com_util.h:189) for lists of CUs:
 * the top-left predictor from neighbours A, B, D and the top-right one from G, C (the first with
 * a valid reference index in list lidx, its MV scaled by the POC distances; zero when none),
 * taken to 1/16 sample, rounded to the affine AMVR resolution and clipped to 18 bits.
 * The motion field has the encoder's layout: map_mv s16 [rows * i_scu][2 lists][2], map_refi s8
 * [rows * i_scu][2], stride i_scu = pic_width_in_scu + 2, the picture's SCU (0, 0) at index
 * i_scu + 1 (one border row above, one border column on each side).  ref_ptr[n_ref][2] holds the
 * POC of refp[i][list]. */
typedef struct {
    int32_t scup;       /* y_scu * i_scu + x_scu of the CU's top-left SCU */
    int16_t cu_width;   /* luma samples */
    int8_t lidx;        /* list 0 / 1 */
    int8_t cur_refi;    /* the CU's reference index in list lidx */
    int8_t mvr;         /* affine AMVR index: 0, 1, 2 (1/4, 1, 1/16 sample) */
    int8_t pad[3];
} uavs3e_cuda_affmvp_req_t;

typedef struct {
    int32_t mvp[2][2];  /* (x, y) of the top-left and top-right control points, 1/16 samples */
} uavs3e_cuda_affmvp_out_t;

/* Host buffers, synchronous.  Requests outside the domain (a neighbour outside the field, a
 * reference index >= n_ref, a zero POC distance, mvr > 2, lidx > 1) get zero predictors and make
 * the call return UAVS3E_CUDA_ERR_ARG after all results are written. */
UAVS3E_CUDA_API int uavs3e_cuda_affine_mvp(int64_t ptr, const int64_t *ref_ptr, int n_ref, const int16_t *map_mv,
                                           const int8_t *map_refi, int i_scu, int rows,
                                           const uavs3e_cuda_affmvp_req_t *reqs, int n,
                                           uavs3e_cuda_affmvp_out_t *out);
/* Device buffers on `stream`; d_err (optional, device int32) gains the number of requests outside
 * the domain. */
UAVS3E_CUDA_API int uavs3e_cuda_affine_mvp_device(int64_t ptr, const int64_t *d_ref_ptr, int n_ref,
                                                  const int16_t *d_map_mv, const int8_t *d_map_refi, int i_scu,
                                                  int rows, const uavs3e_cuda_affmvp_req_t *d_reqs, int n,
                                                  uavs3e_cuda_affmvp_out_t *d_out, int32_t *d_err, void *stream);

/* Affine merge candidates (com_get_affine_merge_candidate, src/com_util.c:1761-1981, with
 * com_derive_affine_model_mv :1566, com_derive_affine_constructed_candidate :1656,
 * get_colocal_scup :303, get_col_mv / get_col_mv_from_list0 :977-1000, scaling_mv1 :322) for lists
 * of CUs: up to 2 candidates inherited from affine neighbours (F, G, C, A, D; the neighbour CU's
 * corner MVs extrapolated to the CU, 4-parameter across a CTU row boundary), then the
 * constructed ones from the control points LT (A, B, D), RT (G, C), LB (F) and the colocated
 * RB (scaled by POC distances) in the reference's 6 model orders, zero-padded to 5.  The maps
 * have the motion field's layout of uavs3e_cuda_affine_mvp (stride i_scu, SCU (0, 0) at index
 * i_scu + 1): map_mv s16 [rows * i_scu][2][2], map_refi s8 [rows * i_scu][2], map_scu u8 (the
 * encoder's com_scu_t byte: bit 0 coded, bit 1 intra, bits 4-5 affine), map_pos u32 (the covering
 * CU's top-left SCU << 6 | log2 height << 3 | log2 width); col_mv / col_refi are the colocated
 * picture's (refp[0][REFP_1] in B slices, refp[0][REFP_0] otherwise) in the same layout. */
typedef struct {
    int64_t ptr;                /* POC of the current picture                                  */
    int64_t ref0_ptr[2];        /* POC of refp[0][REFP_0] and refp[0][REFP_1]                   */
    int64_t col_list_ptr[17];   /* the colocated picture's list_ptr (its list-0 reference POCs)  */
    int32_t i_scu, pic_width_in_scu, pic_height_in_scu, rows;
    int32_t slice_type;         /* 3 = SLICE_B (colocated in list 1, both lists scaled), else P */
    int32_t log2_max_cuwh;
} uavs3e_cuda_affmrg_pic_t;

typedef struct {
    int32_t scup;               /* y_scu * i_scu + x_scu of the CU's top-left SCU               */
    int16_t cu_width, cu_height; /* luma samples, powers of two 16..128                          */
} uavs3e_cuda_affmrg_req_t;

typedef struct {
    int32_t num;                /* candidates derived before the zero padding                   */
    int8_t  cp_num[5];          /* control points of each candidate, 2 or 3                     */
    int8_t  refi[5][2];         /* reference index per list, -1 unused                          */
    int8_t  pad;
    int32_t cpmv[5][2][3][2];   /* control-point MVs, 1/16 samples; vertices past cp_num are 0  */
} uavs3e_cuda_affmrg_out_t;

/* Host buffers, synchronous; returns UAVS3E_CUDA_ERR_ARG when a request falls outside the domain
 * (a map read outside the field, sizes, a colocated reference index >= 17, a zero POC distance):
 * its result is zeroed, the others are valid. */
UAVS3E_CUDA_API int uavs3e_cuda_affine_merge(const uavs3e_cuda_affmrg_pic_t *pic, const int16_t *map_mv,
                                             const int8_t *map_refi, const uint8_t *map_scu,
                                             const uint32_t *map_pos, const int16_t *col_mv, const int8_t *col_refi,
                                             const uavs3e_cuda_affmrg_req_t *reqs, int n,
                                             uavs3e_cuda_affmrg_out_t *out);
/* Device buffers on a stream, no synchronisation; d_err (optional) counts the requests outside
 * the domain. */
UAVS3E_CUDA_API int uavs3e_cuda_affine_merge_device(const uavs3e_cuda_affmrg_pic_t *pic, const int16_t *d_map_mv,
                                                    const int8_t *d_map_refi, const uint8_t *d_map_scu,
                                                    const uint32_t *d_map_pos, const int16_t *d_col_mv,
                                                    const int8_t *d_col_refi, const uavs3e_cuda_affmrg_req_t *d_reqs,
                                                    int n, uavs3e_cuda_affmrg_out_t *d_out, int32_t *d_err,
                                                    void *stream);

/* Device pointer to sample (0,0) of plane `phase` (dy*4 + dx, 0 = integer) of `slot`, and the
 * session's plane stride; for inspection by tests. */
UAVS3E_CUDA_API const uint8_t *uavs3e_cuda_me_plane(uavs3e_cuda_me *me, int slot, int phase);
UAVS3E_CUDA_API int uavs3e_cuda_me_plane_stride(const uavs3e_cuda_me *me);
/* Device pointer to sample (0,0) of chroma plane c (0 U, 1 V) of `slot` (NULL before the first
 * uavs3e_cuda_me_set_ref_chroma), and the chroma stride (0 before it). */
UAVS3E_CUDA_API const uint8_t *uavs3e_cuda_me_chroma_plane(uavs3e_cuda_me *me, int slot, int c);
UAVS3E_CUDA_API int uavs3e_cuda_me_chroma_stride(const uavs3e_cuda_me *me);

/* ------------------------------------------------------------ batched intra lattice */

/*
 * Intra mode decision lattice.  For every CU and every luma intra mode 0..32 this computes what
 * the encoder's intra search evaluates per candidate: the neighbour array of the CU read from
 * `rec` (com_intra_get_nbr, src/com_ipred.c:40, with every in-picture sample outside the CU
 * treated as reconstructed), the prediction (com_intra_pred, :733, IPF on or off), its SATD
 * (calc_satd_intra, src/util.c:200), the forward DCT2 of the residual (trans_dct2,
 * src/transform.c:253-412) and, for each QP, the first RDOQ pass (quant_check + quant_rdoq,
 * src/com_itdq.c:910-954, parameters of rdoq_quant_block src/quant.c:196-231; the context-
 * dependent second pass stays with the CPU), dequantisation (com_dquant :807), inverse DCT2
 * (itrans_dct2 :264-423) and reconstruction (com_recon src/com_util.c:3107).
 *   satd[cu*33 + mode]; q[(cu*33 + mode)*n_qp + qp_index]  (n_qp <= 4)
 * CU sides are powers of two in 4..64, positions multiples of 4 (the encoder's 4x4 grid), CUs
 * inside the picture (others yield zeroed records).
 */
typedef struct { int16_t x, y; uint8_t w, h; uint16_t pad; } uavs3e_cuda_cu_t;

typedef struct {
    uint32_t ssd;         /* SSD(org, reconstruction)                                  */
    uint32_t coef_hash;   /* sum of level * ((pos * 0x9E3779B1 + 0x7F4A7C15) | 1), mod 2^32 */
    uint16_t num_nz;      /* non-zero levels                                           */
    int16_t  last_nz;     /* last non-zero level in zig-zag scan order, -1 if none     */
    uint32_t sum_abs;     /* sum of |level|                                            */
} uavs3e_cuda_lat_q_t;

/* The lattice of a call is one persistent launch walking a device queue of tiles (a tile =
 * several whole CUs of one shape, or one CU and a chunk of its modes), largest shapes first,
 * with no wait on the host between its launches: once the layouts are tuned, a call can be
 * captured into a CUDA graph.  Layout autotuning (on by default): the first call with QPs per
 * device and mode count times, for every shape with at least 512 CUs, the tile layouts given by
 * shared-memory budgets of 16..48 KB on the queue restricted to that shape and keeps the
 * fastest (that call waits for the GPU; make it before any capture); records are the same for
 * every layout.  budgets: per shape (log2 w - 2) * 5 + (log2 h - 2), in bytes, 0 = the default
 * 48 KB (not tuned). */
UAVS3E_CUDA_API void uavs3e_cuda_lattice_autotune(int on);
UAVS3E_CUDA_API int uavs3e_cuda_lattice_budgets(int n_modes, int out[25]);

/* Per-stage SM cycles of the lattice tiles since the last call with clear != 0, as
 * out[25 shape classes][10 stages] (summed over CTAs; thread 0 of a CTA reads clock64 at each
 * CTA barrier of a tile).  Only a library built with UAVS3E_LAT_STAGE_CLOCKS keeps them
 * (python -m uavs3e_gb300.lattice_stages builds one); otherwise UAVS3E_CUDA_ERR_UNSUPPORTED. */
UAVS3E_CUDA_API int uavs3e_cuda_lattice_stage_clocks(unsigned long long *out, int clear);

/*
 * Intra mode candidates: make_ipred_list (src/intra.c:226-367, file-local) for a list of
 * prediction blocks, each with the SATD of its 33 modes taken from row satd_row of an array laid
 * out as the lattice's satd records (satd[row * 33 + mode], e.g. uavs3e_cuda_intra_lattice's
 * satd output with row = CU index) and with the coder state the encoder holds in
 * core->lbac_bakup: the bits of each mode are lbac_enc_intra_dir (src/entropy.c:2118) in
 * counting mode from that range and those intra_dir context models.  Output: ipred_list[0..4] and
 * the return value (the number of candidates the RDO takes), as the reference leaves them.
 */
typedef struct {
    uint32_t satd_row;        /* row of the SATD array                                         */
    uint8_t  pb_w, pb_h;      /* prediction block, 4..64 (powers of two)                       */
    uint8_t  mpm[2];          /* cur_info->mpm[part_idx], 0..33 (33 = IPD_IPCM)                */
    uint8_t  skip_ipd;        /* the skip_ipd argument (no DC / planar / bilinear)             */
    uint8_t  fast;            /* info->intra_fast_rmd                                          */
    uint16_t range;           /* core->lbac_bakup.range, 256..511                              */
    int16_t  ctx[7];          /* core->lbac_bakup.h.intra_dir[0..6] (non-zero LPS probability) */
    uint8_t  pad[6];
    double   sqrt_lambda;     /* core->sqrt_lambda[0], >= 0                                    */
    uint64_t inter_satd;      /* core->inter_satd (UINT64_MAX: none)                           */
    double   satd_threshold;  /* core->satd_threshold                                          */
} uavs3e_cuda_rmd_req_t;

typedef struct {
    int8_t   list[5];         /* ipred_list[0..4] (-1: empty)                                  */
    uint8_t  count;           /* return value; 255 for a request outside the supported domain  */
    uint8_t  pad[2];
} uavs3e_cuda_rmd_out_t;

/* Host buffers, synchronous: satd has n_rows * 33 entries. */
UAVS3E_CUDA_API int uavs3e_cuda_intra_rmd(const uint32_t *satd, size_t n_rows, const uavs3e_cuda_rmd_req_t *reqs,
                                          int n, uavs3e_cuda_rmd_out_t *out);
UAVS3E_CUDA_API int uavs3e_cuda_intra_rmd_device(const uint32_t *d_satd, size_t n_rows,
                                                 const uavs3e_cuda_rmd_req_t *d_reqs, int n,
                                                 uavs3e_cuda_rmd_out_t *d_out, void *stream);

/* The 23-shape lattice (w, h in 4..64, aspect <= 8, largest first) of a picture: writes up to
 * cap records to out (may be NULL) and returns the total count. */
UAVS3E_CUDA_API int uavs3e_cuda_lattice_cus(int width, int height, uavs3e_cuda_cu_t *out, int cap);

/* device buffers in and out, enqueued on `stream`; qps is a host array.  n_qp = 0 writes the SATD
 * records only (no transform stage; d_q may be NULL): the input of uavs3e_cuda_intra_rmd. */
UAVS3E_CUDA_API int uavs3e_cuda_intra_lattice_device(const uint8_t *d_org, int i_org, const uint8_t *d_rec, int i_rec,
                                                     int width, int height, const uavs3e_cuda_cu_t *d_cus, int n_cus,
                                                     int ipf, const int *qps, int n_qp, int is_intra_slice,
                                                     uint32_t *d_satd, uavs3e_cuda_lat_q_t *d_q, void *stream);
/* Host buffers in and out (org / rec with their own strides, cus, satd[n_cus * 33],
 * q[n_cus * 33 * n_qp]), synchronous: the inputs are copied to device buffers the library keeps
 * per device, the lattice runs on a stream of its own, the records are copied back.  Calls on
 * one device are serialised. */
UAVS3E_CUDA_API int uavs3e_cuda_intra_lattice(const uint8_t *org, int i_org, const uint8_t *rec, int i_rec, int width,
                                              int height, const uavs3e_cuda_cu_t *cus, int n_cus, int ipf,
                                              const int *qps, int n_qp, int is_intra_slice, uint32_t *satd,
                                              uavs3e_cuda_lat_q_t *q);
/* The same over a subset of modes: d_modes holds n_modes mode indices (0..32) per CU
 * ([n_cus][n_modes], device); only those (CU, mode) records are written.  Used by the pruned
 * search, which evaluates a shortlist of modes per CU. */
UAVS3E_CUDA_API int uavs3e_cuda_intra_lattice_modes_device(const uint8_t *d_org, int i_org, const uint8_t *d_rec,
                                                           int i_rec, int width, int height,
                                                           const uavs3e_cuda_cu_t *d_cus, int n_cus,
                                                           const uint8_t *d_modes, int n_modes, int ipf,
                                                           const int *qps, int n_qp, int is_intra_slice,
                                                           uint32_t *d_satd, uavs3e_cuda_lat_q_t *d_q, void *stream);

/* ------------------------------------------------------------ lookahead cost estimation */

/*
 * loka_estimate_coding_cost (src/lookahead.c:82-293, declared inc/lookahead.h:51) for a whole
 * picture: for every 16x16 unit (raster order over (width/16) x (height/16)) and every
 * reference, the integer search of me_search_tz (src/me.c:529-568) with the estimate's
 * settings (integer resolution, predictor (0,0), lambda of QP 32, no bi-prediction search),
 * the com_had SATD of the block it finds, the SATD of the two bi-prediction averages, the 11
 * intra modes predicted from the original picture (get_ipred_neighbor, src/lookahead.c:40),
 * the chroma SATD with the best intra mode and the unit's cost_var energy.
 *   cfg        : what the reference reads from inter_search_t and the pictures: size,
 *                is_padding (1 = the encoder's picture-level search, src/uavs3e.c:185/929, whose
 *                references are padded by PIC_PAD_SIZE_L = 144; 0 = the lookahead's scene-cut
 *                estimate, src/uavs3e.c:1326/1257, whose MVs keep the unit inside the picture),
 *                max_search_range (SEARCH_RANGE_IPEL_LD 64 or _RA 384), gop_size, the reference
 *                counts per list (<= 4) and the POCs of the picture and its references;
 *   org planes : the picture's Y (W x H) and U, V (W/2 x H/2) planes;
 *   references : luma planes, pointers to sample (0,0), stride i_ref, padded by ref_pad samples
 *                (>= 144 when is_padding; the host entry reads no padding otherwise, the device
 *                entry wants >= 4 readable samples around the picture and a stride that is a
 *                multiple of 4).
 */
#define UAVS3E_CUDA_LOKA_MAX_REFS 4

typedef struct {
    int     width, height;
    int     is_padding;
    int     max_search_range;
    int     gop_size;
    int     num_ref[2];
    int64_t ptr;
    int64_t ref_ptr[2][UAVS3E_CUDA_LOKA_MAX_REFS];
} uavs3e_cuda_loka_cfg_t;

typedef struct {
    int16_t  mv[2][UAVS3E_CUDA_LOKA_MAX_REFS][2];   /* integer MV per list / reference      */
    uint32_t satd[2][UAVS3E_CUDA_LOKA_MAX_REFS];    /* com_had at that MV                   */
    uint32_t bi_satd;     /* average of the two list winners (pictures with both lists)       */
    uint32_t zero_satd;   /* average of the (0,0) blocks of ref_l0[0] and ref_l1[0]           */
    uint32_t min_cost;    /* smallest inter or intra cost: the unit's share of picture_satd   */
    uint32_t min_icost;   /* smallest intra cost                                              */
    uint32_t icost_u, icost_v;
    uint64_t energy;      /* cost_var of Y 16x16 + U 8x8 + V 8x8                              */
    uint8_t  best_mode, pad[7];
} uavs3e_cuda_loka_unit_t;

/* The whole call on host buffers, synchronous.  Writes the return value of
 * loka_estimate_coding_cost to *cost and, where the pointers are not NULL, icost, icost_uv[2],
 * map_dqp[units] (the reference's outputs) and the unit records. */
UAVS3E_CUDA_API int uavs3e_cuda_loka_estimate(const uavs3e_cuda_loka_cfg_t *cfg, const uint8_t *org_y, int i_org,
                                              const uint8_t *org_u, const uint8_t *org_v, int i_org_c,
                                              const uint8_t *const *ref_l0, const uint8_t *const *ref_l1, int i_ref,
                                              int ref_pad, double *cost, double *icost, double icost_uv[2],
                                              float *map_dqp, uavs3e_cuda_loka_unit_t *units);
/* loka_get_sc_ratio (src/lookahead.c:378-386): the estimate against the previous picture
 * alone, P cost / intra cost. */
UAVS3E_CUDA_API int uavs3e_cuda_loka_sc_ratio(int width, int height, int is_padding, int max_search_range,
                                              int gop_size, int64_t ptr, const uint8_t *org_y, int i_org,
                                              const uint8_t *org_u, const uint8_t *org_v, int i_org_c,
                                              const uint8_t *last_y, int64_t last_ptr, int i_last, int last_pad,
                                              double *ratio);
/* Device buffers in and out, enqueued on `stream`: d_units[units], d_energy[units] (the energies
 * again, contiguous), d_totals[5] = sums of min_cost, min_icost, icost_u, icost_v and the number
 * of 16x16 SADs the searches evaluated.  ref pointer arrays are host arrays of device pointers. */
UAVS3E_CUDA_API int uavs3e_cuda_loka_units_device(const uavs3e_cuda_loka_cfg_t *cfg, const uint8_t *d_org_y,
                                                  int i_org, const uint8_t *d_org_u, const uint8_t *d_org_v,
                                                  int i_org_c, const uint8_t *const *d_ref_l0,
                                                  const uint8_t *const *d_ref_l1, int i_ref, int ref_pad,
                                                  uavs3e_cuda_loka_unit_t *d_units, uint64_t *d_energy,
                                                  uint64_t *d_totals, void *stream);
/* The reference's picture-level results from the totals (host copy) and, for map_dqp, the
 * energies (host copy): returns the picture cost. */
UAVS3E_CUDA_API double uavs3e_cuda_loka_finish(const uavs3e_cuda_loka_cfg_t *cfg, const uint64_t totals[4],
                                               const uint64_t *energy, double *icost, double icost_uv[2],
                                               float *map_dqp);

/* ------------------------------------------------------------ RDOQ of transform blocks */

/*
 * quant_non_zero with flat quantisation (src/quant.c:315-383, declared inc/modules.h:62) ->
 * rdoq_quant_block (:196-313) for a list of transform blocks: coefficients past 32 columns / rows
 * zeroed, quant_check, the first pass (quant_rdoq) and the rate-distortion decision of each level
 * and of the last position with the bin costs the encoder derived from its entropy-coder state
 * (core_t rdoq_bin_est_*, inc/define.h:335-339, rdoq_init_cu_est_bits :139).  The levels are
 * written over each block's coefficients as the reference writes them (blocks whose coefficients
 * stay below the quant_check threshold keep them), num_nz[i] is the call's return value.
 */
typedef struct {
    int32_t ctp[2];
    int32_t cbf[3][2];
    int32_t run[24][2];
    int32_t lvl[24][2];
    int32_t lst[2][6][12][2];
} uavs3e_cuda_rdoq_est_t;

typedef struct {
    uint32_t coef_offset;    /* first coefficient of the w x h block (raster)                  */
    uint8_t  log2w, log2h;   /* 2..6                                                           */
    uint8_t  qp;             /* quantisation step index 0..79                                  */
    uint8_t  is_intra;
    uint8_t  ch_type;        /* 0 Y, 1 U, 2 V                                                  */
    uint8_t  slice_type;     /* SLICE_I = 1 selects the intra dead zone                        */
    uint16_t est;            /* index of the estimate set                                      */
    uint32_t pad;
    int64_t  lambda;         /* (int64_t)(d_lambda * 32768 + 0.5), as rdoq_quant_block forms it */
} uavs3e_cuda_rdoq_req_t;

/* host buffers, synchronous; num_nz[i] = -1 marks a request outside the domain (untouched) */
UAVS3E_CUDA_API int uavs3e_cuda_rdoq(const uavs3e_cuda_rdoq_req_t *reqs, int n, const uavs3e_cuda_rdoq_est_t *ests,
                                     int n_est, int16_t *coefs, size_t n_coefs, int32_t *num_nz);
UAVS3E_CUDA_API int uavs3e_cuda_rdoq_device(const uavs3e_cuda_rdoq_req_t *d_reqs, int n,
                                            const uavs3e_cuda_rdoq_est_t *d_ests, int n_est, int16_t *d_coefs,
                                            size_t n_coefs, int32_t *d_num_nz, void *stream);

/* quant_non_zero's weighted branch (pichdr->pic_wq_enable, src/quant.c:335-380) for the same
 * requests (lambda and est not used): the zero-out past 32, then plain quantisation with the
 * weights of core->wq[0] (wq4, 16, for 4x4 blocks) and core->wq[1] (wq8, 64, the others; weights
 * >= 1).  Levels over the coefficients, num_nz[i] per block (-1 outside the domain). */
UAVS3E_CUDA_API int uavs3e_cuda_quant_wq(const uavs3e_cuda_rdoq_req_t *reqs, int n, const uint8_t *wq4,
                                         const uint8_t *wq8, int16_t *coefs, size_t n_coefs, int32_t *num_nz);
UAVS3E_CUDA_API int uavs3e_cuda_quant_wq_device(const uavs3e_cuda_rdoq_req_t *d_reqs, int n, const uint8_t *d_wq4,
                                                const uint8_t *d_wq8, int16_t *d_coefs, size_t n_coefs,
                                                int32_t *d_num_nz, void *stream);

/* ---------------------------------------------------------------------------------------
 * Learned CU-partition / intra-mode pruning network (no counterpart in the reference: the
 * learned part stands beside the bit-exact path and never changes it).  Implicit-GEMM
 * convolutions on the 5th-generation tensor cores (tcgen05.mma, bf16 operands, FP32
 * accumulation in tensor memory); all pointers are device memory.  Activations NHWC bf16;
 * weights [Cout][Kp] bf16 (k = (ky * ks + kx) * Cin + ci, Kp = ks*ks*Cin rounded up to 16);
 * biases, gradients and Adam state FP32.  Shapes: Cin even (a multiple of 16 for dgrad), Cout a
 * multiple of 16 up to 64, batch x output pixels a multiple of 16, ks 1 or 3 (padding ks/2),
 * stride 1 or 2, fewer than 2^31 elements per activation tensor.  The activation, weight and
 * output tensors start on 16-byte boundaries (they are read and written 8 channels at a time);
 * UC_ERR_ARG otherwise. */

/* y = act(conv(x, w) + bias): y bf16, or FP32 when y_f32; relu 0/1. */
UAVS3E_CUDA_API int uavs3e_cuda_cnn_conv_fwd(const void *x, const void *w, const float *bias, void *y, int y_f32,
                                             int batch, int hin, int win, int cin, int cout, int ks, int stride,
                                             int kp, int relu, void *stream);
/* dx = (x > 0) * conv^T(dy, w): the gradient at the previous layer's pre-activation, bf16.
 * wt_scratch is not used (the weights are read in place) and may be NULL. */
UAVS3E_CUDA_API int uavs3e_cuda_cnn_conv_dgrad(const void *dy, const void *w, const void *x, void *dx, void *wt_scratch,
                                               int batch, int hin, int win, int cin, int cout, int ks, int stride,
                                               int kp, void *stream);
/* dw = dy^T x_col [cout][kp], db = sum dy (both overwritten). */
UAVS3E_CUDA_API int uavs3e_cuda_cnn_conv_wgrad(const void *dy, const void *x, float *dw, float *db, int batch, int hin,
                                               int win, int cin, int cout, int ks, int stride, int kp, void *stream);
/* Number of tensor-core convolution CTAs that gave up waiting for their MMAs (a bounded wait;
 * their outputs were left unwritten) since the previous call; 0 in normal operation. */
UAVS3E_CUDA_API int uavs3e_cuda_cnn_timeouts(void);
/* Network input of n CTUs at (ctu_xy[2i], ctu_xy[2i+1]) of a picture: [n][64][64][2] bf16. */
UAVS3E_CUDA_API int uavs3e_cuda_cnn_input(const uint8_t *d_pic, int stride, int width, int height,
                                          const int *d_ctu_xy, int n, int qp, void *x0, void *stream);
/* Head losses (BCE on the split flags, cross-entropy on the modes) of [batch][16][48] logits
 * against [batch][40] labels; dlogits bf16 scaled by 1/batch, loss[4] = per-part means. */
UAVS3E_CUDA_API int uavs3e_cuda_cnn_head_loss(const float *logits, const uint8_t *labels, int batch, void *dlogits,
                                              float *loss, void *stream);
/* One Adam step (step >= 1) on n FP32 weights; refreshes the bf16 copy when w_bf16 != NULL. */
UAVS3E_CUDA_API int uavs3e_cuda_cnn_adam(float *w, float *m, float *v, const float *g, void *w_bf16, int n, float lr,
                                         float b1, float b2, float eps, int step, void *stream);

#ifdef __cplusplus
}
#endif
#endif
