"""ctypes bindings of the CPU oracles (test infrastructure only).

``Oracle``  wraps ``_build/liboracle.so`` (the C restatement, oracle.c); it builds on any host.
``RefLib``  wraps ``_ref/libuavs3e_ref.so`` (the reference encoder compiled from its own sources
            by ``make -C oracle ref``); it exists only where the reference sources are present.

Both expose the same Python methods with numpy arguments, so a parity test can run one case
through either oracle library and through the GPU library.  Nothing in the product imports this.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libuavs3e_ref.so")
NEIB = 576

P = C.c_void_p
I = C.c_int


def ptr(a):
    return C.c_void_p(a.ctypes.data)


def build_oracle():
    subprocess.run(["make", "-C", HERE, "-s"], check=True)


def build_ref(ref_dir=None):
    """builds oracle/_ref from the uavs3e source tree ref_dir (default: $UAVS3E_REF_TREE);
    False when no tree is given or found"""
    ref_dir = ref_dir or os.environ.get("UAVS3E_REF_TREE")
    if not ref_dir or not os.path.isdir(os.path.join(ref_dir, "src")):
        return False
    subprocess.run(["make", "-C", HERE, "-s", "-j8", "ref", "REF=" + ref_dir], check=True)
    return True


class _Common:
    """Methods with identical argument meaning on both libraries."""

    def sad(self, w, h, o, io, p, ip):
        raise NotImplementedError

    # helpers shared by both bindings -------------------------------------------------
    @staticmethod
    def _u8(a):
        return np.ascontiguousarray(a, dtype=np.uint8)


class Oracle(_Common):
    def __init__(self, path=ORACLE_SO):
        if not os.path.exists(path):
            build_oracle()
        L = C.CDLL(path)
        self.L = L
        L.orc_init()
        L.orc_sad.restype = C.c_uint32
        L.orc_ssd.restype = C.c_uint64
        L.orc_satd_tile.restype = C.c_uint32
        L.orc_had.restype = C.c_uint32
        L.orc_satd_intra.restype = C.c_uint32
        L.orc_quant_check.restype = I
        L.orc_quant_rdoq.restype = I
        L.orc_dct_table.restype = C.POINTER(C.c_int8)
        L.orc_scan.restype = C.POINTER(C.c_uint16)
        L.orc_rdoq_err_scale.restype = C.c_int32
        L.orc_dq_scale.restype = C.c_uint32
        L.orc_dq_shift.restype = C.c_uint32
        L.orc_quant_scale.restype = C.c_uint16
        L.orc_tbl_sqrt.restype = C.c_double
        L.orc_level_hash.restype = C.c_uint32

    # costs
    def sad(self, w, h, o, io, p, ip):
        return self.L.orc_sad(w, h, P(o), io, P(p), ip)

    def ssd(self, w, h, o, io, p, ip):
        return self.L.orc_ssd(w, h, P(o), io, P(p), ip)

    def satd_tile(self, tw, th, o, io, p, ip):
        return self.L.orc_satd_tile(tw, th, P(o), io, P(p), ip)

    def had(self, w, h, o, io, p, ip, bd=8):
        return self.L.orc_had(w, h, P(o), io, P(p), ip, bd)

    def satd_intra(self, w, h, o, p, io, ip, bd=8):
        return self.L.orc_satd_intra(w, h, P(o), P(p), io, ip, bd)

    # mc
    def ipflt(self, t, s, is_, d, id_, w, h, c, mx=255):
        self.L.orc_ipflt(t, P(s), is_, P(d), id_, w, h, ptr(c), mx)

    def ipflt_ext(self, t, s, is_, d, id_, w, h, cx, cy, mx=255):
        self.L.orc_ipflt_ext(t, P(s), is_, P(d), id_, w, h, ptr(cx), ptr(cy), mx)

    def ipcpy(self, s, is_, d, id_, w, h):
        self.L.orc_ipcpy(P(s), is_, P(d), id_, w, h)

    def if_luma_frame(self, plane0_ptr, plane_ptrs, W, H, pad, stride):
        arr = (C.c_void_p * 15)(*plane_ptrs)
        self.L.orc_if_luma_frame(P(plane0_ptr), arr, W, H, pad, stride)

    # pel
    def pel_diff(self, w, h, o, io, p, ip, r, ir):
        self.L.orc_pel_diff(w, h, P(o), io, P(p), ip, P(r), ir)

    def pel_avrg(self, w, h, d, id_, s1, s2):
        self.L.orc_pel_avrg(w, h, P(d), id_, P(s1), P(s2))

    def recon(self, resi, pred, ipred, w, h, rec, irec, cbf, bd=8):
        self.L.orc_recon(P(resi), P(pred), ipred, w, h, P(rec), irec, cbf, bd)

    # intra
    def intra_get_nbr(self, x, y, w, h, src, s_src, top, lcu, avail, nb, scup, coded, n_scu, i_scu, bd=8):
        self.L.orc_intra_get_nbr(x, y, w, h, P(src), s_src, P(top), lcu, avail, ptr(nb), scup, ptr(coded), i_scu, bd)

    def intra_pred(self, nb, dst, ipm, w, h, avail, ipf, bd=8):
        self.L.orc_intra_pred(ptr(nb), ptr(dst), ipm, w, h, bd, avail, ipf)

    def ipred_ang(self, nb, dst, i_dst, mode, w, h):
        self.L.orc_ipred_ang(ptr(nb), ptr(dst), i_dst, mode, w, h)

    # transforms
    def trans_dct2(self, lw, lh, src, dst, bd=8):
        self.L.orc_trans_dct2(lw, lh, ptr(src), ptr(dst), bd)

    def trans_dct8_dst7(self, t, ln, src, dst, shift, line):
        self.L.orc_trans_dct8_dst7(t, ln, ptr(src), ptr(dst), shift, line)

    def transform(self, nxn, blk, coef, resi, lw, lh, bd=8, sec=0, alt4=0):
        self.L.orc_transform(nxn, blk, ptr(coef), ptr(resi), lw, lh, bd, sec, alt4)

    def itrans_dct2(self, lh, lw, coef, resi, bd=8):
        self.L.orc_itrans_dct2(lh, lw, ptr(coef), ptr(resi), bd)

    def itrans_dct8_dst7(self, t, ln, coef, blk, shift, line, mx, mn):
        self.L.orc_itrans_dct8_dst7(t, ln, ptr(coef), ptr(blk), shift, line, mx, mn)

    def dquant(self, flat, coef, out, wq4, wq8, lw, lh, scale, shift, bd=8):
        self.L.orc_dquant(flat, ptr(coef), ptr(out), ptr(wq4), ptr(wq8), lw, lh, scale, shift, bd)

    def invqt(self, nxn, blk, coef, resi, wq4, wq8, lw, lh, qp, bd=8, sec=0, alt4=0):
        w4 = None if wq4 is None else ptr(wq4)
        w8 = None if wq8 is None else ptr(wq8)
        self.L.orc_invqt(nxn, blk, ptr(coef), ptr(resi), w4, w8, lw, lh, qp, bd, sec, alt4)

    def quant_check(self, coef, num, thr):
        return self.L.orc_quant_check(ptr(coef), num, thr)

    def quant_rdoq(self, coef, num, qv, qb, es, pb, abs_coef, abs_level, err):
        return self.L.orc_quant_rdoq(ptr(coef), num, qv, qb, es, pb, ptr(abs_coef), ptr(abs_level), ptr(err))

    # tables
    def dct_table(self, ln):
        n = 1 << ln
        return np.ctypeslib.as_array(self.L.orc_dct_table(ln), shape=(3, n, n)).copy()

    def scan(self, lw, lh):
        return np.ctypeslib.as_array(self.L.orc_scan(lw, lh), shape=(1 << (lw + lh),)).copy()

    # batched workloads
    def me_frame(self, org, i_org, plane_ptrs, i_ref, W, H, n_refs, blocks, rng, lambda_mv, threads=1):
        """blocks: structured array of ME_BLOCK; returns structured array of ME_RESULT."""
        out = np.zeros(len(blocks) * n_refs, dtype=ME_RESULT)
        arr = (C.c_void_p * len(plane_ptrs))(*plane_ptrs)
        self.L.orc_me_frame(P(org), i_org, arr, i_ref, W, H, n_refs, ptr(blocks), len(blocks), rng,
                            C.c_uint32(lambda_mv), ptr(out), threads)
        return out

    def intra_lattice(self, org, i_org, rec, i_rec, W, H, cus, ipf, qps, is_intra=1, threads=1):
        qps = np.ascontiguousarray(qps, dtype=np.int32)
        satd = np.zeros(len(cus) * 33, dtype=np.uint32)
        q = np.zeros(len(cus) * 33 * len(qps), dtype=LAT_Q)
        self.L.orc_intra_lattice(P(org), i_org, P(rec), i_rec, W, H, ptr(cus), len(cus), ipf, ptr(qps),
                                 len(qps), is_intra, ptr(satd), ptr(q), threads)
        return satd, q

    def loka_units(self, cfg, org_y, i_org, org_u, org_v, i_org_c, ref_l0, ref_l1, i_ref, threads=1):
        """cfg: LOKA_CFG record; ref_l0/ref_l1: lists of sample-(0,0) addresses; returns LOKA_UNIT array"""
        cfg = np.ascontiguousarray(cfg, dtype=LOKA_CFG).reshape(1)
        n = (int(cfg["width"][0]) // 16) * (int(cfg["height"][0]) // 16)
        out = np.zeros(n, dtype=LOKA_UNIT)
        a0 = (C.c_void_p * 4)(*(list(ref_l0) + [None] * (4 - len(ref_l0))))
        a1 = (C.c_void_p * 4)(*(list(ref_l1) + [None] * (4 - len(ref_l1))))
        self.L.orc_loka_units(ptr(cfg), ptr(org_y), i_org, ptr(org_u), ptr(org_v), i_org_c, a0, a1, i_ref, ptr(out),
                              threads)
        return out

    def loka_estimate(self, cfg, org_y, i_org, org_u, org_v, i_org_c, ref_l0, ref_l1, i_ref, want_uv=True,
                      want_dqp=True, threads=1):
        """the same tuple as RefLib.loka_estimate, from loka_units + loka_finish"""
        units = self.loka_units(cfg, org_y, i_org, org_u, org_v, i_org_c, ref_l0, ref_l1, i_ref, threads)
        cost, icost, icost_uv, dqp = self.loka_finish(cfg, units)
        return cost, icost, icost_uv if want_uv else None, dqp if want_dqp else None

    def me_tz(self, pic, org, i_org, plane_ptrs, i_ref, reqs, threads=1):
        """per-call TZ searches: pic = (W, H, is_padding, max_search_range, gop_size); plane_ptrs =
        slot-major addresses of the 16 planes of each reference; reqs: TZ_REQ array -> TZ_OUT"""
        p = (C.c_int * 5)(*pic)
        arr = (C.c_void_p * len(plane_ptrs))(*plane_ptrs)
        reqs = np.ascontiguousarray(reqs, dtype=TZ_REQ)
        out = np.zeros(len(reqs), dtype=TZ_OUT)
        self.L.orc_me_tz(p, ptr(org), i_org, arr, i_ref, ptr(reqs), len(reqs), ptr(out), threads)
        return out

    def mc_cu(self, W, H, plane_ptrs, i_ref, chroma_ptrs, i_c, reqs, out_bytes):
        """com_mc_cu for every MC_REQ; returns the output buffer (uint8, out_bytes)"""
        arr = (C.c_void_p * len(plane_ptrs))(*plane_ptrs)
        carr = (C.c_void_p * len(chroma_ptrs))(*chroma_ptrs)
        reqs = np.ascontiguousarray(reqs, dtype=MC_REQ)
        out = np.zeros(max(1, out_bytes), dtype=np.uint8)
        self.L.orc_mc_cu(W, H, arr, i_ref, carr, i_c, ptr(reqs), len(reqs), ptr(out))
        return out[:out_bytes]

    def mc_affine(self, W, H, plane_ptrs, i_ref, chroma_ptrs, i_c, reqs, out_bytes):
        """com_mc_cu_affine for every AFFINE_REQ; returns the output buffer"""
        arr = (C.c_void_p * len(plane_ptrs))(*plane_ptrs)
        carr = (C.c_void_p * len(chroma_ptrs))(*chroma_ptrs)
        reqs = np.ascontiguousarray(reqs, dtype=AFFINE_REQ)
        out = np.zeros(max(1, out_bytes), dtype=np.uint8)
        self.L.orc_mc_affine(W, H, arr, i_ref, carr, i_c, ptr(reqs), len(reqs), ptr(out))
        return out[:out_bytes]

    def quant_wq(self, reqs, wq4, wq8, coefs):
        """quant_non_zero with weighted quantisation for every RDOQ_REQ; coefs updated, num_nz returned"""
        reqs = np.ascontiguousarray(reqs, dtype=RDOQ_REQ)
        wq4 = np.ascontiguousarray(wq4, dtype=np.uint8)
        wq8 = np.ascontiguousarray(wq8, dtype=np.uint8)
        nz = np.zeros(len(reqs), dtype=np.int32)
        self.L.orc_quant_wq(ptr(reqs), len(reqs), ptr(wq4), ptr(wq8), ptr(coefs), ptr(nz))
        return nz

    def affine_mvp(self, ptr_cur, ref_ptr, map_mv, map_refi, i_scu, reqs):
        """com_get_affine_mvp_scaling for every AFFMVP_REQ; map_mv int16 [rows * i_scu, 2, 2], map_refi
        int8 [rows * i_scu, 2] (SCU (0, 0) at index i_scu + 1), ref_ptr int64 [n_ref, 2].
        Returns (out, number of requests outside the domain)"""
        ref_ptr = np.ascontiguousarray(ref_ptr, dtype=np.int64)
        map_mv = np.ascontiguousarray(map_mv, dtype=np.int16)
        map_refi = np.ascontiguousarray(map_refi, dtype=np.int8)
        reqs = np.ascontiguousarray(reqs, dtype=AFFMVP_REQ)
        out = np.zeros(len(reqs), dtype=AFFMVP_OUT)
        rows = len(map_refi) // i_scu
        bad = self.L.orc_affine_mvp(C.c_int64(ptr_cur), ptr(ref_ptr), len(ref_ptr), ptr(map_mv), ptr(map_refi),
                                    i_scu, rows, ptr(reqs), len(reqs), ptr(out))
        return out, bad

    def affine_merge(self, pic, map_mv, map_refi, map_scu, map_pos, col_mv, col_refi, reqs):
        """com_get_affine_merge_candidate for every AFFMRG_REQ: pic an AFFMRG_PIC record, the maps in
        the reference's layout (SCU (0, 0) at index i_scu + 1): map_mv / col_mv int16 [rows * i_scu, 2,
        2], map_refi / col_refi int8 [rows * i_scu, 2], map_scu uint8, map_pos uint32 [rows * i_scu].
        Returns (out, number of requests outside the domain)"""
        pic = np.ascontiguousarray(pic, dtype=AFFMRG_PIC).reshape(1)
        arrs = [np.ascontiguousarray(a, dtype=t) for a, t in ((map_mv, np.int16), (map_refi, np.int8),
                                                               (map_scu, np.uint8), (map_pos, np.uint32),
                                                               (col_mv, np.int16), (col_refi, np.int8))]
        reqs = np.ascontiguousarray(reqs, dtype=AFFMRG_REQ)
        out = np.zeros(len(reqs), dtype=AFFMRG_OUT)
        bad = self.L.orc_affine_merge(ptr(pic), *[ptr(a) for a in arrs], ptr(reqs), len(reqs), ptr(out))
        return out, bad

    def coef_rate(self, levels, reqs):
        """lbac_enc_run_length_cc_rdo for every COEF_RATE_REQ on levels (int16)"""
        levels = np.ascontiguousarray(levels, dtype=np.int16)
        reqs = np.ascontiguousarray(reqs, dtype=COEF_RATE_REQ)
        out = np.zeros(len(reqs), dtype=COEF_RATE_OUT)
        self.L.orc_coef_rate(ptr(levels), ptr(reqs), len(reqs), ptr(out))
        return out

    def lbac_next(self, model, mps):
        return self.L.orc_lbac_next(int(model), int(mps))

    def intra_rmd(self, satd, reqs):
        """make_ipred_list for every RMD_REQ from the 33 SATDs of row satd_row of satd"""
        satd = np.ascontiguousarray(satd, dtype=np.uint32)
        reqs = np.ascontiguousarray(reqs, dtype=RMD_REQ)
        out = np.zeros(len(reqs), dtype=RMD_OUT)
        self.L.orc_intra_rmd(ptr(satd), ptr(reqs), len(reqs), ptr(out))
        return out

    def me_affine(self, W, H, org, i_org, plane_ptrs, i_ref, reqs, threads=1):
        """affine gradient searches (affine_me_gradient, with the uni start / bi org of its callers)
        for every AFFME_REQ; plane_ptrs as me_tz (only each slot's integer plane is read)"""
        arr = (C.c_void_p * len(plane_ptrs))(*plane_ptrs)
        reqs = np.ascontiguousarray(reqs, dtype=AFFME_REQ)
        out = np.zeros(len(reqs), dtype=AFFME_OUT)
        self.L.orc_me_affine(W, H, ptr(org), i_org, arr, i_ref, ptr(reqs), len(reqs), ptr(out), threads)
        return out

    def rdoq(self, reqs, ests, coefs):
        """quant_non_zero (flat) for every RDOQ_REQ; coefs (int16) is updated in place; returns num_nz"""
        reqs = np.ascontiguousarray(reqs, dtype=RDOQ_REQ)
        ests = np.ascontiguousarray(ests, dtype=RDOQ_EST)
        nz = np.zeros(len(reqs), dtype=np.int32)
        self.L.orc_rdoq(ptr(reqs), len(reqs), ptr(ests), ptr(coefs), ptr(nz))
        return nz

    def loka_finish(self, cfg, units):
        """(picture cost, icost, icost_uv[2], map_dqp) from the unit records"""
        cfg = np.ascontiguousarray(cfg, dtype=LOKA_CFG).reshape(1)
        icost = C.c_double()
        icost_uv = (C.c_double * 2)()
        dqp = np.zeros(len(units), dtype=np.float32)
        self.L.orc_loka_finish.restype = C.c_double
        cost = self.L.orc_loka_finish(ptr(cfg), ptr(units), C.byref(icost), icost_uv, ptr(dqp))
        return cost, icost.value, (icost_uv[0], icost_uv[1]), dqp


class RefLib(_Common):
    """The reference's own C kernels (through oracle/ref_glue.c)."""

    def __init__(self, path=REF_SO):
        L = C.CDLL(path)
        self.L = L
        L.refk_init()
        for n in ("refk_sad", "refk_satd", "refk_had", "refk_satd_intra"):
            getattr(L, n).restype = C.c_uint32
        L.refk_ssd.restype = C.c_uint64
        L.refk_quant_check.restype = I
        L.refk_quant_rdoq.restype = I
        L.refk_dct_table.restype = C.POINTER(C.c_int8)
        L.refk_scan.restype = C.POINTER(C.c_uint16)
        L.refk_tbl_sqrt.restype = C.c_double

    @staticmethod
    def widx(w):
        return int(w).bit_length() - 3

    def sad(self, w, h, o, io, p, ip):
        return self.L.refk_sad(self.widx(w), P(o), io, P(p), ip, h)

    def ssd(self, w, h, o, io, p, ip):
        return self.L.refk_ssd(self.widx(w), P(o), io, P(p), ip, h)

    def satd_tile(self, tw, th, o, io, p, ip):
        return self.L.refk_satd(tw.bit_length() - 3, th.bit_length() - 3, P(o), io, P(p), ip)

    def had(self, w, h, o, io, p, ip, bd=8):
        return self.L.refk_had(w, h, P(o), io, P(p), ip, bd)

    def satd_intra(self, w, h, o, p, io, ip, bd=8):
        return self.L.refk_satd_intra(w, h, P(o), P(p), io, ip, bd)

    def ipflt(self, t, s, is_, d, id_, w, h, c, mx=255):
        self.L.refk_ipflt(t, self.widx(w), P(s), is_, P(d), id_, w, h, ptr(c), mx)

    def ipflt_ext(self, t, s, is_, d, id_, w, h, cx, cy, mx=255):
        self.L.refk_ipflt_ext(t, self.widx(w), P(s), is_, P(d), id_, w, h, ptr(cx), ptr(cy), mx)

    def ipcpy(self, s, is_, d, id_, w, h):
        self.L.refk_ipcpy(self.widx(w), P(s), is_, P(d), id_, w, h)

    def if_luma_frame(self, plane0_ptr, plane_ptrs, W, H, pad, stride):
        arr = (C.c_void_p * 15)(*plane_ptrs)
        self.L.refk_if_luma_frame(P(plane0_ptr), arr, W, H, pad, stride)

    def pel_diff(self, w, h, o, io, p, ip, r, ir):
        self.L.refk_pel_diff(self.widx(w), P(o), io, P(p), ip, P(r), ir, h)

    def pel_avrg(self, w, h, d, id_, s1, s2):
        self.L.refk_pel_avrg(self.widx(w), P(d), id_, P(s1), P(s2), h)

    def recon(self, resi, pred, ipred, w, h, rec, irec, cbf, bd=8):
        self.L.refk_recon(self.widx(w), P(resi), P(pred), ipred, w, h, P(rec), irec, cbf, bd)

    def intra_get_nbr(self, x, y, w, h, src, s_src, top, lcu, avail, nb, scup, coded, n_scu, i_scu, bd=8):
        self.L.refk_intra_get_nbr(x, y, w, h, P(src), s_src, P(top), lcu, avail, ptr(nb), scup, ptr(coded),
                                  n_scu, i_scu, bd)

    def intra_pred(self, nb, dst, ipm, w, h, avail, ipf, bd=8):
        self.L.refk_intra_pred(ptr(nb), ptr(dst), ipm, w, h, bd, avail, ipf)

    def ipred_ang(self, nb, dst, i_dst, mode, w, h):
        self.L.refk_intra_ang_entry(mode, ptr(nb), ptr(dst), i_dst, mode, w, h)

    def trans_dct2(self, lw, lh, src, dst, bd=8):
        self.L.refk_trans_dct2(lw, lh, ptr(src), ptr(dst), bd)

    def trans_dct8_dst7(self, t, ln, src, dst, shift, line):
        self.L.refk_trans_dct8_dst7(t, ln, ptr(src), ptr(dst), shift, line)

    def transform(self, nxn, blk, coef, resi, lw, lh, bd=8, sec=0, alt4=0):
        self.L.refk_transform(nxn, blk, ptr(coef), ptr(resi), lw, lh, bd, sec, alt4)

    def itrans_dct2(self, lh, lw, coef, resi, bd=8):
        self.L.refk_itrans_dct2(lh, lw, ptr(coef), ptr(resi), bd)

    def itrans_dct8_dst7(self, t, ln, coef, blk, shift, line, mx, mn):
        self.L.refk_itrans_dct8_dst7(t, ln, ptr(coef), ptr(blk), shift, line, mx, mn)

    def dquant(self, flat, coef, out, wq4, wq8, lw, lh, scale, shift, bd=8):
        self.L.refk_dquant(flat, ptr(coef), ptr(out), ptr(wq4), ptr(wq8), lw, lh, scale, shift, bd)

    def invqt(self, nxn, blk, coef, resi, wq4, wq8, lw, lh, qp, bd=8, sec=0, alt4=0):
        w4 = None if wq4 is None else ptr(wq4)
        w8 = None if wq8 is None else ptr(wq8)
        self.L.refk_invqt(nxn, blk, ptr(coef), ptr(resi), w4, w8, lw, lh, qp, bd, sec, alt4)

    def quant_check(self, coef, num, thr):
        return self.L.refk_quant_check(ptr(coef), num, thr)

    def quant_rdoq(self, coef, num, qv, qb, es, pb, abs_coef, abs_level, err):
        return self.L.refk_quant_rdoq(ptr(coef), num, qv, qb, es, pb, ptr(abs_coef), ptr(abs_level), ptr(err))

    def dct_table(self, ln):
        n = 1 << ln
        return np.ctypeslib.as_array(self.L.refk_dct_table(ln), shape=(3, n, n)).copy()

    def scan(self, lw, lh):
        return np.ctypeslib.as_array(self.L.refk_scan(lw, lh), shape=(1 << (lw + lh),)).copy()

    def loka_estimate(self, cfg, org_y, i_org, org_u, org_v, i_org_c, ref_l0, ref_l1, i_ref, want_uv=True,
                      want_dqp=True):
        """loka_estimate_coding_cost itself: (picture cost, icost, icost_uv or None, map_dqp or None)"""
        c = np.ascontiguousarray(cfg, dtype=LOKA_CFG).reshape(1)[0]
        W, H = int(c["width"]), int(c["height"])
        n0, n1 = int(c["num_ref"][0]), int(c["num_ref"][1])
        r0 = (C.c_void_p * 4)(*(list(ref_l0) + [None] * (4 - len(ref_l0))))
        r1 = (C.c_void_p * 4)(*(list(ref_l1) + [None] * (4 - len(ref_l1))))
        p0 = (C.c_longlong * 4)(*[int(v) for v in c["ref_ptr"][0]])
        p1 = (C.c_longlong * 4)(*[int(v) for v in c["ref_ptr"][1]])
        icost = C.c_double()
        icost_uv = (C.c_double * 2)()
        dqp = np.zeros((W // 16) * (H // 16), dtype=np.float32)
        self.L.refk_loka_estimate.restype = C.c_double
        cost = self.L.refk_loka_estimate(W, H, int(c["is_padding"]), int(c["max_search_range"]), int(c["gop_size"]),
                                         C.c_longlong(int(c["ptr"])), ptr(org_y), i_org, ptr(org_u), ptr(org_v), i_org_c,
                                         n0, r0, p0, n1, r1, p1, i_ref, C.byref(icost),
                                         icost_uv if want_uv else None, ptr(dqp) if want_dqp else None)
        return (cost, icost.value, (icost_uv[0], icost_uv[1]) if want_uv else None, dqp if want_dqp else None)

    def me_tz(self, pic, org, i_org, plane_ptrs, i_ref, reqs, threads=1):
        """me_search_tz itself, one call per request (same arguments as Oracle.me_tz)"""
        arr = (C.c_void_p * len(plane_ptrs))(*plane_ptrs)
        reqs = np.ascontiguousarray(reqs, dtype=TZ_REQ)
        out = np.zeros(len(reqs), dtype=TZ_OUT)
        for i in range(len(reqs)):
            self.L.refk_me_tz(pic[0], pic[1], pic[2], pic[3], pic[4], ptr(org), i_org, arr, i_ref,
                              C.c_void_p(reqs.ctypes.data + i * TZ_REQ.itemsize),
                              C.c_void_p(out.ctypes.data + i * TZ_OUT.itemsize))
        return out

    def mc_cu(self, W, H, plane_ptrs, i_ref, chroma_ptrs, i_c, reqs, out_bytes):
        """com_mc_cu itself, one call per request (same arguments as Oracle.mc_cu)"""
        arr = (C.c_void_p * len(plane_ptrs))(*plane_ptrs)
        carr = (C.c_void_p * len(chroma_ptrs))(*chroma_ptrs)
        reqs = np.ascontiguousarray(reqs, dtype=MC_REQ)
        out = np.zeros(max(1, out_bytes), dtype=np.uint8)
        for i in range(len(reqs)):
            self.L.refk_mc_cu(W, H, arr, len(plane_ptrs) // 16, i_ref, carr, i_c,
                              C.c_void_p(reqs.ctypes.data + i * MC_REQ.itemsize), ptr(out))
        return out[:out_bytes]

    def mc_affine(self, W, H, plane_ptrs, i_ref, chroma_ptrs, i_c, reqs, out_bytes):
        """com_mc_cu_affine itself, one call per request (same arguments as Oracle.mc_affine)"""
        arr = (C.c_void_p * len(plane_ptrs))(*plane_ptrs)
        carr = (C.c_void_p * len(chroma_ptrs))(*chroma_ptrs)
        reqs = np.ascontiguousarray(reqs, dtype=AFFINE_REQ)
        out = np.zeros(max(1, out_bytes), dtype=np.uint8)
        for i in range(len(reqs)):
            self.L.refk_mc_affine(W, H, arr, len(plane_ptrs) // 16, i_ref, carr, i_c,
                                  C.c_void_p(reqs.ctypes.data + i * AFFINE_REQ.itemsize), ptr(out))
        return out[:out_bytes]

    def quant_wq(self, reqs, wq4, wq8, coefs):
        """the reference's quant_non_zero with pic_wq_enable, one block per request"""
        reqs = np.ascontiguousarray(reqs, dtype=RDOQ_REQ)
        wq4 = np.ascontiguousarray(wq4, dtype=np.uint8)
        wq8 = np.ascontiguousarray(wq8, dtype=np.uint8)
        nz = np.zeros(len(reqs), dtype=np.int32)
        for i in range(len(reqs)):
            nz[i] = self.L.refk_quant_wq(C.c_void_p(reqs.ctypes.data + i * RDOQ_REQ.itemsize), ptr(wq4), ptr(wq8),
                                         ptr(coefs))
        return nz

    def affine_mvp(self, ptr_cur, ref_ptr, map_mv, map_refi, i_scu, reqs):
        """the reference's com_get_affine_mvp_scaling, one CU per request (requests in the domain)"""
        ref_ptr = np.ascontiguousarray(ref_ptr, dtype=np.int64)
        map_mv = np.ascontiguousarray(map_mv, dtype=np.int16)
        map_refi = np.ascontiguousarray(map_refi, dtype=np.int8)
        reqs = np.ascontiguousarray(reqs, dtype=AFFMVP_REQ)
        out = np.zeros(len(reqs), dtype=AFFMVP_OUT)
        org = i_scu + 1
        mv0 = C.c_void_p(map_mv.ctypes.data + org * 8)
        refi0 = C.c_void_p(map_refi.ctypes.data + org * 2)
        for i, q in enumerate(reqs):
            self.L.refk_affine_mvp(C.c_int64(ptr_cur), ptr(ref_ptr), len(ref_ptr), mv0, refi0, i_scu, int(q["scup"]),
                                   int(q["lidx"]), int(q["cur_refi"]), int(q["cu_width"]), int(q["mvr"]),
                                   C.c_void_p(out.ctypes.data + i * AFFMVP_OUT.itemsize))
        return out

    def affine_merge(self, pic, map_mv, map_refi, map_scu, map_pos, col_mv, col_refi, reqs):
        """the reference's com_get_affine_merge_candidate, one CU per request (requests in the domain)"""
        pic = np.ascontiguousarray(pic, dtype=AFFMRG_PIC).reshape(1)[0]
        i_scu = int(pic["i_scu"])
        org = i_scu + 1
        mv = np.ascontiguousarray(map_mv, dtype=np.int16)
        refi = np.ascontiguousarray(map_refi, dtype=np.int8)
        scu = np.ascontiguousarray(map_scu, dtype=np.uint8)
        pos = np.ascontiguousarray(map_pos, dtype=np.uint32)
        cmv = np.ascontiguousarray(col_mv, dtype=np.int16)
        crefi = np.ascontiguousarray(col_refi, dtype=np.int8)
        ref0 = np.ascontiguousarray(pic["ref0_ptr"], dtype=np.int64)
        clist = np.ascontiguousarray(pic["col_list_ptr"], dtype=np.int64)
        reqs = np.ascontiguousarray(reqs, dtype=AFFMRG_REQ)
        out = np.zeros(len(reqs), dtype=AFFMRG_OUT)
        at = lambda a, b: C.c_void_p(a.ctypes.data + org * b)  # noqa: E731
        num = C.c_int32()
        for i, q in enumerate(reqs):
            o = out[i:i + 1]
            cp = np.zeros(5, np.int8)
            rf = np.zeros((5, 2), np.int8)
            mvs = np.zeros((5, 2, 3, 2), np.int32)
            self.L.refk_affine_merge(C.c_int64(int(pic["ptr"])), ptr(ref0), ptr(clist), at(mv, 8), at(refi, 2),
                                     at(scu, 1), at(pos, 4), at(cmv, 8), at(crefi, 2), i_scu,
                                     int(pic["pic_width_in_scu"]), int(pic["pic_height_in_scu"]),
                                     int(pic["slice_type"]), int(pic["log2_max_cuwh"]), int(q["scup"]),
                                     int(q["cu_width"]), int(q["cu_height"]), C.byref(num), ptr(cp), ptr(rf), ptr(mvs))
            o["num"] = num.value
            o["cp_num"] = cp
            o["refi"] = rf
            o["cpmv"] = mvs
        return out

    def coef_rate(self, levels, reqs):
        """the reference's lbac_enc_run_length_cc_rdo, one block per request"""
        levels = np.ascontiguousarray(levels, dtype=np.int16)
        reqs = np.ascontiguousarray(reqs, dtype=COEF_RATE_REQ)
        out = np.zeros(len(reqs), dtype=COEF_RATE_OUT)
        for i in range(len(reqs)):
            self.L.refk_coef_rate(ptr(levels), C.c_void_p(reqs.ctypes.data + i * COEF_RATE_REQ.itemsize),
                                  C.c_void_p(out.ctypes.data + i * COEF_RATE_OUT.itemsize))
        return out

    def lbac_next(self, model, mps):
        return self.L.refk_lbac_next(int(model), int(mps))

    def make_ipred_list(self, nb, org, s_org, avail, ipf, req):
        """the reference's make_ipred_list for one block; returns (RMD_OUT record, satd[33])"""
        req = np.ascontiguousarray(np.asarray(req).reshape(1), dtype=RMD_REQ)
        out = np.zeros(1, dtype=RMD_OUT)
        satd = np.zeros(33, dtype=np.uint32)
        self.L.refk_make_ipred_list(ptr(nb), C.c_void_p(org), s_org, avail, ipf, ptr(req), ptr(out), ptr(satd))
        return out[0], satd

    def me_affine(self, W, H, org, i_org, plane_ptrs, i_ref, reqs, threads=1):
        """the reference's affine_me_gradient, one call per request (same arguments as Oracle.me_affine)"""
        arr = (C.c_void_p * len(plane_ptrs))(*plane_ptrs)
        reqs = np.ascontiguousarray(reqs, dtype=AFFME_REQ)
        out = np.zeros(len(reqs), dtype=AFFME_OUT)
        for i in range(len(reqs)):
            self.L.refk_affine_me(W, H, ptr(org), i_org, arr, i_ref,
                                  C.c_void_p(reqs.ctypes.data + i * AFFME_REQ.itemsize),
                                  C.c_void_p(out.ctypes.data + i * AFFME_OUT.itemsize))
        return out

    def rdoq(self, reqs, ests, coefs):
        """quant_non_zero itself, one call per request (same arguments as Oracle.rdoq)"""
        reqs = np.ascontiguousarray(reqs, dtype=RDOQ_REQ)
        ests = np.ascontiguousarray(ests, dtype=RDOQ_EST)
        nz = np.zeros(len(reqs), dtype=np.int32)
        for i in range(len(reqs)):
            nz[i] = self.L.refk_rdoq(C.c_void_p(reqs.ctypes.data + i * RDOQ_REQ.itemsize),
                                     C.c_void_p(ests.ctypes.data + int(reqs[i]["est"]) * RDOQ_EST.itemsize),
                                     ptr(coefs))
        return nz

    def rdoq_est_from_ctx(self, ctx):
        """rdoq_init_cu_est_bits of 86 context models (ctp, cbf[3], run[24], level[24], last1[12],
        last2[22])"""
        ctx = np.ascontiguousarray(ctx, dtype=np.uint16)
        e = np.zeros(1, dtype=RDOQ_EST)
        self.L.refk_rdoq_est_from_ctx(ptr(ctx), ptr(e))
        return e[0]

    def loka_search(self, cfg, org_y, i_org, ref, i_ref, ref_ptr, refi, num_refp, x, y):
        """me_search_tz of one 16x16 unit with the lookahead's settings: (mv_x, mv_y, cost)"""
        c = np.ascontiguousarray(cfg, dtype=LOKA_CFG).reshape(1)[0]
        mv = (C.c_short * 2)()
        self.L.refk_loka_search.restype = C.c_ulonglong
        cost = self.L.refk_loka_search(int(c["width"]), int(c["height"]), int(c["is_padding"]),
                                       int(c["max_search_range"]), int(c["gop_size"]), C.c_longlong(int(c["ptr"])),
                                       ptr(org_y), i_org, P(ref), i_ref, C.c_longlong(int(ref_ptr)), refi, num_refp,
                                       x, y, mv)
        return mv[0], mv[1], cost


ME_BLOCK = np.dtype([("x", "<i2"), ("y", "<i2"), ("w", "u1"), ("h", "u1"), ("pad", "<u2")])
ME_RESULT = np.dtype([("mv_int", "<i2", (2,)), ("mv_sub", "<i2", (2,)), ("sad_int", "<u4"), ("satd_sub", "<u4"),
                      ("cost_int", "<u8"), ("cost_sub", "<u8")])
CU = ME_BLOCK
LOKA_CFG = np.dtype([("width", "<i4"), ("height", "<i4"), ("is_padding", "<i4"), ("max_search_range", "<i4"),
                     ("gop_size", "<i4"), ("num_ref", "<i4", (2,)), ("ptr", "<i8"), ("ref_ptr", "<i8", (2, 4))],
                    align=True)
LOKA_UNIT = np.dtype([("mv", "<i2", (2, 4, 2)), ("satd", "<u4", (2, 4)), ("bi_satd", "<u4"), ("zero_satd", "<u4"),
                      ("min_cost", "<u4"), ("min_icost", "<u4"), ("icost_u", "<u4"), ("icost_v", "<u4"),
                      ("energy", "<u8"), ("best_mode", "u1"), ("pad", "u1", (7,))])
TZ_REQ = np.dtype([("x", "<i2"), ("y", "<i2"), ("w", "u1"), ("h", "u1"), ("ref_slot", "u1"), ("refi", "i1"),
                   ("num_refp", "u1"), ("mvr", "u1"), ("bi", "u1"), ("flags", "u1"), ("mvp", "<i2", (2,)),
                   ("mv", "<i2", (2,)), ("mv_ipel", "<i2", (2,)), ("other_mv", "<i2", (2,)), ("other_slot", "u1"),
                   ("pad0", "u1", (3,)), ("mot_bits_other", "<i4"), ("lambda_mv", "<u4"), ("dist", "<i4"),
                   ("pad1", "<i4")])
TZ_OUT = np.dtype([("mv", "<i2", (2,)), ("mv_ipel", "<i2", (2,)), ("cost", "<u8")])
MC_REQ = np.dtype([("x", "<i2"), ("y", "<i2"), ("w", "u1"), ("h", "u1"), ("slot", "i1", (2,)),
                   ("mv", "<i2", (2, 2)), ("channel", "u1"), ("pad", "u1", (3,)), ("out_offset", "<u4")])
AFFINE_REQ = np.dtype([("x", "<i2"), ("y", "<i2"), ("w", "u1"), ("h", "u1"), ("slot", "i1", (2,)), ("cp_num", "u1"),
                       ("sub8", "u1"), ("pad", "u1", (2,)), ("cpmv", "<i4", (2, 3, 2)), ("out_offset", "<u4")])
COEF_CTX = [("run", "<i2", (12,)), ("run_rdoq", "<i2", (12,)), ("level", "<i2", (12,)), ("last1", "<i2", (6,)),
            ("last2", "<i2", (12,))]
COEF_RATE_REQ = np.dtype([("coef_offset", "<u4"), ("log2w", "u1"), ("log2h", "u1"), ("ch_type", "u1"), ("pad", "u1"),
                          ("num_sig", "<u2"), ("range", "<u2")] + COEF_CTX)
COEF_RATE_OUT = np.dtype([("bits", "<u4"), ("range", "<u2"), ("pad", "<u2")] + COEF_CTX)
RMD_REQ = np.dtype([("satd_row", "<u4"), ("pb_w", "u1"), ("pb_h", "u1"), ("mpm", "u1", (2,)), ("skip_ipd", "u1"),
                    ("fast", "u1"), ("range", "<u2"), ("ctx", "<i2", (7,)), ("pad", "u1", (6,)),
                    ("sqrt_lambda", "<f8"), ("inter_satd", "<u8"), ("satd_threshold", "<f8")])
RMD_OUT = np.dtype([("list", "i1", (5,)), ("count", "u1"), ("pad", "u1", (2,))])
AFFME_BI, AFFME_UNI_START, AFFME_SUB8 = 1, 2, 4
AFFME_REQ = np.dtype([("x", "<i2"), ("y", "<i2"), ("w", "u1"), ("h", "u1"), ("ref_slot", "u1"), ("refi", "i1"),
                      ("num_refp", "u1"), ("mvr", "u1"), ("flags", "u1"), ("other_slot", "u1"), ("lambda_mv", "<u4"),
                      ("mot_bits_other", "<i4"), ("pad", "<i4"), ("mvp", "<i4", (2, 2)), ("mv", "<i4", (2, 2)),
                      ("other_mv", "<i4", (2, 2))])
AFFME_OUT = np.dtype([("mv", "<i4", (2, 2)), ("satd", "<u4"), ("bits", "<i4"), ("cost", "<u8")])
RDOQ_EST = np.dtype([("ctp", "<i4", (2,)), ("cbf", "<i4", (3, 2)), ("run", "<i4", (24, 2)), ("lvl", "<i4", (24, 2)),
                     ("lst", "<i4", (2, 6, 12, 2))])
RDOQ_REQ = np.dtype([("coef_offset", "<u4"), ("log2w", "u1"), ("log2h", "u1"), ("qp", "u1"), ("is_intra", "u1"),
                     ("ch_type", "u1"), ("slice_type", "u1"), ("est", "<u2"), ("pad", "<u4"), ("lambda_", "<i8")])
AFFMVP_REQ = np.dtype([("scup", "<i4"), ("cu_width", "<i2"), ("lidx", "i1"), ("cur_refi", "i1"), ("mvr", "i1"),
                       ("pad", "i1", (3,))])
AFFMVP_OUT = np.dtype([("mvp", "<i4", (2, 2))])
AFFMRG_PIC = np.dtype([("ptr", "<i8"), ("ref0_ptr", "<i8", (2,)), ("col_list_ptr", "<i8", (17,)), ("i_scu", "<i4"),
                       ("pic_width_in_scu", "<i4"), ("pic_height_in_scu", "<i4"), ("rows", "<i4"),
                       ("slice_type", "<i4"), ("log2_max_cuwh", "<i4")])
AFFMRG_REQ = np.dtype([("scup", "<i4"), ("cu_width", "<i2"), ("cu_height", "<i2")])
AFFMRG_OUT = np.dtype([("num", "<i4"), ("cp_num", "i1", (5,)), ("refi", "i1", (5, 2)), ("pad", "i1"),
                       ("cpmv", "<i4", (5, 2, 3, 2))])
LAT_Q = np.dtype([("ssd", "<u4"), ("coef_hash", "<u4"), ("num_nz", "<u2"), ("last_nz", "<i2"), ("sum_abs", "<u4")])

MC_LUMA = np.array([[0, 0, 0, 64, 0, 0, 0, 0], [-1, 4, -10, 57, 19, -7, 3, -1], [-1, 4, -11, 40, 40, -11, 4, -1],
                    [-1, 3, -7, 19, 57, -10, 4, -1]], dtype=np.int8)
MC_CHROMA = np.array([[0, 64, 0, 0], [-4, 62, 6, 0], [-6, 56, 15, -1], [-5, 47, 25, -3], [-4, 36, 36, -4],
                      [-3, 25, 47, -5], [-1, 15, 56, -6], [0, 6, 62, -4]], dtype=np.int8)


def has_ref():
    return os.path.exists(REF_SO)
