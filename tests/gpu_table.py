"""GPU backend for the golden cases: the pyoracle method set implemented by calling the
libuavs3e_cuda kernel-table entries (include/uavs3e_cuda_table.h) through ctypes."""
import ctypes as C

import numpy as np

P = C.c_void_p
W_OF = {4: 0, 8: 1, 16: 2, 32: 3, 64: 4, 128: 5}


def _p(a):
    return C.c_void_p(a.ctypes.data)


class GpuTable:
    def __init__(self, L):
        self.L = L
        for n in ("cost_sad", "cost_satd"):
            pass
        for w in W_OF:
            getattr(L, f"uavs3e_cuda_cost_sad_{w}").restype = C.c_uint32
            getattr(L, f"uavs3e_cuda_cost_ssd_{w}").restype = C.c_uint64
        for s in ("4x4", "8x4", "4x8", "8x8", "16x8", "8x16"):
            getattr(L, f"uavs3e_cuda_cost_satd_{s}").restype = C.c_uint32
        L.uavs3e_cuda_quant_rdoq.restype = C.c_int
        L.uavs3e_cuda_quant_check.restype = C.c_int

    def sad(self, w, h, o, io, p, ip):
        return getattr(self.L, f"uavs3e_cuda_cost_sad_{w}")(P(o), io, P(p), ip, h)

    def ssd(self, w, h, o, io, p, ip):
        return getattr(self.L, f"uavs3e_cuda_cost_ssd_{w}")(P(o), io, P(p), ip, h)

    def satd_tile(self, tw, th, o, io, p, ip):
        return getattr(self.L, f"uavs3e_cuda_cost_satd_{tw}x{th}")(P(o), io, P(p), ip)

    def had(self, w, h, o, io, p, ip, bd=8):
        raise NotImplementedError("com_had is not a table entry")

    def ipflt(self, t, s, is_, d, id_, w, h, c, mx=255):
        fn = ("h8", "h4", "v8", "v4")[t]
        getattr(self.L, f"uavs3e_cuda_ipflt_{fn}")(P(s), is_, P(d), id_, w, h, _p(c), mx)

    def ipflt_ext(self, t, s, is_, d, id_, w, h, cx, cy, mx=255):
        getattr(self.L, f"uavs3e_cuda_ipflt_ext{8 if t == 0 else 4}")(P(s), is_, P(d), id_, w, h, _p(cx), _p(cy), mx)

    def ipcpy(self, s, is_, d, id_, w, h):
        self.L.uavs3e_cuda_ipcpy(P(s), is_, P(d), id_, w, h)

    def if_luma_frame(self, plane0_ptr, plane_ptrs, W, H, pad, stride):
        """com_if_luma_frame composed from the ip_flt_y_* entries and the padding rule"""
        coef = np.array([[-1, 4, -10, 57, 19, -7, 3, -1], [-1, 4, -11, 40, 40, -11, 4, -1],
                         [-1, 3, -7, 19, 57, -10, 4, -1]], dtype=np.int8)
        ts = W + 16
        tmp = [np.zeros(ts * (H + 16), np.int16) for _ in range(3)]
        TmpArr = C.c_void_p * 3
        d = (C.c_void_p * 3)(*[plane_ptrs[i] - 8 * stride - 8 for i in range(3)])
        self.L.uavs3e_cuda_ip_flt_y_hor(P(plane0_ptr - 8 * stride - 8), stride, d, stride,
                                        TmpArr(*[t.ctypes.data for t in tmp]), ts, W + 16, H + 16, _p(coef), 8)
        d = (C.c_void_p * 3)(*[plane_ptrs[4 * k - 1] - 4 * stride - 4 for k in (1, 2, 3)])
        self.L.uavs3e_cuda_ip_flt_y_ver(P(plane0_ptr - 4 * stride - 4), stride, d, stride, W + 8, H + 8, _p(coef), 8)
        for dx in (1, 2, 3):
            d = (C.c_void_p * 3)(*[plane_ptrs[4 * k + dx - 1] - 4 * stride - 4 for k in (1, 2, 3)])
            self.L.uavs3e_cuda_ip_flt_y_ver_ext(P(tmp[dx - 1].ctypes.data + 2 * (4 * ts + 4)), ts, d, stride, W + 8,
                                                H + 8, _p(coef), 8)
        # the edge padding of each fractional plane (com_img_padding(img, 1, 4)) on the host view
        rows = H + 2 * pad
        for q in plane_ptrs:
            buf = np.ctypeslib.as_array((C.c_uint8 * (rows * stride)).from_address(q - pad * stride - pad))
            img = buf.reshape(rows, stride)
            r0, r1, c0, c1 = pad - 4, pad + H + 4, pad - 4, pad + W + 4
            img[r0:r1, :c0] = img[r0:r1, c0:c0 + 1]
            img[r0:r1, c1:] = img[r0:r1, c1 - 1:c1]
            img[:r0] = img[r0]
            img[r1:] = img[r1 - 1]

    def pel_diff(self, w, h, o, io, p, ip, r, ir):
        getattr(self.L, f"uavs3e_cuda_pel_diff_{w}")(P(o), io, P(p), ip, P(r), ir, h)

    def pel_avrg(self, w, h, d, id_, s1, s2):
        getattr(self.L, f"uavs3e_cuda_pel_avrg_{w}")(P(d), id_, P(s1), P(s2), h)

    def recon(self, resi, pred, ipred, w, h, rec, irec, cbf, bd=8):
        self.L.uavs3e_cuda_recon(P(resi), P(pred), ipred, w, h, P(rec), irec, cbf, bd)

    def intra_get_nbr(self, *a, **k):
        raise NotImplementedError("com_intra_get_nbr is not a table entry")

    def intra_pred(self, nb, dst, ipm, w, h, avail, ipf, bd=8):
        """com_intra_pred (src/com_ipred.c:733) composed from the table entries, as the encoder does"""
        L = self.L
        mid = nb.ctypes.data + 288
        d = dst.ctypes.data
        if ipm not in (1, 2):
            if ipm == 12:
                L.uavs3e_cuda_intra_pred_ver(P(mid + 1), P(d), w, w, h)
            elif ipm == 24:
                L.uavs3e_cuda_intra_pred_hor(P(mid - 1), P(d), w, w, h)
            elif ipm == 0:
                L.uavs3e_cuda_intra_pred_dc(P(mid), P(d), w, w, h, avail, bd)
            else:
                getattr(L, f"uavs3e_cuda_intra_pred_ang_{ipm}")(P(mid), P(d), w, ipm, w, h)
            if ipf:
                L.uavs3e_cuda_intra_pred_ipf_core(P(mid), P(d), w, ipm, w, h, bd)
        elif ipf:
            tmp = np.zeros(w * h, np.int16)
            if ipm == 1:
                L.uavs3e_cuda_intra_pred_plane_ipf(P(mid), _p(tmp), w, h)
            else:
                L.uavs3e_cuda_intra_pred_bi_ipf(P(mid), _p(tmp), w, h)
            L.uavs3e_cuda_intra_pred_ipf_core_s16(P(mid), P(d), w, _p(tmp), ipm, w, h, bd)
        elif ipm == 1:
            L.uavs3e_cuda_intra_pred_plane(P(mid), P(d), w, w, h, bd)
        else:
            L.uavs3e_cuda_intra_pred_bi(P(mid), P(d), w, w, h, bd)

    def ipred_ang(self, nb, dst, i_dst, mode, w, h):
        getattr(self.L, f"uavs3e_cuda_intra_pred_ang_{mode}")(P(nb.ctypes.data + 288), _p(dst), i_dst, mode, w, h)

    def trans_dct2(self, lw, lh, src, dst, bd=8):
        getattr(self.L, f"uavs3e_cuda_trans_dct2_w{1 << lw}_h{1 << lh}")(_p(src), _p(dst), bd)

    def itrans_dct2(self, lh, lw, coef, resi, bd=8):
        getattr(self.L, f"uavs3e_cuda_itrans_dct2_h{1 << lh}_w{1 << lw}")(_p(coef), _p(resi), bd)

    def trans_dct8_dst7(self, t, ln, src, dst, shift, line):
        getattr(self.L, f"uavs3e_cuda_tx_{('dct8', 'dst7')[t]}_{1 << ln}")(_p(src), _p(dst), shift, line)

    def itrans_dct8_dst7(self, t, ln, coef, blk, shift, line, mx, mn):
        getattr(self.L, f"uavs3e_cuda_itx_{('dct8', 'dst7')[t]}_{1 << ln}")(_p(coef), _p(blk), shift, line, mx, mn)

    def transform(self, *a, **k):
        raise NotImplementedError("transform() is a caller of the table, not an entry")

    def invqt(self, *a, **k):
        raise NotImplementedError("com_invqt is a caller of the table, not an entry")

    def dquant(self, flat, coef, out, wq4, wq8, lw, lh, scale, shift, bd=8):
        arr = (C.c_void_p * 2)(wq4.ctypes.data, wq8.ctypes.data)
        fn = self.L.uavs3e_cuda_dquant if flat else self.L.uavs3e_cuda_dquant_wq
        fn(_p(coef), _p(out), arr, lw, lh, scale, shift, bd)

    def quant_check(self, coef, num, thr):
        return self.L.uavs3e_cuda_quant_check(_p(coef), num, thr)

    def quant_rdoq(self, coef, num, qv, qb, es, pb, abs_coef, abs_level, err):
        return self.L.uavs3e_cuda_quant_rdoq(_p(coef), num, qv, qb, es, pb, _p(abs_coef), _p(abs_level), _p(err))

    def dct_table(self, ln):
        raise NotImplementedError

    def scan(self, lw, lh):
        raise NotImplementedError
