"""uavs3e_gb300 -- GB300 (sm_103a) implementation of uavs3e's mode-decision hot path.

The product is the C-ABI library ``libuavs3e_cuda.so`` (include/uavs3e_cuda.h).  This package
builds it in-tree (``build()``) and binds it with ctypes for Python callers (tests, bench).
There is no CPU implementation here: every call runs on the GPU, and loading fails loudly when
the library is missing.
"""
import ctypes as C
import os

import numpy as np

from .build import LIB, build  # noqa: F401

_lib = None

ME_RESULT = np.dtype([("mv_int", "<i2", (2,)), ("mv_sub", "<i2", (2,)), ("sad_int", "<u4"), ("satd_sub", "<u4"),
                      ("cost_int", "<u8"), ("cost_sub", "<u8")])


class CudaError(RuntimeError):
    pass


def lib():
    """The loaded libuavs3e_cuda (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise CudaError("libuavs3e_cuda.so is not built (run uavs3e_gb300.build())")
        L = C.CDLL(LIB)
        _declare(L)
        _lib = L
    return _lib


def _declare(L):
    P, I, U32 = C.c_void_p, C.c_int, C.c_uint32
    L.uavs3e_cuda_init.argtypes = [I]
    L.uavs3e_cuda_status.restype = I
    L.uavs3e_cuda_status_string.restype = C.c_char_p
    L.uavs3e_cuda_version.restype = C.c_char_p
    L.uavs3e_cuda_subpel_planes.argtypes = [P, P, I, I, I, I, P]
    L.uavs3e_cuda_pad_plane.argtypes = [P, I, I, I, I, P]
    L.uavs3e_cuda_me_open.restype = P
    L.uavs3e_cuda_me_open.argtypes = [I, I, I, I, I]
    L.uavs3e_cuda_me_close.argtypes = [P]
    L.uavs3e_cuda_me_num_results.argtypes = [P]
    L.uavs3e_cuda_me_set_ref.argtypes = [P, I, P, I]
    L.uavs3e_cuda_me_set_ref_device.argtypes = [P, I, P, I, P]
    L.uavs3e_cuda_me_run.argtypes = [P, P, I, U32, P]
    L.uavs3e_cuda_me_run_device.argtypes = [P, P, I, U32, P, P]
    L.uavs3e_cuda_me_frame_graph.argtypes = [P, I, P, I, P, I, U32, P, P]
    L.uavs3e_cuda_me_plane.restype = P
    L.uavs3e_cuda_me_plane.argtypes = [P, I, I]
    L.uavs3e_cuda_me_plane_stride.argtypes = [P]
    L.uavs3e_cuda_lattice_cus.argtypes = [I, I, P, I]
    L.uavs3e_cuda_lattice_autotune.argtypes = [I]
    L.uavs3e_cuda_lattice_autotune.restype = None
    L.uavs3e_cuda_lattice_budgets.argtypes = [I, P]
    L.uavs3e_cuda_intra_lattice_device.argtypes = [P, I, P, I, I, I, P, I, I, P, I, I, P, P, P]
    L.uavs3e_cuda_intra_lattice.argtypes = [P, I, P, I, I, I, P, I, I, P, I, I, P, P]
    L.uavs3e_cuda_intra_lattice_modes_device.argtypes = [P, I, P, I, I, I, P, I, P, I, I, P, I, I, P, P, P]
    L.uavs3e_cuda_profile_enable.argtypes = [I]
    L.uavs3e_cuda_launch_count.restype = C.c_ulonglong
    L.uavs3e_cuda_profile_collect.argtypes = [P, P, I]
    L.uavs3e_cuda_loka_estimate.argtypes = [P, P, I, P, P, I, P, P, I, I, P, P, P, P, P]
    L.uavs3e_cuda_loka_units_device.argtypes = [P, P, I, P, P, I, P, P, I, I, P, P, P, P]
    L.uavs3e_cuda_loka_finish.argtypes = [P, P, P, P, P, P]
    L.uavs3e_cuda_loka_finish.restype = C.c_double
    L.uavs3e_cuda_loka_sc_ratio.argtypes = [I, I, I, I, I, C.c_int64, P, I, P, P, I, P, C.c_int64, I, I, P]
    L.uavs3e_cuda_me_tz.argtypes = [P, P, P, I, P, I, P]
    L.uavs3e_cuda_me_tz_device.argtypes = [P, P, I, P, I, I, I, P, I, P, P]
    L.uavs3e_cuda_me_set_ref_chroma.argtypes = [P, I, P, P, I]
    L.uavs3e_cuda_me_chroma_plane.restype = P
    L.uavs3e_cuda_me_chroma_plane.argtypes = [P, I, I]
    L.uavs3e_cuda_me_chroma_stride.argtypes = [P]
    L.uavs3e_cuda_mc_cu.argtypes = [P, P, I, P, C.c_size_t]
    L.uavs3e_cuda_mc_cu_device.argtypes = [I, I, P, I, I, I, P, I, I, P, I, P, C.c_size_t, P]
    L.uavs3e_cuda_mc_affine.argtypes = [P, P, I, P, C.c_size_t]
    L.uavs3e_cuda_mc_affine_device.argtypes = [I, I, P, I, I, I, P, I, I, P, I, P, C.c_size_t, P]
    L.uavs3e_cuda_rdoq.argtypes = [P, I, P, I, P, C.c_size_t, P]
    L.uavs3e_cuda_me_affine.argtypes = [P, P, I, P, I, P]
    L.uavs3e_cuda_me_frame.argtypes = [P, I, P, I, P, I, C.c_uint32, P]
    L.uavs3e_cuda_affine_mvp.argtypes = [C.c_int64, P, I, P, P, I, I, P, I, P]
    L.uavs3e_cuda_affine_mvp_device.argtypes = [C.c_int64, P, I, P, P, I, I, P, I, P, P, P]
    L.uavs3e_cuda_affine_merge.argtypes = [P, P, P, P, P, P, P, P, I, P]
    L.uavs3e_cuda_affine_merge_device.argtypes = [P, P, P, P, P, P, P, P, I, P, P, P]
    L.uavs3e_cuda_intra_rmd.argtypes = [P, C.c_size_t, P, I, P]
    L.uavs3e_cuda_coef_rate.argtypes = [P, I, P, C.c_size_t, P]
    L.uavs3e_cuda_quant_wq.argtypes = [P, I, P, P, P, C.c_size_t, P]
    L.uavs3e_cuda_quant_wq_device.argtypes = [P, I, P, P, P, C.c_size_t, P, P]
    L.uavs3e_cuda_coef_rate_device.argtypes = [P, I, P, C.c_size_t, P, P]
    L.uavs3e_cuda_intra_rmd_device.argtypes = [P, C.c_size_t, P, I, P, P]
    L.uavs3e_cuda_me_affine_device.argtypes = [I, I, P, I, P, I, I, I, P, I, P, P]
    L.uavs3e_cuda_rdoq_device.argtypes = [P, I, P, I, P, C.c_size_t, P, P]


def check(rc, what="uavs3e_cuda"):
    if rc != 0:
        L = lib()
        msg = L.uavs3e_cuda_status_string().decode()
        L.uavs3e_cuda_clear_status()
        raise CudaError(f"{what} failed ({rc}): {msg}")
    return rc


def init(device=0):
    check(lib().uavs3e_cuda_init(device), "uavs3e_cuda_init")


PROF_KERNELS = ("pad", "subpel_planes", "me_int", "me_sub", "intra_lattice", "loka", "tz", "mc", "rdoq", "affme",
                "shift_planes")

CU = np.dtype([("x", "<i2"), ("y", "<i2"), ("w", "u1"), ("h", "u1"), ("pad", "<u2")])
LAT_Q = np.dtype([("ssd", "<u4"), ("coef_hash", "<u4"), ("num_nz", "<u2"), ("last_nz", "<i2"), ("sum_abs", "<u4")])


def lattice_cus(width, height):
    """the 23-shape CU lattice of a picture (largest shapes first)"""
    n = lib().uavs3e_cuda_lattice_cus(width, height, None, 0)
    out = np.zeros(n, dtype=CU)
    lib().uavs3e_cuda_lattice_cus(width, height, out.ctypes.data, n)
    return out


def lattice_autotune(on=True):
    """switch the lattice's CTA-layout autotuning on (default) or off"""
    lib().uavs3e_cuda_lattice_autotune(1 if on else 0)


def lattice_budgets(n_modes=33):
    """tuned shared-memory budget (bytes) per shape (log2 w - 2) * 5 + (log2 h - 2); 0 = default"""
    out = (C.c_int * 25)()
    check(lib().uavs3e_cuda_lattice_budgets(n_modes, out), "lattice_budgets")
    return list(out)


def intra_lattice(org, rec, cus, qps=(27, 32, 37, 42), ipf=0, is_intra=1, stream=None):
    """Intra lattice on the GPU from host arrays; returns (satd[n_cus*33], q[n_cus*33*n_qp])."""
    import torch
    H, W = org.shape
    d_org = torch.from_numpy(np.ascontiguousarray(org)).cuda()
    d_rec = torch.from_numpy(np.ascontiguousarray(rec)).cuda()
    d_cus = torch.from_numpy(np.ascontiguousarray(cus).view(np.uint8)).cuda()
    n = len(cus)
    q = np.ascontiguousarray(qps, dtype=np.int32)
    d_satd = torch.zeros(max(1, n * 33), dtype=torch.int32, device="cuda")
    d_q = torch.zeros(max(1, n * 33 * len(q) * LAT_Q.itemsize), dtype=torch.uint8, device="cuda")
    sp = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    check(lib().uavs3e_cuda_intra_lattice_device(d_org.data_ptr(), W, d_rec.data_ptr(), W, W, H, d_cus.data_ptr(), n,
                                                 ipf, q.ctypes.data, len(q), is_intra, d_satd.data_ptr(),
                                                 d_q.data_ptr(), sp), "intra_lattice")
    torch.cuda.synchronize()
    return (d_satd.cpu().numpy().view(np.uint32)[:n * 33].copy(),
            d_q.cpu().numpy().view(LAT_Q)[:n * 33 * len(q)].copy())


def intra_lattice_host(org, rec, cus, qps=(27, 32, 37, 42), ipf=0, is_intra=1, satd=None, q=None):
    """Intra lattice through the host-buffer entry uavs3e_cuda_intra_lattice (copies inside the
    call); returns (satd[n_cus*33], q[n_cus*33*n_qp]).  satd / q may be given (e.g. pinned)."""
    H, W = org.shape
    # rows must be contiguous; a row stride larger than the width is passed through
    org = org if org.dtype == np.uint8 and org.strides[1] == 1 else np.ascontiguousarray(org, np.uint8)
    rec = rec if rec.dtype == np.uint8 and rec.strides[1] == 1 else np.ascontiguousarray(rec, np.uint8)
    cus = np.ascontiguousarray(cus)
    n = len(cus)
    qa = np.ascontiguousarray(qps, dtype=np.int32)
    if satd is None:
        satd = np.zeros(n * 33, np.uint32)
    if q is None:
        q = np.zeros(n * 33 * max(1, len(qa)), LAT_Q)
    check(lib().uavs3e_cuda_intra_lattice(org.ctypes.data, org.strides[0], rec.ctypes.data, rec.strides[0], W, H,
                                          cus.ctypes.data, n, ipf, qa.ctypes.data, len(qa), is_intra,
                                          satd.ctypes.data, q.ctypes.data), "intra_lattice")
    return satd, q


# ------------------------------------------------------------------ lookahead cost estimation
LOKA_CFG = np.dtype([("width", "<i4"), ("height", "<i4"), ("is_padding", "<i4"), ("max_search_range", "<i4"),
                     ("gop_size", "<i4"), ("num_ref", "<i4", (2,)), ("ptr", "<i8"), ("ref_ptr", "<i8", (2, 4))],
                    align=True)
LOKA_UNIT = np.dtype([("mv", "<i2", (2, 4, 2)), ("satd", "<u4", (2, 4)), ("bi_satd", "<u4"), ("zero_satd", "<u4"),
                      ("min_cost", "<u4"), ("min_icost", "<u4"), ("icost_u", "<u4"), ("icost_v", "<u4"),
                      ("energy", "<u8"), ("best_mode", "u1"), ("pad", "u1", (7,))])


def loka_cfg(width, height, is_padding, max_search_range, gop_size, ptr, ref_ptr_l0=(), ref_ptr_l1=()):
    """the uavs3e_cuda_loka_cfg_t record of one picture"""
    c = np.zeros(1, dtype=LOKA_CFG)
    c["width"], c["height"], c["is_padding"] = width, height, is_padding
    c["max_search_range"], c["gop_size"], c["ptr"] = max_search_range, gop_size, ptr
    c["num_ref"][0] = [len(ref_ptr_l0), len(ref_ptr_l1)]
    for li, lst in enumerate((ref_ptr_l0, ref_ptr_l1)):
        for r, t in enumerate(lst):
            c["ref_ptr"][0, li, r] = t
    return c


def _addrs(planes, pad):
    """sample-(0,0) addresses of padded 2-D planes"""
    arr = (C.c_void_p * 4)()
    for i, p in enumerate(planes):
        arr[i] = p.ctypes.data + pad * p.strides[0] + pad
    return arr


def loka_estimate(cfg, org_y, org_u, org_v, refs_l0, refs_l1, ref_pad, units=False):
    """loka_estimate_coding_cost on host planes: refs are 2-D uint8 planes padded by ref_pad.
    Returns dict(cost, icost, icost_uv, map_dqp[, units])."""
    cfg = np.ascontiguousarray(cfg, dtype=LOKA_CFG).reshape(1)
    W, H = int(cfg["width"][0]), int(cfg["height"][0])
    n = (W // 16) * (H // 16)
    refs = [np.ascontiguousarray(r) for r in refs_l0] + [np.ascontiguousarray(r) for r in refs_l1]
    i_ref = refs[0].strides[0] if refs else 0
    a0, a1 = _addrs(refs[:len(refs_l0)], ref_pad), _addrs(refs[len(refs_l0):], ref_pad)
    cost, icost = C.c_double(), C.c_double()
    icost_uv = (C.c_double * 2)()
    dqp = np.zeros(max(1, n), dtype=np.float32)
    out = np.zeros(max(1, n), dtype=LOKA_UNIT) if units else None
    check(lib().uavs3e_cuda_loka_estimate(cfg.ctypes.data, org_y.ctypes.data, org_y.strides[0], org_u.ctypes.data,
                                          org_v.ctypes.data, org_u.strides[0], a0, a1, i_ref, ref_pad,
                                          C.byref(cost), C.byref(icost), icost_uv, dqp.ctypes.data,
                                          out.ctypes.data if units else None), "loka_estimate")
    r = dict(cost=cost.value, icost=icost.value, icost_uv=(icost_uv[0], icost_uv[1]), map_dqp=dqp[:n])
    if units:
        r["units"] = out[:n]
    return r


def loka_sc_ratio(width, height, is_padding, max_search_range, gop_size, ptr, org_y, org_u, org_v, last_y, last_ptr,
                  last_pad):
    """loka_get_sc_ratio: last_y is the previous picture's luma plane padded by last_pad"""
    ratio = C.c_double()
    addr = last_y.ctypes.data + last_pad * last_y.strides[0] + last_pad
    check(lib().uavs3e_cuda_loka_sc_ratio(width, height, is_padding, max_search_range, gop_size, ptr,
                                          org_y.ctypes.data, org_y.strides[0], org_u.ctypes.data, org_v.ctypes.data,
                                          org_u.strides[0], addr, last_ptr, last_y.strides[0], last_pad,
                                          C.byref(ratio)), "loka_sc_ratio")
    return ratio.value


def loka_units_device(cfg, d_org_y, i_org, d_org_u, d_org_v, i_org_c, d_refs_l0, d_refs_l1, i_ref, ref_pad, d_units,
                      d_energy, d_totals, stream=None):
    """device-buffer entry (addresses as ints), enqueued on `stream` (default: torch's current)"""
    cfg = np.ascontiguousarray(cfg, dtype=LOKA_CFG).reshape(1)
    a0 = (C.c_void_p * 4)(*(list(d_refs_l0) + [None] * (4 - len(d_refs_l0))))
    a1 = (C.c_void_p * 4)(*(list(d_refs_l1) + [None] * (4 - len(d_refs_l1))))
    if stream is None:
        import torch
        stream = torch.cuda.current_stream().cuda_stream
    check(lib().uavs3e_cuda_loka_units_device(cfg.ctypes.data, d_org_y, i_org, d_org_u, d_org_v, i_org_c, a0, a1,
                                              i_ref, ref_pad, d_units, d_energy, d_totals, stream),
          "loka_units_device")


def loka_finish(cfg, totals, energy=None):
    """(cost, icost, icost_uv, map_dqp or None) from host totals[>=4] and energies"""
    cfg = np.ascontiguousarray(cfg, dtype=LOKA_CFG).reshape(1)
    t = np.ascontiguousarray(totals, dtype=np.uint64)
    icost = C.c_double()
    icost_uv = (C.c_double * 2)()
    dqp = None
    if energy is not None:
        energy = np.ascontiguousarray(energy, dtype=np.uint64)
        dqp = np.zeros(len(energy), dtype=np.float32)
    cost = lib().uavs3e_cuda_loka_finish(cfg.ctypes.data, t.ctypes.data,
                                         energy.ctypes.data if energy is not None else None, C.byref(icost),
                                         icost_uv, dqp.ctypes.data if dqp is not None else None)
    return cost, icost.value, (icost_uv[0], icost_uv[1]), dqp


def profile_enable(on=True):
    lib().uavs3e_cuda_profile_enable(1 if on else 0)


def measure_sad4_rate():
    """(ops/s, ops per clock per SM) of vabsdiff4-with-accumulate on the current device"""
    a, b = C.c_double(), C.c_double()
    check(lib().uavs3e_cuda_measure_sad4_rate(C.byref(a), C.byref(b)), "measure_sad4_rate")
    return a.value, b.value


def measure_dp2a_rate():
    """(ops/s, ops per clock per SM) of dp2a (2 multiply-adds each) on the current device"""
    a, b = C.c_double(), C.c_double()
    check(lib().uavs3e_cuda_measure_dp2a_rate(C.byref(a), C.byref(b)), "measure_dp2a_rate")
    return a.value, b.value


def launch_count():
    return int(lib().uavs3e_cuda_launch_count())


def profile_collect():
    """{kernel: (total_ms, launches)} since the last collect"""
    ms = (C.c_double * 12)()
    cnt = (C.c_int * 12)()
    check(lib().uavs3e_cuda_profile_collect(ms, cnt, 12), "profile_collect")
    return {k: (ms[i], cnt[i]) for i, k in enumerate(PROF_KERNELS)}


# the ten block shapes of the motion search, in result order
ME_SHAPES = ((8, 8), (16, 8), (8, 16), (16, 16), (32, 16), (16, 32), (32, 32), (64, 32), (32, 64), (64, 64))


def me_block_table():
    """(x, y, w, h) of the 169 blocks of a 64x64 CTU in result order: the shapes of ME_SHAPES,
    each in raster order.  Plain Python: the CPU baseline uses it without loading the library;
    uavs3e_cuda_me_block_table returns the same table (tests/test_capi.py)."""
    return np.array([(x, y, w, h) for w, h in ME_SHAPES for y in range(0, 64, h) for x in range(0, 64, w)],
                    dtype=np.int32)


def me_blocks(width, height):
    """(x, y, w, h, ctu, local) of every result slot in [ctu][block] order."""
    t = me_block_table()
    cw, ch = (width + 63) // 64, (height + 63) // 64
    ctu = np.arange(cw * ch, dtype=np.int32)
    out = np.zeros((cw * ch, len(t), 6), dtype=np.int32)
    out[:, :, 0] = (ctu % cw)[:, None] * 64 + t[None, :, 0]
    out[:, :, 1] = (ctu // cw)[:, None] * 64 + t[None, :, 1]
    out[:, :, 2] = t[None, :, 2]
    out[:, :, 3] = t[None, :, 3]
    out[:, :, 4] = ctu[:, None]
    out[:, :, 5] = np.arange(len(t), dtype=np.int32)[None, :]
    return out.reshape(-1, 6)


class MotionSearch:
    """Batched motion-search session (uavs3e_cuda_me_*)."""

    def __init__(self, width, height, n_refs=2, search_range=64, pad=144):
        L = lib()
        self.h = L.uavs3e_cuda_me_open(width, height, n_refs, search_range, pad)
        if not self.h:
            check(L.uavs3e_cuda_status() or -1, "uavs3e_cuda_me_open")
        self.width, self.height, self.n_refs, self.range, self.pad = width, height, n_refs, search_range, pad
        self.n_results = L.uavs3e_cuda_me_num_results(self.h)
        self.stride = L.uavs3e_cuda_me_plane_stride(self.h)

    def close(self):
        if self.h:
            lib().uavs3e_cuda_me_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_ref(self, slot, plane):
        plane = np.ascontiguousarray(plane, dtype=np.uint8)
        check(lib().uavs3e_cuda_me_set_ref(self.h, slot, plane.ctypes.data, plane.strides[0]), "me_set_ref")

    def set_ref_device(self, slot, d_ptr, stride, stream=None):
        check(lib().uavs3e_cuda_me_set_ref_device(self.h, slot, d_ptr, stride, stream), "me_set_ref_device")

    def run(self, org, lambda_mv, out=None):
        org = np.ascontiguousarray(org, dtype=np.uint8)
        if out is None:
            out = np.zeros(self.n_results, dtype=ME_RESULT)
        check(lib().uavs3e_cuda_me_run(self.h, org.ctypes.data, org.strides[0], lambda_mv, out.ctypes.data), "me_run")
        return out

    def run_ptr(self, org_ptr, i_org, lambda_mv, out_ptr):
        """host pointers (e.g. pinned buffers) in and out; synchronous"""
        check(lib().uavs3e_cuda_me_run(self.h, org_ptr, i_org, lambda_mv, out_ptr), "me_run")

    def run_device(self, d_org, i_org, lambda_mv, d_out, stream=None):
        check(lib().uavs3e_cuda_me_run_device(self.h, d_org, i_org, lambda_mv, d_out, stream), "me_run_device")

    def frame_graph(self, slot, d_ref, i_src, d_org, i_org, lambda_mv, d_out, stream=None):
        """set_ref_device(slot, d_ref) + run_device(d_org) replayed as a captured CUDA graph"""
        check(lib().uavs3e_cuda_me_frame_graph(self.h, slot, d_ref, i_src, d_org, i_org, lambda_mv, d_out, stream),
              "me_frame_graph")

    def frame_ptr(self, slot, ref_ptr, i_ref, org_ptr, i_org, lambda_mv, out_ptr):
        """host pointers: set_ref(slot, ref) + run(org) as one graph replay and one synchronisation"""
        check(lib().uavs3e_cuda_me_frame(self.h, slot, ref_ptr, i_ref, org_ptr, i_org, lambda_mv, out_ptr),
              "me_frame")

    def plane_ptr(self, slot, phase):
        return lib().uavs3e_cuda_me_plane(self.h, slot, phase)

    def tz(self, pic, org, reqs):
        """me_search_tz calls (TZ_REQ array) against the session's references; returns TZ_OUT"""
        org = np.ascontiguousarray(org, dtype=np.uint8)
        reqs = np.ascontiguousarray(reqs, dtype=TZ_REQ)
        out = np.zeros(max(1, len(reqs)), dtype=TZ_OUT)
        p = np.array(pic, dtype=np.int32)
        check(lib().uavs3e_cuda_me_tz(self.h, p.ctypes.data, org.ctypes.data, org.strides[0], reqs.ctypes.data,
                                      len(reqs), out.ctypes.data), "me_tz")
        return out[:len(reqs)]

    def affine(self, org, reqs):
        """affine_me_gradient calls (AFFME_REQ array) against the session's references; returns
        AFFME_OUT"""
        org = np.ascontiguousarray(org, dtype=np.uint8)
        reqs = np.ascontiguousarray(reqs, dtype=AFFME_REQ)
        out = np.zeros(max(1, len(reqs)), dtype=AFFME_OUT)
        check(lib().uavs3e_cuda_me_affine(self.h, org.ctypes.data, org.strides[0], reqs.ctypes.data, len(reqs),
                                          out.ctypes.data), "me_affine")
        return out[:len(reqs)]

    def set_ref_chroma(self, slot, u, v):
        u = np.ascontiguousarray(u, dtype=np.uint8)
        v = np.ascontiguousarray(v, dtype=np.uint8)
        assert u.strides[0] == v.strides[0]
        check(lib().uavs3e_cuda_me_set_ref_chroma(self.h, slot, u.ctypes.data, v.ctypes.data, u.strides[0]),
              "me_set_ref_chroma")

    def chroma_plane_ptr(self, slot, c):
        return lib().uavs3e_cuda_me_chroma_plane(self.h, slot, c)

    def chroma_stride(self):
        return lib().uavs3e_cuda_me_chroma_stride(self.h)

    def mc_cu(self, reqs, out_bytes):
        """com_mc_cu for every MC_REQ against the session's references; returns the output bytes"""
        reqs = np.ascontiguousarray(reqs, dtype=MC_REQ)
        out = np.zeros(max(1, out_bytes), dtype=np.uint8)
        check(lib().uavs3e_cuda_mc_cu(self.h, reqs.ctypes.data, len(reqs), out.ctypes.data, out_bytes), "mc_cu")
        return out[:out_bytes]


    def mc_affine(self, reqs, out_bytes):
        """com_mc_cu_affine for every AFFINE_REQ against the session's references"""
        reqs = np.ascontiguousarray(reqs, dtype=AFFINE_REQ)
        out = np.zeros(max(1, out_bytes), dtype=np.uint8)
        check(lib().uavs3e_cuda_mc_affine(self.h, reqs.ctypes.data, len(reqs), out.ctypes.data, out_bytes),
              "mc_affine")
        return out[:out_bytes]


AFFINE_REQ = np.dtype([("x", "<i2"), ("y", "<i2"), ("w", "u1"), ("h", "u1"), ("slot", "i1", (2,)), ("cp_num", "u1"),
                       ("sub8", "u1"), ("pad", "u1", (2,)), ("cpmv", "<i4", (2, 3, 2)), ("out_offset", "<u4")])


def mc_affine_device(width, height, d_planes, i_ref, pad, d_chroma, i_c, pad_c, d_reqs, n, d_out, out_bytes,
                     stream=None):
    """device form of com_mc_cu_affine over a list of CUs"""
    a = (C.c_void_p * len(d_planes))(*d_planes)
    c = (C.c_void_p * len(d_chroma))(*d_chroma)
    if stream is None:
        import torch
        stream = torch.cuda.current_stream().cuda_stream
    check(lib().uavs3e_cuda_mc_affine_device(width, height, a, len(d_planes) // 16, i_ref, pad, c, i_c, pad_c, d_reqs,
                                             n, d_out, out_bytes, stream), "mc_affine_device")


MC_REQ = np.dtype([("x", "<i2"), ("y", "<i2"), ("w", "u1"), ("h", "u1"), ("slot", "i1", (2,)),
                   ("mv", "<i2", (2, 2)), ("channel", "u1"), ("pad", "u1", (3,)), ("out_offset", "<u4")])


def mc_cu_device(width, height, d_planes, i_ref, pad, d_chroma, i_c, pad_c, d_reqs, n, d_out, out_bytes,
                 stream=None):
    """device form of com_mc_cu over a list of CUs (addresses as ints)"""
    a = (C.c_void_p * len(d_planes))(*d_planes)
    c = (C.c_void_p * len(d_chroma))(*d_chroma)
    if stream is None:
        import torch
        stream = torch.cuda.current_stream().cuda_stream
    check(lib().uavs3e_cuda_mc_cu_device(width, height, a, len(d_planes) // 16, i_ref, pad, c, i_c, pad_c, d_reqs, n,
                                         d_out, out_bytes, stream), "mc_cu_device")


# ------------------------------------------------------------------ RDOQ of transform blocks
RDOQ_EST = np.dtype([("ctp", "<i4", (2,)), ("cbf", "<i4", (3, 2)), ("run", "<i4", (24, 2)), ("lvl", "<i4", (24, 2)),
                     ("lst", "<i4", (2, 6, 12, 2))])
RDOQ_REQ = np.dtype([("coef_offset", "<u4"), ("log2w", "u1"), ("log2h", "u1"), ("qp", "u1"), ("is_intra", "u1"),
                     ("ch_type", "u1"), ("slice_type", "u1"), ("est", "<u2"), ("pad", "<u4"), ("lambda_", "<i8")])


def rdoq(reqs, ests, coefs):
    """quant_non_zero (flat) for every RDOQ_REQ on host arrays: coefs (int16) updated in place;
    returns num_nz"""
    reqs = np.ascontiguousarray(reqs, dtype=RDOQ_REQ)
    ests = np.ascontiguousarray(ests, dtype=RDOQ_EST)
    assert coefs.dtype == np.int16 and coefs.flags["C_CONTIGUOUS"]
    nz = np.zeros(max(1, len(reqs)), dtype=np.int32)
    check(lib().uavs3e_cuda_rdoq(reqs.ctypes.data, len(reqs), ests.ctypes.data, len(ests), coefs.ctypes.data,
                                 coefs.size, nz.ctypes.data), "rdoq")
    return nz[:len(reqs)]


def quant_wq(reqs, wq4, wq8, coefs):
    """quant_non_zero with weighted quantisation for every RDOQ_REQ on host arrays: coefs (int16)
    updated in place; returns num_nz"""
    reqs = np.ascontiguousarray(reqs, dtype=RDOQ_REQ)
    wq4 = np.ascontiguousarray(wq4, dtype=np.uint8)
    wq8 = np.ascontiguousarray(wq8, dtype=np.uint8)
    assert coefs.dtype == np.int16 and coefs.flags["C_CONTIGUOUS"]
    nz = np.zeros(max(1, len(reqs)), dtype=np.int32)
    check(lib().uavs3e_cuda_quant_wq(reqs.ctypes.data, len(reqs), wq4.ctypes.data, wq8.ctypes.data, coefs.ctypes.data,
                                     coefs.size, nz.ctypes.data), "quant_wq")
    return nz[:len(reqs)]


def rdoq_device(d_reqs, n, d_ests, n_est, d_coefs, n_coefs, d_num_nz, stream=None):
    if stream is None:
        import torch
        stream = torch.cuda.current_stream().cuda_stream
    check(lib().uavs3e_cuda_rdoq_device(d_reqs, n, d_ests, n_est, d_coefs, n_coefs, d_num_nz, stream), "rdoq_device")


# ------------------------------------------------------------------ per-call TZ motion search
TZ_REQ = np.dtype([("x", "<i2"), ("y", "<i2"), ("w", "u1"), ("h", "u1"), ("ref_slot", "u1"), ("refi", "i1"),
                   ("num_refp", "u1"), ("mvr", "u1"), ("bi", "u1"), ("flags", "u1"), ("mvp", "<i2", (2,)),
                   ("mv", "<i2", (2,)), ("mv_ipel", "<i2", (2,)), ("other_mv", "<i2", (2,)), ("other_slot", "u1"),
                   ("pad0", "u1", (3,)), ("mot_bits_other", "<i4"), ("lambda_mv", "<u4"), ("dist", "<i4"),
                   ("pad1", "<i4")])
TZ_OUT = np.dtype([("mv", "<i2", (2,)), ("mv_ipel", "<i2", (2,)), ("cost", "<u8")])


def me_tz_device(pic, d_org, i_org, d_planes, i_ref, pad, d_reqs, n, d_out, stream=None):
    """device form: pic = (W, H, is_padding, max_search_range, gop_size); d_planes = slot-major
    list of 16 device addresses per reference"""
    p = np.array(pic, dtype=np.int32)
    arr = (C.c_void_p * len(d_planes))(*d_planes)
    if stream is None:
        import torch
        stream = torch.cuda.current_stream().cuda_stream
    check(lib().uavs3e_cuda_me_tz_device(p.ctypes.data, d_org, i_org, arr, len(d_planes) // 16, i_ref, pad, d_reqs,
                                         n, d_out, stream), "me_tz_device")


# ------------------------------------------------------------------ affine motion search
AFFME_BI, AFFME_UNI_START, AFFME_SUB8 = 1, 2, 4
AFFME_REQ = np.dtype([("x", "<i2"), ("y", "<i2"), ("w", "u1"), ("h", "u1"), ("ref_slot", "u1"), ("refi", "i1"),
                      ("num_refp", "u1"), ("mvr", "u1"), ("flags", "u1"), ("other_slot", "u1"), ("lambda_mv", "<u4"),
                      ("mot_bits_other", "<i4"), ("pad", "<i4"), ("mvp", "<i4", (2, 2)), ("mv", "<i4", (2, 2)),
                      ("other_mv", "<i4", (2, 2))])
AFFME_OUT = np.dtype([("mv", "<i4", (2, 2)), ("satd", "<u4"), ("bits", "<i4"), ("cost", "<u8")])


def me_affine_device(width, height, d_org, i_org, d_planes, i_ref, pad, d_reqs, n, d_out, stream=None):
    """device form of the affine search: d_planes = slot-major list of 16 device addresses per
    reference (only each slot's integer plane is read)"""
    arr = (C.c_void_p * len(d_planes))(*d_planes)
    if stream is None:
        import torch
        stream = torch.cuda.current_stream().cuda_stream
    check(lib().uavs3e_cuda_me_affine_device(width, height, d_org, i_org, arr, len(d_planes) // 16, i_ref, pad, d_reqs,
                                             n, d_out, stream), "me_affine_device")


# ------------------------------------------------------------------ intra mode candidates
RMD_REQ = np.dtype([("satd_row", "<u4"), ("pb_w", "u1"), ("pb_h", "u1"), ("mpm", "u1", (2,)), ("skip_ipd", "u1"),
                    ("fast", "u1"), ("range", "<u2"), ("ctx", "<i2", (7,)), ("pad", "u1", (6,)),
                    ("sqrt_lambda", "<f8"), ("inter_satd", "<u8"), ("satd_threshold", "<f8")])
RMD_OUT = np.dtype([("list", "i1", (5,)), ("count", "u1"), ("pad", "u1", (2,))])


def intra_rmd(satd, reqs):
    """make_ipred_list for every RMD_REQ on host arrays: satd (rows x 33, uint32); returns RMD_OUT"""
    satd = np.ascontiguousarray(satd, dtype=np.uint32)
    reqs = np.ascontiguousarray(reqs, dtype=RMD_REQ)
    out = np.zeros(max(1, len(reqs)), dtype=RMD_OUT)
    check(lib().uavs3e_cuda_intra_rmd(satd.ctypes.data, satd.size // 33, reqs.ctypes.data, len(reqs),
                                      out.ctypes.data), "intra_rmd")
    return out[:len(reqs)]


def intra_rmd_device(d_satd, n_rows, d_reqs, n, d_out, stream=None):
    if stream is None:
        import torch
        stream = torch.cuda.current_stream().cuda_stream
    check(lib().uavs3e_cuda_intra_rmd_device(d_satd, n_rows, d_reqs, n, d_out, stream), "intra_rmd_device")


# ------------------------------------------------------------------ coefficient rate
COEF_CTX = [("run", "<i2", (12,)), ("run_rdoq", "<i2", (12,)), ("level", "<i2", (12,)), ("last1", "<i2", (6,)),
            ("last2", "<i2", (12,))]
COEF_RATE_REQ = np.dtype([("coef_offset", "<u4"), ("log2w", "u1"), ("log2h", "u1"), ("ch_type", "u1"), ("pad", "u1"),
                          ("num_sig", "<u2"), ("range", "<u2")] + COEF_CTX)
COEF_RATE_OUT = np.dtype([("bits", "<u4"), ("range", "<u2"), ("pad", "<u2")] + COEF_CTX)


def coef_rate(levels, reqs):
    """lbac_enc_run_length_cc_rdo for every COEF_RATE_REQ on host levels (int16); returns COEF_RATE_OUT"""
    levels = np.ascontiguousarray(levels, dtype=np.int16)
    reqs = np.ascontiguousarray(reqs, dtype=COEF_RATE_REQ)
    out = np.zeros(max(1, len(reqs)), dtype=COEF_RATE_OUT)
    check(lib().uavs3e_cuda_coef_rate(reqs.ctypes.data, len(reqs), levels.ctypes.data, levels.size, out.ctypes.data),
          "coef_rate")
    return out[:len(reqs)]


def coef_rate_device(d_reqs, n, d_levels, n_levels, d_out, stream=None):
    if stream is None:
        import torch
        stream = torch.cuda.current_stream().cuda_stream
    check(lib().uavs3e_cuda_coef_rate_device(d_reqs, n, d_levels, n_levels, d_out, stream), "coef_rate_device")


AFFMVP_REQ = np.dtype([("scup", "<i4"), ("cu_width", "<i2"), ("lidx", "i1"), ("cur_refi", "i1"), ("mvr", "i1"),
                       ("pad", "i1", (3,))])
AFFMVP_OUT = np.dtype([("mvp", "<i4", (2, 2))])


def affine_mvp(ptr_cur, ref_ptr, map_mv, map_refi, i_scu, reqs):
    """uavs3e_cuda_affine_mvp: com_get_affine_mvp_scaling for every AFFMVP_REQ against the motion
    field map_mv int16 [rows * i_scu, 2, 2] / map_refi int8 [rows * i_scu, 2] (the encoder's layout:
    SCU (0, 0) at index i_scu + 1), ref_ptr int64 [n_ref, 2]; returns AFFMVP_OUT"""
    ref_ptr = np.ascontiguousarray(ref_ptr, dtype=np.int64)
    map_mv = np.ascontiguousarray(map_mv, dtype=np.int16)
    map_refi = np.ascontiguousarray(map_refi, dtype=np.int8)
    reqs = np.ascontiguousarray(reqs, dtype=AFFMVP_REQ)
    out = np.zeros(max(1, len(reqs)), dtype=AFFMVP_OUT)
    check(lib().uavs3e_cuda_affine_mvp(int(ptr_cur), ref_ptr.ctypes.data, len(ref_ptr), map_mv.ctypes.data,
                                       map_refi.ctypes.data, i_scu, len(map_refi) // i_scu, reqs.ctypes.data,
                                       len(reqs), out.ctypes.data), "affine_mvp")
    return out[:len(reqs)]


def affine_mvp_device(ptr_cur, d_ref_ptr, n_ref, d_map_mv, d_map_refi, i_scu, rows, d_reqs, n, d_out, d_err=None,
                      stream=None):
    check(lib().uavs3e_cuda_affine_mvp_device(int(ptr_cur), d_ref_ptr, n_ref, d_map_mv, d_map_refi, i_scu, rows,
                                              d_reqs, n, d_out, d_err, stream), "affine_mvp_device")


AFFMRG_PIC = np.dtype([("ptr", "<i8"), ("ref0_ptr", "<i8", (2,)), ("col_list_ptr", "<i8", (17,)), ("i_scu", "<i4"),
                       ("pic_width_in_scu", "<i4"), ("pic_height_in_scu", "<i4"), ("rows", "<i4"),
                       ("slice_type", "<i4"), ("log2_max_cuwh", "<i4")])
AFFMRG_REQ = np.dtype([("scup", "<i4"), ("cu_width", "<i2"), ("cu_height", "<i2")])
AFFMRG_OUT = np.dtype([("num", "<i4"), ("cp_num", "i1", (5,)), ("refi", "i1", (5, 2)), ("pad", "i1"),
                       ("cpmv", "<i4", (5, 2, 3, 2))])


def affine_merge(pic, map_mv, map_refi, map_scu, map_pos, col_mv, col_refi, reqs):
    """uavs3e_cuda_affine_merge: com_get_affine_merge_candidate for every AFFMRG_REQ; pic an
    AFFMRG_PIC record, the maps in the encoder's layout (SCU (0, 0) at index i_scu + 1): map_mv /
    col_mv int16 [rows * i_scu, 2, 2], map_refi / col_refi int8 [rows * i_scu, 2], map_scu uint8 and
    map_pos uint32 [rows * i_scu]; returns AFFMRG_OUT"""
    pic = np.ascontiguousarray(pic, dtype=AFFMRG_PIC).reshape(1)
    arrs = [np.ascontiguousarray(a, dtype=t) for a, t in ((map_mv, np.int16), (map_refi, np.int8), (map_scu, np.uint8),
                                                           (map_pos, np.uint32), (col_mv, np.int16),
                                                           (col_refi, np.int8))]
    reqs = np.ascontiguousarray(reqs, dtype=AFFMRG_REQ)
    out = np.zeros(max(1, len(reqs)), dtype=AFFMRG_OUT)
    check(lib().uavs3e_cuda_affine_merge(pic.ctypes.data, *[a.ctypes.data for a in arrs], reqs.ctypes.data, len(reqs),
                                         out.ctypes.data), "affine_merge")
    return out[:len(reqs)]


def affine_merge_device(pic, d_map_mv, d_map_refi, d_map_scu, d_map_pos, d_col_mv, d_col_refi, d_reqs, n, d_out,
                        d_err=None, stream=None):
    pic = np.ascontiguousarray(pic, dtype=AFFMRG_PIC).reshape(1)
    check(lib().uavs3e_cuda_affine_merge_device(pic.ctypes.data, d_map_mv, d_map_refi, d_map_scu, d_map_pos, d_col_mv,
                                                d_col_refi, d_reqs, n, d_out, d_err, stream), "affine_merge_device")
