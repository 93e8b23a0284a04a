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
    L.uavs3e_cuda_me_plane.restype = P
    L.uavs3e_cuda_me_plane.argtypes = [P, I, I]
    L.uavs3e_cuda_me_plane_stride.argtypes = [P]
    L.uavs3e_cuda_lattice_cus.argtypes = [I, I, P, I]
    L.uavs3e_cuda_intra_lattice_device.argtypes = [P, I, P, I, I, I, P, I, I, P, I, I, P, P, P]
    L.uavs3e_cuda_profile_enable.argtypes = [I]
    L.uavs3e_cuda_launch_count.restype = C.c_ulonglong
    L.uavs3e_cuda_profile_collect.argtypes = [P, P, I]


def check(rc, what="uavs3e_cuda"):
    if rc != 0:
        L = lib()
        msg = L.uavs3e_cuda_status_string().decode()
        L.uavs3e_cuda_clear_status()
        raise CudaError(f"{what} failed ({rc}): {msg}")
    return rc


def init(device=0):
    check(lib().uavs3e_cuda_init(device), "uavs3e_cuda_init")


PROF_KERNELS = ("pad", "subpel_planes", "me_int", "me_sub", "intra_lattice")

CU = np.dtype([("x", "<i2"), ("y", "<i2"), ("w", "u1"), ("h", "u1"), ("pad", "<u2")])
LAT_Q = np.dtype([("ssd", "<u4"), ("coef_hash", "<u4"), ("num_nz", "<u2"), ("last_nz", "<i2"), ("sum_abs", "<u4")])


def lattice_cus(width, height):
    """the 23-shape CU lattice of a picture (largest shapes first)"""
    n = lib().uavs3e_cuda_lattice_cus(width, height, None, 0)
    out = np.zeros(n, dtype=CU)
    lib().uavs3e_cuda_lattice_cus(width, height, out.ctypes.data, n)
    return out


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
    ms = (C.c_double * 8)()
    cnt = (C.c_int * 8)()
    check(lib().uavs3e_cuda_profile_collect(ms, cnt, 8), "profile_collect")
    return {k: (ms[i], cnt[i]) for i, k in enumerate(PROF_KERNELS)}


def me_block_table():
    t = (C.c_int * (169 * 4))()
    lib().uavs3e_cuda_me_block_table(t)
    return np.array(t, dtype=np.int32).reshape(169, 4)


def me_blocks(width, height):
    """(x, y, w, h, ctu, local) of every result slot in [ctu][block] order."""
    t = me_block_table()
    cw, ch = (width + 63) // 64, (height + 63) // 64
    out = []
    for cy in range(ch):
        for cx in range(cw):
            for i, (bx, by, bw, bh) in enumerate(t):
                out.append((cx * 64 + bx, cy * 64 + by, bw, bh, cy * cw + cx, i))
    return np.array(out, dtype=np.int32)


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

    def plane_ptr(self, slot, phase):
        return lib().uavs3e_cuda_me_plane(self.h, slot, phase)
