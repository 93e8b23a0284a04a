"""GPU: uavs3e_cuda_me_search_noalloc, the motion search that allocates nothing.

It is for callers that cannot allocate device memory while they search a frame (a fixed memory
budget set up at start-up, or code that must not call cudaMalloc/cudaFree because they
synchronise the device).  The caller owns every buffer; the scratch is one static device array.
Its results must equal the allocating session entry point's (uavs3e_cuda_me_run_device) on the
same inputs, call after call -- the shared scratch keeps the previous call's contents, so two
calls in a row with different frames and lambdas are checked.
"""
import ctypes as C

import numpy as np
import pytest

from uavs3e_gb300.synth import lambda_mv_for_qp, motion_sequence

pytestmark = pytest.mark.gpu

W, H, REFS, RANGE, PAD = 320, 192, 2, 48, 144


def _declare(L):
    P, I = C.c_void_p, C.c_int
    L.uavs3e_cuda_me_search_noalloc.argtypes = [P, I, P, I, I, I, I, I, I, C.c_uint32, P, P]
    L.uavs3e_cuda_me_search_noalloc.restype = I
    L.uavs3e_cuda_pad_plane.argtypes = [P, I, I, I, I, P]
    L.uavs3e_cuda_subpel_planes.argtypes = [P, P, I, I, I, I, P]


class CallerPlanes:
    """reference planes owned by the caller (torch allocations made before the search)"""

    def __init__(self, torch, L, frames, stream):
        self.stride = ((W + 2 * PAD) + 15) & ~15
        rows = H + 2 * PAD
        self.buf = torch.zeros((len(frames), 16, rows * self.stride), dtype=torch.uint8, device="cuda")
        base = PAD * self.stride + PAD
        self.ptrs = []
        for r, f in enumerate(frames):
            view = self.buf[r, 0].view(rows, self.stride)
            view[PAD:PAD + H, PAD:PAD + W] = torch.from_numpy(f).cuda()
            p = [self.buf[r, q].data_ptr() + base for q in range(16)]
            assert L.uavs3e_cuda_pad_plane(p[0], W, H, PAD, self.stride, stream) == 0
            frac = (C.c_void_p * 15)(*p[1:])
            assert L.uavs3e_cuda_subpel_planes(p[0], frac, W, H, PAD, self.stride, stream) == 0
            self.ptrs += p


def session_results(gpu, frames, org, lam, rng):
    """the allocating session (the existing entry point) on the same inputs"""
    ms = gpu.MotionSearch(W, H, n_refs=REFS, search_range=rng, pad=PAD)
    for r, f in enumerate(frames):
        ms.set_ref(r, f)
    want = ms.run(org, lam)
    ms.close()
    return want


def noalloc_call(gpu, torch, planes, d_org, d_out, lam, rng):
    L = gpu.lib()
    stream = torch.cuda.current_stream().cuda_stream
    arr = (C.c_void_p * len(planes.ptrs))(*planes.ptrs)
    rc = L.uavs3e_cuda_me_search_noalloc(d_org.data_ptr(), W, arr, planes.stride, PAD, W, H, REFS, rng, lam,
                                         d_out.data_ptr(), stream)
    assert rc == 0, L.uavs3e_cuda_status_string()
    torch.cuda.synchronize()
    return d_out.cpu().numpy().view(gpu.ME_RESULT).copy()


def run_both(gpu, torch, frames, org, lam, rng=RANGE):
    L = gpu.lib()
    _declare(L)
    want = session_results(gpu, frames, org, lam, rng)
    planes = CallerPlanes(torch, L, frames, torch.cuda.current_stream().cuda_stream)
    d_org = torch.from_numpy(np.ascontiguousarray(org)).cuda()
    d_out = torch.zeros(len(want) * 32, dtype=torch.uint8, device="cuda")
    return noalloc_call(gpu, torch, planes, d_org, d_out, lam, rng), want


def test_noalloc_matches_session_twice_in_a_row(gpu):
    import torch
    seq = motion_sequence(W, H, 4, seed=21, n_rects=4)
    # call 1: refs (1, 0), org 2, QP 32
    got, want = run_both(gpu, torch, [seq[1], seq[0]], seq[2], lambda_mv_for_qp(32))
    assert np.array_equal(got, want)
    # call 2 right after: other frames and another lambda (new tables, reused scratch)
    got, want = run_both(gpu, torch, [seq[2], seq[1]], seq[3], lambda_mv_for_qp(40))
    assert np.array_equal(got, want)
    # call 3: the same size, range and lambda as call 2 with other frames (the tables already on
    # the device are reused), call 4: a smaller range (a shorter table upload)
    got, want = run_both(gpu, torch, [seq[1], seq[0]], seq[3], lambda_mv_for_qp(40))
    assert np.array_equal(got, want)
    got, want = run_both(gpu, torch, [seq[3], seq[2]], seq[1], lambda_mv_for_qp(40), rng=13)
    assert np.array_equal(got, want)


def test_noalloc_call_allocates_no_device_memory(gpu):
    # with every caller buffer made beforehand, a call changes neither the device's free memory
    # nor the caller's allocator: the scratch is the library's static array
    import torch
    L = gpu.lib()
    _declare(L)
    seq = motion_sequence(W, H, 3, seed=5, n_rects=3)
    planes = CallerPlanes(torch, L, [seq[1], seq[0]], torch.cuda.current_stream().cuda_stream)
    d_org = torch.from_numpy(np.ascontiguousarray(seq[2])).cuda()
    n = ((W + 63) // 64) * ((H + 63) // 64) * 169 * REFS
    d_out = torch.zeros(n * 32, dtype=torch.uint8, device="cuda")
    lam = lambda_mv_for_qp(30)
    first = noalloc_call(gpu, torch, planes, d_org, d_out, lam, RANGE)      # set-up call
    free0, alloc0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
    for qp in (30, 33):                              # a table-cache hit, then a new lambda
        noalloc_call(gpu, torch, planes, d_org, d_out, lambda_mv_for_qp(qp), RANGE)
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_allocated() == alloc0
    again = noalloc_call(gpu, torch, planes, d_org, d_out, lam, RANGE)
    assert np.array_equal(first, again)


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    L = gpu.lib()
    _declare(L)
    dummy = (C.c_void_p * 32)(*([1] * 32))
    # 3840x2160 is beyond the 510-CTU scratch: rejected before any device work
    rc = L.uavs3e_cuda_me_search_noalloc(1, 3840, dummy, 4128, PAD, 3840, 2160, 2, 64, 1000, 1, None)
    assert rc == -101
    assert b"static scratch" in L.uavs3e_cuda_status_string()
    L.uavs3e_cuda_clear_status()
    # more references than the scratch holds
    rc = L.uavs3e_cuda_me_search_noalloc(1, W, dummy, 624, PAD, W, H, 3, 64, 1000, 1, None)
    assert rc == -101
    L.uavs3e_cuda_clear_status()
