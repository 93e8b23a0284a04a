"""GPU: the unchanged reference encoder on libuavs3e_cuda's kernel-table entries.

The reference encoder application (oracle/_ref/uavs3enc, compiled from the uavs3e sources by
`make -C oracle ref REF=<uavs3e source tree>`) encodes the seeded 416x240 8-bit 4:2:0 sequence of
the CPU-runnable configuration (low delay, QP 37, 64x64 CTU, one thread) twice: with its own C
kernel table, and with uavs3e_cuda_preload.so, which installs every hot-path member of the table
as the GPU entries right after uavs3e_create.  The bitstream and the reconstruction must be
identical, the library must report status 0 and must have launched kernels, and the record of
every cost call (uavs3e_gb300/dropin/costlog.h: each SAD / SAD x3 / x4 / SSD / SATD call's
block size and result, in call order) must equal the reference table's record.

Every call of the encoder's search loops is then one GPU round trip (the per-call entries; the
batched entry points are the throughput path), so this is a boundary check, not a speed run.
UAVS3E_DROPIN_FRAMES sets the frame count (default 2: one intra and one inter picture).
Skipped where the encoder is not built (the uavs3e sources are not on every GPU host).
"""
import os
import re
import time

import pytest

from test_dropin_encode import ENC, SHIM, costlog, encode, reference_costlog, write_yuv

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not (os.path.exists(ENC) and os.path.exists(SHIM)),
                                 reason="reference encoder not built on this host (make -C oracle ref REF=<uavs3e "
                                        "source tree>)")]

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PRELOAD = os.path.join(ROOT, "uavs3e_gb300", "libuavs3e_cuda_preload.so")


def test_reference_encoder_on_gpu_entries_gives_the_reference_bitstream(gpu, tmp_path):
    n = int(os.environ.get("UAVS3E_DROPIN_FRAMES", "2"))
    tmp = str(tmp_path)
    write_yuv(os.path.join(tmp, "in.yuv"), n)
    t0 = time.perf_counter()
    plain, _ = encode(tmp, "plain", n_frames=n)
    t1 = time.perf_counter()
    got, log = encode(tmp, "gpu", {"LD_PRELOAD": PRELOAD, "UAVS3E_CUDA_COSTLOG": "1"}, n_frames=n, timeout=5400)
    t2 = time.perf_counter()
    ref_md5, ref_costs = reference_costlog(tmp, n)
    assert ref_md5 == plain
    assert costlog(log) == ref_costs, f"cost calls {costlog(log)} != reference {ref_costs}"
    assert "kernel table installed (GPU entries)" in log
    m = re.search(r"uavs3e_cuda_preload: status (-?\d+) \(([^)]*)\), (\d+) kernel launches", log)
    assert m, log[-2000:]
    assert int(m.group(1)) == 0, m.group(2)
    assert int(m.group(3)) > 0
    assert got == plain, f"md5 (bitstream, reconstruction) {got} != reference {plain}"
    print(f"\ndrop-in encode, {n} frames: md5 {plain[0]} (both); reference C table {t1 - t0:.1f} s, "
          f"GPU entries {t2 - t1:.1f} s, {m.group(3)} kernel launches; cost calls {sum(ref_costs[:5])} "
          f"(sad, x3, x4, ssd, satd = {ref_costs[:5]}), record hash {ref_costs[5]} (both)")


def test_gpu_entries_under_wavefront_threads(gpu, tmp_path):
    # the encoder's WPP threads call the shared kernel table concurrently; each thread stages its
    # calls separately (per-thread buffers and stream), so one frame coded with 4 threads on the
    # GPU entries gives the reference's 4-thread bitstream
    tmp = str(tmp_path)
    write_yuv(os.path.join(tmp, "in.yuv"), 1)
    plain, _ = encode(tmp, "plain4", n_frames=1, wpp_threads=4)
    got, log = encode(tmp, "gpu4", {"LD_PRELOAD": PRELOAD}, n_frames=1, timeout=3600, wpp_threads=4)
    assert "kernel table installed (GPU entries)" in log
    m = re.search(r"uavs3e_cuda_preload: status (-?\d+) \(([^)]*)\), (\d+) kernel launches", log)
    assert m and int(m.group(1)) == 0, log[-2000:]
    assert got == plain, f"md5 (bitstream, reconstruction) {got} != reference {plain}"
