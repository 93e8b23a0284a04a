"""CPU: the kernel-table boundary as a drop-in, on the reference encoder itself.

The reference encoder (oracle/_ref/uavs3enc, compiled from the reference's own sources by
`make -C oracle ref`) encodes the 416x240 8-bit 4:2:0 sequence of the CPU-runnable
configuration (8 frames, low delay, QP 37, 64x64 CTU, one thread) twice: with its own kernel
table, and with every hot-path member swapped for the oracle restatement (oracle/dropin.c,
LD_PRELOAD) -- the code the GPU entries are checked against bit for bit.  The bitstream and
reconstruction md5 must be identical; a planted mistake (one more unit of 8x8 SATD) must change
the bitstream.  Skipped where the reference is not built (the GPU host).
"""
import hashlib
import os
import re
import subprocess

import numpy as np
import pytest

from uavs3e_gb300.synth import config0_sequence

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ENC = os.path.join(ROOT, "oracle", "_ref", "uavs3enc")
SHIM = os.path.join(ROOT, "oracle", "_ref", "libdropin.so")

pytestmark = pytest.mark.skipif(not (os.path.exists(ENC) and os.path.exists(SHIM)),
                                reason="reference encoder not built here (make -C oracle ref)")


def write_yuv(path, n_frames=8):
    """luma from the seeded generator; chroma = 2x2-averaged luma + 16 (U) / - 16 (V)"""
    with open(path, "wb") as f:
        for y in config0_sequence(seed=0, n_frames=n_frames):
            t = y.astype(np.int32)
            d = (t[0::2, 0::2] + t[1::2, 0::2] + t[0::2, 1::2] + t[1::2, 1::2] + 2) >> 2
            f.write(y.tobytes())
            f.write(np.clip(d + 16, 0, 255).astype(np.uint8).tobytes())
            f.write(np.clip(d - 16, 0, 255).astype(np.uint8).tobytes())


def encode(tmp, tag, env_extra=None, n_frames=8, timeout=600, wpp_threads=1):
    env = dict(os.environ)
    env.update(env_extra or {})
    bs, rec = os.path.join(tmp, tag + ".bin"), os.path.join(tmp, tag + "_rec.yuv")
    cmd = [ENC, "-i", os.path.join(tmp, "in.yuv"), "-w", "416", "-h", "240", "-d", "8", "-f", str(n_frames), "-q", "37",
           "-p", "0", "-g", "0", "--ctu_size", "64", "--wpp_threads", str(wpp_threads), "--frm_threads", "1",
           "--fps_num", "30",
           "--fps_den", "1", "-v", "0", "-o", bs, "-r", rec]
    # the encoder writes psnr.txt into its working directory: run it inside the test's folder
    r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=timeout, cwd=tmp)
    assert r.returncode == 0, r.stderr[-2000:]
    md5 = [hashlib.md5(open(p, "rb").read()).hexdigest() for p in (bs, rec)]
    return md5, r.stderr + r.stdout


def test_oracle_kernel_table_encodes_the_reference_bitstream(tmp_path):
    tmp = str(tmp_path)
    write_yuv(os.path.join(tmp, "in.yuv"))
    plain, _ = encode(tmp, "plain")
    dropin, log = encode(tmp, "dropin", {"LD_PRELOAD": SHIM})
    assert "kernel table replaced by the oracle restatement" in log
    assert dropin == plain
    planted, log = encode(tmp, "planted", {"LD_PRELOAD": SHIM, "UAVS3E_DROPIN_PLANT": "satd"})
    assert "kernel table replaced" in log
    assert planted[0] != plain[0]


ALL_FAMILIES = "intra,mc,frame,recon,dquant,itx,tx,sad,ssd,satd,pel,quant"


def costlog(log):
    """the 'costlog:' line of an encode's stderr (uavs3e_gb300/dropin/costlog.h) as a tuple"""
    m = re.search(r"costlog: sad (\d+) sad_x3 (\d+) sad_x4 (\d+) ssd (\d+) satd (\d+) hash ([0-9a-f]{16})", log)
    assert m, log[-2000:]
    return tuple(int(v) for v in m.groups()[:5]) + (m.group(6),)


def reference_costlog(tmp, n_frames):
    """md5 and cost-call record of the reference's own kernel table (every family left in place,
    its cost members wrapped by the record)"""
    md5, log = encode(tmp, "refcost", {"LD_PRELOAD": SHIM, "UAVS3E_DROPIN_SKIP": ALL_FAMILIES,
                                       "UAVS3E_DROPIN_COSTLOG": "1"}, n_frames=n_frames)
    return md5, costlog(log)


def test_cost_calls_of_the_oracle_table_match_the_reference(tmp_path):
    # every SAD / SAD x3 / x4 / SSD / SATD call of a 2-frame encode returns the same value, in
    # the same order, through the oracle restatement as through the reference's own functions
    tmp = str(tmp_path)
    write_yuv(os.path.join(tmp, "in.yuv"), 2)
    plain, _ = encode(tmp, "plain", n_frames=2)
    ref_md5, ref_log = reference_costlog(tmp, 2)
    assert ref_md5 == plain
    assert sum(ref_log[:5]) > 100000
    md5, log = encode(tmp, "oracle", {"LD_PRELOAD": SHIM, "UAVS3E_DROPIN_COSTLOG": "1"}, n_frames=2)
    assert md5 == plain
    assert costlog(log) == ref_log
    # a planted SATD mistake shows up in the record
    _, log = encode(tmp, "planted", {"LD_PRELOAD": SHIM, "UAVS3E_DROPIN_COSTLOG": "1", "UAVS3E_DROPIN_PLANT": "satd"},
                    n_frames=2)
    assert costlog(log)[5] != ref_log[5]


def test_oracle_kernel_table_under_wavefront_threads(tmp_path):
    # 4 WPP threads share the kernel table: one frame through the oracle table gives the
    # reference's 4-thread bitstream (the reference's own output is the same on every run)
    tmp = str(tmp_path)
    write_yuv(os.path.join(tmp, "in.yuv"), 1)
    plain, _ = encode(tmp, "plain4", n_frames=1, wpp_threads=4)
    again, _ = encode(tmp, "again4", n_frames=1, wpp_threads=4)
    assert again == plain
    dropin, log = encode(tmp, "dropin4", {"LD_PRELOAD": SHIM}, n_frames=1, wpp_threads=4)
    assert "kernel table replaced by the oracle restatement" in log
    assert dropin == plain
