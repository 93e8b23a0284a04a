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


def encode(tmp, tag, env_extra=None, n_frames=8, timeout=600):
    env = dict(os.environ)
    env.update(env_extra or {})
    bs, rec = os.path.join(tmp, tag + ".bin"), os.path.join(tmp, tag + "_rec.yuv")
    cmd = [ENC, "-i", os.path.join(tmp, "in.yuv"), "-w", "416", "-h", "240", "-d", "8", "-f", str(n_frames), "-q", "37",
           "-p", "0", "-g", "0", "--ctu_size", "64", "--wpp_threads", "1", "--frm_threads", "1", "--fps_num", "30",
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
