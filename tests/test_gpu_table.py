"""GPU: the kernel-table entries (include/uavs3e_cuda_table.h) against the reference's golden
digests, and the installer against the table layout."""
import json
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402
from gpu_table import GpuTable  # noqa: E402

GOLDEN = json.load(open(os.path.join(HERE, "golden", "golden.json")))["cases"]
# kernels whose golden runner only calls table entries (com_had, the neighbour fetch, transform()
# and com_invqt are the encoder's callers of the table, not entries)
ENTRY_KERNELS = {"sad", "satd_tile", "ipflt", "ipflt_ext", "ipcpy", "if_luma_frame", "pel", "intra", "ang_entry",
                 "fdct2", "dct87", "quant", "dquant"}
SEL = [c for c in GOLDEN if c["kernel"] in ENTRY_KERNELS]


def _id(c):
    return c["kernel"] + "-" + "-".join(f"{k}{v}" for k, v in c["params"].items())


@pytest.fixture(scope="module")
def table(gpu):
    return GpuTable(gpu.lib())


@pytest.mark.gpu
@pytest.mark.parametrize("case", SEL, ids=[_id(c) for c in SEL])
def test_table_entry_matches_reference_golden(table, gpu, case):
    got = cases.run_case(table, case)
    st = gpu.lib().uavs3e_cuda_status()
    assert st == 0, gpu.lib().uavs3e_cuda_status_string()
    assert got == case["md5"]


@pytest.mark.gpu
def test_table_entries_from_concurrent_threads(table, oracle):
    """the encoder's WPP and frame threads share one table: 8 host threads call SAD, SATD and
    filter entries at once (ctypes releases the interpreter lock during each call), each with
    its own blocks, and every result equals the oracle's"""
    import threading

    import numpy as np
    rng = np.random.default_rng(123)
    jobs = []
    for t in range(8):
        work = []
        for k in range(60):
            w = int(rng.choice([4, 8, 16, 32, 64]))
            h = int(rng.choice([4, 8, 16]))
            o = rng.integers(0, 256, (h, w + 8), dtype=np.uint8)
            p = rng.integers(0, 256, (h + 8, w + 16), dtype=np.uint8)
            work.append((w, h, o, p))
        jobs.append(work)
    want = [[(oracle.sad(w, h, o.ctypes.data, w + 8, p.ctypes.data, w + 16),
              oracle.satd_tile(8, 8, p.ctypes.data, w + 16, o.ctypes.data, w + 8) if w >= 8 and h >= 8 else 0)
             for (w, h, o, p) in work] for work in jobs]
    got = [[None] * len(w) for w in jobs]
    errors = []

    def run(t):
        try:
            for k, (w, h, o, p) in enumerate(jobs[t]):
                s = table.sad(w, h, o.ctypes.data, w + 8, p.ctypes.data, w + 16)
                d = table.satd_tile(8, 8, p.ctypes.data, w + 16, o.ctypes.data, w + 8) if w >= 8 and h >= 8 else 0
                got[t][k] = (s, d)
        except Exception as e:     # reported below, after every thread has ended
            errors.append(e)

    threads = [threading.Thread(target=run, args=(t,)) for t in range(8)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors[0]
    assert got == want
