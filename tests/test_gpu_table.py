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
