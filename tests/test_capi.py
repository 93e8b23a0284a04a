"""CPU: the C-ABI library builds, loads without a GPU, exports every function the public headers
declare, and fails cleanly (no CPU fallback) when no device is present."""
import ctypes as C
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        names |= set(re.findall(r"UAVS3E_CUDA_API\s+[\w\s\*]+?\b(uavs3e_cuda_\w+)\s*\(", txt))
    return names


@pytest.fixture(scope="module")
def lib():
    import uavs3e_gb300 as u
    u.build()
    return u.lib()


def test_headers_declare_the_table_and_batched_api():
    names = declared_functions()
    assert len(names) > 150
    for n in ("uavs3e_cuda_install", "uavs3e_cuda_me_run", "uavs3e_cuda_intra_lattice_device",
              "uavs3e_cuda_subpel_planes", "uavs3e_cuda_cost_sad_64", "uavs3e_cuda_trans_dct2_w64_h64",
              "uavs3e_cuda_intra_pred_ang_32", "uavs3e_cuda_quant_rdoq"):
        assert n in names


def test_library_exports_every_declared_function(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib._name], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (uavs3e_cuda_\w+)", out))
    missing = declared_functions() - exported
    assert not missing, sorted(missing)
    for n in declared_functions():
        assert hasattr(lib, n)


def test_headers_compile_as_c():
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        subprocess.run(["gcc", "-fsyntax-only", "-std=c99", "-Wall", "-Werror", "-x", "c", h], check=True)


def test_no_gpu_fails_loudly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib.uavs3e_cuda_status_string.restype = C.c_char_p
    lib.uavs3e_cuda_clear_status()
    assert lib.uavs3e_cuda_init(0) == -111
    assert lib.uavs3e_cuda_status() == -111
    lib.uavs3e_cuda_clear_status()
    # a kernel-table entry with no device: no result, error recorded, outputs untouched
    import numpy as np
    o = np.arange(64, dtype=np.uint8)
    p = np.zeros(64, dtype=np.uint8)
    lib.uavs3e_cuda_cost_sad_8.restype = C.c_uint32
    assert lib.uavs3e_cuda_cost_sad_8(o.ctypes.data, 8, p.ctypes.data, 8, 8) == 0
    assert lib.uavs3e_cuda_status() != 0
    lib.uavs3e_cuda_clear_status()
    table = (C.c_char * 2072)()
    assert lib.uavs3e_cuda_install(table) != 0
    assert bytes(table) == b"\0" * 2072
    lib.uavs3e_cuda_clear_status()


def test_table_twin_has_reference_layout(ref):
    # oracle/ref_glue.c static-asserts every member offset of uavs3e_cuda_funs_t against the
    # reference's funs_handle_t; building it is the check, the size is read back here
    ref.L.refk_table_size.restype = C.c_size_t
    assert ref.L.refk_table_size() == 2072


def test_block_table_matches_library(lib):
    # the library's 169-block CTU table (a host query, no device needed) equals the package's
    # plain-Python table used by the CPU baseline
    import numpy as np
    import uavs3e_gb300 as u
    t = (C.c_int * (169 * 4))()
    assert lib.uavs3e_cuda_me_block_table(t) == 0
    assert np.array_equal(np.array(t, dtype=np.int32).reshape(169, 4), u.me_block_table())
    b = u.me_blocks(200, 136)
    assert b.shape == (4 * 3 * 169, 6)
    assert tuple(b[169 * 5 + 3]) == (64 + 24, 64, 8, 8, 5, 3)
