"""Build recipe of libuavs3e_cuda.so (in-tree, sm_103a only).

Each .cu under csrc/ is compiled by nvcc in parallel and linked into
uavs3e_gb300/libuavs3e_cuda.so.  Run as ``python -m uavs3e_gb300.build`` or call build().
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libuavs3e_cuda.so")
PRELOAD = os.path.join(HERE, "libuavs3e_cuda_preload.so")
STAGECLK_LIB = os.path.join(HERE, "libuavs3e_cuda_stageclk.so")
PRELOAD_SRC = os.path.join(HERE, "dropin", "preload.c")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden", "--expt-relaxed-constexpr"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: libuavs3e_cuda needs the CUDA toolkit to build")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, ptxas_info=False, stage_clocks=False):
    """Builds the library (and the LD_PRELOAD wrapper); with stage_clocks, a separate
    libuavs3e_cuda_stageclk.so whose lattice keeps per-stage clocks (a profiling build)."""
    if stage_clocks:
        return _build_lib(os.path.join(HERE, "_build_stageclk"), STAGECLK_LIB, ["-DUAVS3E_LAT_STAGE_CLOCKS"], verbose,
                          ptxas_info)
    _build_lib(OBJ, LIB, [], verbose, ptxas_info)
    # the LD_PRELOAD wrapper that installs the entries into an unchanged encoder
    if _stale(PRELOAD, [PRELOAD_SRC, os.path.join(HERE, "dropin", "costlog.h"), LIB] + _headers()):
        cc = os.environ.get("CC", "gcc")
        cmd = [cc, "-O2", "-fPIC", "-shared", "-std=gnu11", "-Wall", "-o", PRELOAD, PRELOAD_SRC, "-L" + HERE,
               "-luavs3e_cuda", "-Wl,-rpath,$ORIGIN", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("preload build failed")
    return LIB


def _headers():
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h", ".inc"))]
    headers.append(os.path.join(HERE, "..", "include", "uavs3e_cuda.h"))
    headers += [os.path.join(HERE, "..", "include", f) for f in os.listdir(os.path.join(HERE, "..", "include"))]
    return headers


def _build_lib(obj_dir, lib_path, defines, verbose, ptxas_info):
    os.makedirs(obj_dir, exist_ok=True)
    nv = nvcc()
    headers = _headers()
    objs, jobs = [], []
    for src in sources():
        s = os.path.join(CSRC, src)
        o = os.path.join(obj_dir, src[:-3] + ".o")
        objs.append(o)
        if _stale(o, [s, __file__] + headers) or ptxas_info:
            cmd = [nv] + ARCH + NVCC_FLAGS + defines + (["-Xptxas", "-v"] if ptxas_info else []) + ["-c", s, "-o", o]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        res = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
    for cmd, r in zip(jobs, res):
        if verbose or ptxas_info or r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if jobs or not os.path.exists(lib_path):
        cmd = [nv] + ARCH + ["-shared", "-o", lib_path] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return lib_path


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
    print(LIB)
