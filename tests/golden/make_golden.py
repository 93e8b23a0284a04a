"""Generate tests/golden/golden.json: md5 digests of the reference's own C kernels on the
seeded cases of cases.py.

Run where the uavs3e source tree is available (it builds oracle/_ref from it):
    python tests/golden/make_golden.py /path/to/uavs3e      (or set UAVS3E_REF_TREE)
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import cases  # noqa: E402
import pyoracle  # noqa: E402


def main():
    ref_dir = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("UAVS3E_REF_TREE")
    if not ref_dir:
        sys.exit("usage: make_golden.py <uavs3e source tree> (or set UAVS3E_REF_TREE)")
    if not pyoracle.build_ref(ref_dir):
        sys.exit(f"reference sources not found at {ref_dir}")
    R = pyoracle.RefLib()
    out = []
    for c in cases.all_cases():
        out.append(dict(c, md5=cases.run_case(R, c)))
    path = os.path.join(HERE, "golden.json")
    with open(path, "w") as f:
        json.dump({"source": "uavs3e C kernel table (uavs3e_funs_init_c) and exported helpers, 8-bit build",
                   "generator": "tests/golden/make_golden.py", "cases": out}, f, indent=0)
    print(f"{len(out)} cases -> {path}")


if __name__ == "__main__":
    main()
