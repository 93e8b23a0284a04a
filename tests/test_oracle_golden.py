"""CPU: the oracle restatement against the reference's golden digests (tests/golden/golden.json),
and -- where the reference build is present -- directly against the reference on extra seeds."""
import json
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402

GOLDEN = json.load(open(os.path.join(HERE, "golden", "golden.json")))["cases"]


def _id(c):
    return c["kernel"] + "-" + "-".join(f"{k}{v}" for k, v in c["params"].items())


@pytest.mark.parametrize("case", GOLDEN, ids=[_id(c) for c in GOLDEN])
def test_oracle_matches_reference_golden(oracle, case):
    assert cases.run_case(oracle, case) == case["md5"]


def test_golden_covers_every_kernel():
    assert {c["kernel"] for c in GOLDEN} == set(cases.RUNNERS)


@pytest.mark.parametrize("kernel", sorted(cases.RUNNERS))
def test_oracle_matches_reference_new_seeds(oracle, ref, kernel):
    for c in cases.all_cases():
        if c["kernel"] != kernel:
            continue
        c = dict(c, seed=c["seed"] + 77777)
        assert cases.run_case(oracle, c) == cases.run_case(ref, c), _id(c)
