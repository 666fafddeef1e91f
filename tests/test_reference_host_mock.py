"""The reference's own CPU path, built from its unchanged sources by
oracle/ref_cpu/build_mock.py (its host mock backend with exact GMP
verification of every site): on the C1 configuration and on the reference's
own oracle cases its stdout equals the golden fixtures, which pins them a
further way.  Skipped where the binary was not built (no reference tree)."""

import hashlib
import os
import subprocess
from pathlib import Path

import pytest

MOCK = Path(__file__).resolve().parent.parent / "oracle" / "_ref" / "mock_ratpoints_gpu"
pytestmark = pytest.mark.skipif(not MOCK.exists(), reason="reference host mock not built")


def run(args, devices=8):
    env = dict(os.environ, RATPOINTS_TEST_DEVICE_COUNT=str(devices))
    env.pop("CUDA_VISIBLE_DEVICES", None)
    return subprocess.run([str(MOCK), *map(str, args)], capture_output=True, env=env, timeout=300)


def test_c1_configuration(golden):
    c1 = golden["c1"]
    # at most 2,000,000 sites per mock worker (tests/mock_backend.cpp:106-108)
    r = run([c1["coefficients"], c1["height"], "-du", c1["last"], "--devices", "all",
             "--batch-size", "249"])
    assert r.returncode == 0, r.stderr
    assert hashlib.sha256(r.stdout).hexdigest() == c1["sha256"]


def test_oracle_cases(golden):
    for case in golden["oracle_cases"]:
        r = run([case["coefficients"], case["height"], "-dl", case["first"], "-du", case["last"],
                 "--devices", "0,1"], devices=2)
        assert r.returncode == 0, r.stderr
        assert r.stdout.decode() == case["stdout"], case["coefficients"]
