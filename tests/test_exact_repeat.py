"""pbf::rep_add (novaphy_gb300/csrc/exact_repeat.h), the exact repeated
addition the cooperative walk applies to runs of particles with bit-identical
state, equals m single float additions bit for bit: random magnitudes and
signs, ties at the binade spacing in both parities, sums from +0 and -0,
sums through zero, subnormal, infinite and NaN values, long runs (2^22)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_rep_add_equals_single_additions(tmp_path):
    exe = str(tmp_path / "exact_repeat_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I",
                    os.path.join(ROOT, "novaphy_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "exact_repeat_check.cpp"), "-o", exe], check=True)
    for seed in (1, 2, 3):
        out = subprocess.run([exe, str(seed)], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout
        assert " 0 mismatches" in out.stdout
