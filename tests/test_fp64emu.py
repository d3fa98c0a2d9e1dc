"""The integer-pipe FP64 multiply (csrc/tl_fp64emu.cuh), built for the host, against the FPU's
multiply: the same bits on 4 M seeded operand pairs of every class (no GPU needed)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_integer_multiply_matches_ieee_rounding(tmp_path):
    exe = str(tmp_path / "fp64emu_host")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "tealeaf_ref_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "fp64emu_host.cpp"), "-o", exe], check=True)
    for seed in (1, 2):
        r = subprocess.run([exe, "2000000", str(seed)], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "mismatch 0" in r.stdout
