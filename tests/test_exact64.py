"""The correctly rounded FP64 square root and division that the sweeps compute
on the integer and FP32 pipes (mps_gb300/csrc/exact64.cuh).

Host: the same header compiled with the host compiler, its raw FP32 starting
approximations perturbed by up to 2^-12 (the routines refine them with one
Newton step; the hardware's documented bound is 2 ulp), against the host's
IEEE square root and division.  GPU: the device build against the GPU's FP64 instructions on
2^26 seeded cases of each, through mps_selftest_exact64."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_exact64_host_against_ieee(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "exact64_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                    os.path.join(HERE, "exact64_check.cpp")], check=True)
    out = subprocess.run([exe, "400000", "20261204"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.count("bit-identical") == 5, out.stdout


@pytest.mark.gpu
def test_exact64_device_against_fp64_instructions():
    from mps_gb300 import engine
    n = 1 << 26
    rc, r = engine.selftest_exact64(n, seed=7)
    assert rc == 0
    assert r["sqrt_mismatches"] == 0 and r["div_mismatches"] == 0, r
    assert r["other_mismatches"] == 0, r
    # nearly every generated case is inside the integer path
    assert r["sqrt_fast"] == n
    assert r["div_fast"] > 0.9 * n
