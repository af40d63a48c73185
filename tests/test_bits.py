"""The FP32 -> FP64 widening through bit patterns (csrc/hmec_bits.cuh), which
the marker gathers and the Arnoldi step use instead of the conversion
instruction (it runs at the FP64 rate on GB300), agrees bit for bit with the
compiler's conversion on random bit patterns (FP32 subnormals give 0)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "h-mecs-2d_gb300", "csrc")


def test_bit_pattern_widening_matches_the_compiler(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "bits_check")
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                        os.path.join(HERE, "bits_check.cpp"), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "f2d 0/" in r.stdout, r.stdout


def test_double_float_exp_matches_long_double_exp(tmp_path):
    """df_exp (csrc/hmec_dfexp.cuh, the marker-property kernel's exp(-alpha
    por)) against the long-double exp over [-60, 60]: relative error below
    2e-14."""
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "dfexp_check")
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                        os.path.join(HERE, "dfexp_check.cpp"), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
