"""The integer-assembled FP64 product of two floats used by the solver's FP64 dot products
(waves_gb300/csrc/exact_product.h) gives the FP64 multiply's bits for every class of input."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_exact_product_matches_the_fp64_multiply(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "exact_product_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "exact_product_check.cpp")], check=True)
    r = subprocess.run([exe, "2000000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 mismatches" in r.stdout
