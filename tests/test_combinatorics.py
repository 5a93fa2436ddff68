"""The CI-test kernels' subset combinatorics on the host: the device code of
csrc/stats.cuh (binomials with constant divisors, bisection unranking for large
neighbour counts) compiled by nvcc as a host program and checked against the plain
lexicographic unranking (the order of ithCombination, src/util/cuda_util.cu:34-50)."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_unranking_matches_lexicographic_order():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "unrank_check")
        subprocess.run([nvcc, "-x", "cu", "-O2", "-std=c++17", os.path.join(ROOT, "tests", "unrank_check.cu"), "-o",
                        exe], check=True, capture_output=True, timeout=300)
        out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok ")
