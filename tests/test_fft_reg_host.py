"""The register transforms of the FP32 transform kernels (csrc/fft_reg.cuh),
compiled by nvcc as host code and checked against a direct transform in
long double (tests/fft_reg_check.cu): every length the kernels use, both
signs, double and float, the two-pass line factorisations, and the
compile-time twiddle constants."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "open-3d-wallturbulence_gb300", "csrc")


def test_register_transforms_match_direct_dft(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc absent")
    exe = str(tmp_path / "fft_reg_check")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I" + CSRC, os.path.join(ROOT, "tests", "fft_reg_check.cu"),
                    "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
