"""The masked band solves of the mode kernel and the adjoint
(csrc/owt_device.cuh), compiled by nvcc as host code and run against their
full-band forms on factors built as the setup builds them
(tests/band_masks_check.cu): the v-system's one-ring and two-ring masked
solves and the masked transposed solve at both finite-difference orders, and
the omega_y-system's masked solve, bitwise, over grids of 65 to 257 points
and a sweep of wavenumbers."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "open-3d-wallturbulence_gb300", "csrc")


def test_masked_band_solves_equal_full_band(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc absent")
    exe = str(tmp_path / "band_masks_check")
    subprocess.run([nvcc, "-std=c++17", "-O2", "--expt-relaxed-constexpr", "-I" + CSRC,
                    os.path.join(ROOT, "tests", "band_masks_check.cu"),
                    os.path.join(CSRC, "setup_host.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
