"""The banded augmented v- and omega_y-systems of the mode kernel
(csrc/setup_host.cpp: d_t kept as unknowns, d4 substituted on interior nodes,
right-hand sides through the row tables, rows equilibrated) solved with the
library's own band solve, against the reference's dense per-mode systems
(src/solver.cpp:577-603) built from the same stencils, on the CPU
(tests/augmented_check.cu): the banded v is a backward-stable solution of the
dense v-system (normwise backward error <= 2e-14) and g agrees to 1e-12, for
grids of 33 to 257 points, both finite-difference orders and wavenumbers from
0.5 to 300."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "open-3d-wallturbulence_gb300", "csrc")


def test_augmented_systems_solve_the_dense_ones(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc absent")
    exe = str(tmp_path / "augmented_check")
    subprocess.run([nvcc, "-std=c++17", "-O2", "--expt-relaxed-constexpr", "-I" + CSRC,
                    os.path.join(ROOT, "tests", "augmented_check.cu"),
                    os.path.join(CSRC, "setup_host.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
