"""The tables owt_dy1_noalloc builds for itself (csrc/noalloc_setup.h) are
the handle's first-derivative operator: built on the host with g++ beside
csrc/setup_host.cpp and compared entry for entry (noalloc_tables_check.cpp)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "open-3d-wallturbulence_gb300", "csrc")


def test_noalloc_tables_equal_setup_host_stencils(tmp_path):
    exe = str(tmp_path / "noalloc_tables_check")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + CSRC, os.path.join(ROOT, "tests", "noalloc_tables_check.cpp"),
                    os.path.join(CSRC, "setup_host.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
