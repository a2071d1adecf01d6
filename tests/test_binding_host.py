"""The reference-side drop-in (open-3d-wallturbulence_gb300/binding/solver_gpu.cpp)
compiles against the reference's own headers and links with its unmodified
driver (src/main.cpp) and I/O (src/IO.cpp) plus libowt_gpu.so: every name the
driver calls resolves to the binding, every owt_* call to the library.

Where the reference sources are present (OWT_REFERENCE_SRC, default the
reference checkout), the driver is then run on a small case file: without a
GPU it must get through load_params and allocate_var and stop in init_mat
with the library's own error from owt_create.  Elsewhere the test is
skipped, as the reference oracle build is."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = os.environ.get("OWT_REFERENCE_SRC", os.path.join(os.sep, "root", "reference", "src"))
SHIM = os.path.join(ROOT, "oracle", "shim")
BINDING = os.path.join(ROOT, "open-3d-wallturbulence_gb300", "binding", "solver_gpu.cpp")

CASE = """dt = 0.005
dkx = 0.5
dkz = 1.5
NX = 16
NY = 17
NZ = 16
alpha_mesh = 2.0
NT = 2
PX = 1
PZ = 1
save_interval = 1
nu = 3.5714285714285714e-4
"""


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF_SRC, "main.cpp")), reason="reference sources absent")
def test_binding_links_with_reference_driver(gpu_lib, tmp_path):
    libdir = os.path.dirname(gpu_lib)
    inc = ["-I" + SHIM, "-I" + REF_SRC, "-I" + os.path.join(ROOT, "include")]
    objs = []
    for src in (os.path.join(REF_SRC, "main.cpp"), os.path.join(REF_SRC, "IO.cpp"), BINDING,
                os.path.join(SHIM, "shim_impl.cpp"), os.path.join(SHIM, "hdf5_stub.cpp")):
        obj = str(tmp_path / (os.path.basename(src) + ".o"))
        r = subprocess.run(["g++", "-std=c++17", "-O1", "-w", "-c", src, "-o", obj] + inc,
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        objs.append(obj)
    exe = str(tmp_path / "channel_gpu")
    r = subprocess.run(["g++", "-o", exe] + objs + ["-L" + libdir, "-lowt_gpu", "-Wl,-rpath," + libdir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nm = subprocess.run(["nm", "-C", exe], capture_output=True, text=True).stdout
    for name in ("allocate_var()", "init_mat()", "init_fft()", "init_fields()", "time_Integration()",
                 "cleanup_fft()"):
        assert any(line.split()[1:2] == ["T"] and line.endswith(name) for line in nm.splitlines()), name
    und = subprocess.run(["nm", "-u", exe], capture_output=True, text=True).stdout
    assert "owt_time_integration" in und and "owt_create" in und
    case = tmp_path / "case.toml"
    case.write_text(CASE)
    run = subprocess.run([exe, str(case)], capture_output=True, text=True, cwd=tmp_path, timeout=120)
    out = run.stdout + run.stderr
    print(out[-2000:])
    assert "NX, NY, NZ = 16 17 16" in out  # load_params of src/IO.cpp ran
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        assert run.returncode != 0 and "owt_create" in out
