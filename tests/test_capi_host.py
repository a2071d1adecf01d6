"""The C ABI library: it loads, exports every function include/owt_gpu.h
declares, and rejects bad parameters before touching a GPU."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "owt_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(owt_\w+)\s*\(", text, re.M)))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for n in ("owt_create", "owt_destroy", "owt_init_fields", "owt_time_integration", "owt_get_field",
              "owt_set_field", "owt_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol(gpu_lib):
    lib = C.CDLL(gpu_lib)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def _params(**kw):
    from owt.lib import OwtParams
    d = dict(dt=0.005, dkx=0.5, dkz=1.5, alpha_mesh=2.0, nu=1 / 2800., NX=16, NY=17, NZ=16, precision=0, device=0)
    d.update(kw)
    return OwtParams(**d)


@pytest.mark.parametrize("bad,msg", [
    (dict(NX=15), "even"), (dict(NY=5), "at least 7"), (dict(dt=-1.0), "positive"),
    (dict(precision=7), "precision"), (dict(NX=28), "2^a 3^b 5^c"),
])
def test_create_rejects_bad_parameters_without_a_gpu(gpu_lib, bad, msg):
    from owt import lib as L
    lib = L.load(gpu_lib)
    h = C.c_void_p()
    rc = lib.owt_create(C.byref(_params(**bad)), C.byref(h))
    assert rc == L.OK + 1  # OWT_ERR_INVALID
    assert h.value is None
    assert msg in lib.owt_last_error(None).decode()


def test_null_handle_calls_fail_cleanly(gpu_lib):
    from owt import lib as L
    lib = L.load(gpu_lib)
    assert lib.owt_time_integration(None, 1) == 1
    assert lib.owt_synchronize(None) == 1
    assert lib.owt_destroy(None) == 0


def test_batch_seeded_and_selftest_entry_points_refuse_bad_arguments_without_a_gpu(gpu_lib):
    from owt import lib as L
    lib = L.load(gpu_lib)
    b = C.c_void_p()
    assert lib.owt_batch_create(None, 0, C.byref(b)) == L.OK + 1
    assert b.value is None and "at least one handle" in lib.owt_last_error(None).decode()
    assert lib.owt_batch_step(None, 1) == L.OK + 1
    assert lib.owt_batch_destroy(None) == L.OK
    assert lib.owt_batch_tuning_report(None) == b""
    assert lib.owt_init_seeded(None, 1, 0.1) == L.OK + 1
    assert lib.owt_setup_report(None) == b""
    bad, t1, t2 = C.c_int64(0), C.c_float(0), C.c_float(0)
    # band widths the library does not use, and empty systems, are refused before any device work
    assert lib.owt_band_factor_selftest(15, 13, 10, 4, 1, C.byref(bad), C.byref(t1), C.byref(t2)) == L.OK + 1
    assert lib.owt_band_factor_selftest(15, 16, 0, 4, 1, C.byref(bad), C.byref(t1), C.byref(t2)) == L.OK + 1
    assert "bad arguments" in lib.owt_last_error(None).decode()
