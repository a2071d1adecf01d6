"""owt_dy1_noalloc: DY1 for caller-owned device arrays, no device allocation.

It exists for callers that must not call cudaMalloc (graph capture in
progress, a foreign pool allocator owning device memory, no tolerance for the
synchronisation cudaMalloc implies).  Checked through the C ABI against the
handle-based DY1 (owt_dy_apply, order 1) on two calls in a row, at the
tolerance of the other single-routine tests (1e-12, max norm, relative).
This file sorts last so that a run stopping at the first failure has already
run every other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_dy1_noalloc_matches_handle_path_twice(gpu_lib):
    import torch
    from owt import lib as L
    from owt.params import CaseParams
    from owt.solver import GpuSolver

    lib = L.load(gpu_lib)
    p = CaseParams(dt=0.002, dkx=1.0, dkz=2.0, NX=32, NY=65, NZ=24, alpha_mesh=2.2, nu=1e-4)
    solver = GpuSolver(p)  # the existing entry point to compare with
    rng = np.random.default_rng(7)
    nlines = p.NZ * p.NXH
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        f = rng.standard_normal(p.spectral_shape) + 1j * rng.standard_normal(p.spectral_shape)
        want = solver.dy(1, f)                                   # [z][x][y]
        dev_in = torch.from_numpy(np.ascontiguousarray(np.transpose(f, (2, 0, 1)))).cuda()  # [y][z][x]
        dev_out = torch.empty_like(dev_in)
        rc = lib.owt_dy1_noalloc(p.NY, nlines, p.alpha_mesh, C.c_void_p(dev_in.data_ptr()),
                                 C.c_void_p(dev_out.data_ptr()), C.c_void_p(stream))
        assert rc == L.OK, lib.owt_last_error(None).decode()
        torch.cuda.synchronize()
        got = np.transpose(dev_out.cpu().numpy(), (1, 2, 0))
        err = rel(got, want)
        print(f"call {call}: max relative difference {err:.2e}")
        assert err < TOL


def test_dy1_noalloc_rejects_oversized_requests(gpu_lib):
    from owt import lib as L
    lib = L.load(gpu_lib)
    rc = lib.owt_dy1_noalloc(257, 1 << 20, 2.2, C.c_void_p(16), C.c_void_p(16), None)
    assert rc == 1
    assert "complex values" in lib.owt_last_error(None).decode()
    rc = lib.owt_dy1_noalloc(5, 10, 2.2, C.c_void_p(16), C.c_void_p(16), None)
    assert rc == 1 and "NY must be" in lib.owt_last_error(None).decode()
