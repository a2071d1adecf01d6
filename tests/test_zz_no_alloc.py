"""owt_dy1_noalloc: DY1 for caller-owned device arrays, no device allocation.

Some callers cannot call cudaMalloc: a program whose own pool allocator owns
the device memory, or a loop that cannot accept the device-wide
synchronisation cudaMalloc brings.  This entry point keeps its scratch in a
static device array instead.  Checked through the C ABI against the
handle-based DY1 (owt_dy_apply, order 1) at the tolerance of the other
single-routine tests (1e-12, max norm, relative): two calls in a row at one
size, then a call at a smaller size and another stretching after the larger
ones, which shows that a call does not read what an earlier call left in the
shared array.
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


def _noalloc_dy1(lib, L, p, f, stream):
    import torch
    nlines = p.NZ * p.NXH
    dev_in = torch.from_numpy(np.ascontiguousarray(np.transpose(f, (2, 0, 1)))).cuda()  # [y][z][x]
    dev_out = torch.empty_like(dev_in)
    rc = lib.owt_dy1_noalloc(p.NY, nlines, p.alpha_mesh, C.c_void_p(dev_in.data_ptr()),
                             C.c_void_p(dev_out.data_ptr()), C.c_void_p(stream))
    assert rc == L.OK, lib.owt_last_error(None).decode()
    torch.cuda.synchronize()
    return np.transpose(dev_out.cpu().numpy(), (1, 2, 0))


def test_dy1_noalloc_matches_handle_path_twice(gpu_lib):
    import torch
    from owt import lib as L
    from owt.params import CaseParams
    from owt.solver import GpuSolver

    lib = L.load(gpu_lib)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(7)
    # (NX, NY, NZ, alpha): two calls at the first size, then a smaller NY and
    # another stretching after the larger system
    cases = [(32, 65, 24, 2.2), (32, 65, 24, 2.2), (16, 129, 16, 2.0), (24, 33, 16, 1.7)]
    for call, (nx, ny, nz, al) in enumerate(cases):
        p = CaseParams(dt=0.002, dkx=1.0, dkz=2.0, NX=nx, NY=ny, NZ=nz, alpha_mesh=al, nu=1e-4)
        solver = GpuSolver(p)  # the existing entry point to compare with
        f = rng.standard_normal(p.spectral_shape) + 1j * rng.standard_normal(p.spectral_shape)
        want = solver.dy(1, f)  # [z][x][y]
        got = _noalloc_dy1(lib, L, p, f, stream)
        solver.close()
        err = rel(got, want)
        print(f"call {call} (NY={ny}, alpha={al}): max relative difference {err:.2e}")
        assert err < TOL


def test_dy1_noalloc_rejects_oversized_requests(gpu_lib):
    from owt import lib as L
    lib = L.load(gpu_lib)
    rc = lib.owt_dy1_noalloc(257, 1 << 20, 2.2, C.c_void_p(16), C.c_void_p(16), None)
    assert rc == 1
    assert "complex values" in lib.owt_last_error(None).decode()
    rc = lib.owt_dy1_noalloc(5, 10, 2.2, C.c_void_p(16), C.c_void_p(16), None)
    assert rc == 1 and "NY must be" in lib.owt_last_error(None).decode()
