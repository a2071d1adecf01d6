"""The seeded initial condition generated on the device (owt_init_seeded)
against its numpy restatement, and the properties the construction promises."""
import numpy as np
import pytest

from seeded_ic_ref import seeded_velocity_device_restated

pytestmark = pytest.mark.gpu


def _case(nx, ny, nz):
    from owt.params import CaseParams
    return CaseParams(dt=0.004, dkx=0.5, dkz=1.5, NX=nx, NY=ny, NZ=nz, alpha_mesh=2.0, nu=1 / 2800.)


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("size,seed", [((16, 33, 16), 3), ((20, 25, 40), 11), ((64, 97, 48), 2 ** 40 + 5)])
def test_device_field_matches_restatement(gpu_lib, size, seed):
    from owt.solver import GpuSolver
    p = _case(*size)
    s = GpuSolver(p)
    s.init_seeded(seed, 0.1)
    want = seeded_velocity_device_restated(p, seed, 0.1)
    for name, ref in zip(("velx", "vely", "velz"), want):
        err = _rel(s.get(name), ref)
        print(size, name, f"{err:.1e}")
        assert err < 1e-12, (name, err)


def test_device_field_properties_and_determinism(gpu_lib):
    from owt.operators import dy1, wavenumbers
    from owt.solver import GpuSolver
    p = _case(32, 65, 48)
    a, b, c = GpuSolver(p), GpuSolver(p), GpuSolver(p)
    a.init_seeded(7, 0.1)
    b.init_seeded(7, 0.1)
    c.init_seeded(8, 0.1)
    u, v, w = a.get("velx"), a.get("vely"), a.get("velz")
    np.testing.assert_array_equal(u, b.get("velx"))
    np.testing.assert_array_equal(v, b.get("vely"))
    assert not np.array_equal(v, c.get("vely"))
    # walls, Nyquist row, Hermitian kx = 0 column: exact
    assert not v[..., 0].any() and not v[..., -1].any()
    assert not v[p.NZH].any() and not u[p.NZH].any()
    k = np.arange(1, p.NZH)
    for f in (u, v, w):
        np.testing.assert_array_equal(f[p.NZ - k, 0], np.conj(f[k, 0]))
    # divergence-free with the compact DY1, RMS as asked
    kx, kz = wavenumbers(p)
    D1 = dy1(p.NY, p.alpha_mesh)
    div = 1j * kx[None, :, None] * u + np.einsum("ij,zxj->zxi", D1, v) + 1j * kz[:, None, None] * w
    div[0, 0] = 0.0
    assert np.abs(div).max() < 1e-11 * np.abs(kz).max() * np.abs(v).max()
    uf = u.copy()
    uf[0, 0] = 0.0
    wx = np.full(p.NXH, 2.0)
    wx[0] = 1.0
    from owt.operators import grid
    yy, _, _ = grid(p.NY, p.alpha_mesh)
    wy = np.zeros(p.NY)
    wy[:-1] += np.diff(yy) / 2
    wy[1:] += np.diff(yy) / 2
    wy /= wy.sum()
    e = sum((np.abs(f) ** 2 * wx[None, :, None] * wy[None, None, :]).sum() for f in (uf, v, w))
    assert abs(np.sqrt(e / 3) - 0.1) < 1e-13
    # the step runs from it and matches a step from the same field given by the host
    h = GpuSolver(p)
    h.init_fields(u, v, w)
    a.time_Integration(2)
    h.time_Integration(2)
    for n in ("vely", "vory", "Hv"):
        np.testing.assert_array_equal(a.get(n), h.get(n))
