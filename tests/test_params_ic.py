"""Host-side logic: case-file parsing and the seeded initial condition."""
import os

import numpy as np
import pytest

from owt.params import CaseParams, load_params, parse_toml_text, channel_180, channel_550
from owt.ic import seeded_velocity
from owt.operators import dy1, grid, wavenumbers

CASE = """# physics
nu = 3.571428571428571e-4 # kinetic viscosity
# CFD
dt = 2.0e-3 # time step size
dkx = 0.25 # Lx=2*pi/dkx
dkz = 0.5 # Lz=2*pi/dkx
NX = 320 # number of cells in x direction
NY = 160 # number of cells in y direction
NZ = 320 # number of cells in z direction
alpha_mesh = 2.0 # the de-sigularity size of mesh y=tanh(alpha eta)/tanh(alpha)
NT = 100000 # number of time steps
initial_condition = 1 # 1 - "laminar only", 2 - "laminar perturbation", 3 - "renewal"
# MPI
PX = 16  # number of processors in x direction
PZ = 8 # number of processors in z direction
# IO
save_interval = 500 # save results every $(save_interval) time steps
"""


def test_case_file_keys_and_derived_sizes():
    p = load_params(CASE)
    assert (p.NX, p.NY, p.NZ, p.PX, p.PZ, p.NT, p.save_interval) == (320, 160, 320, 16, 8, 100000, 500)
    assert p.dt == 2.0e-3 and p.dkx == 0.25 and p.dkz == 0.5 and p.alpha_mesh == 2.0
    assert (p.NXH, p.NZH, p.NX2, p.NZ2) == (160, 160, 480, 480)   # src/IO.cpp:27-30
    assert p.extra["initial_condition"] == 1                         # read, then ignored


def test_case_file_missing_key_raises():
    with pytest.raises(KeyError):
        load_params(CASE.replace("dkz = 0.5", ""))


def test_case_file_from_path(tmp_path):
    f = tmp_path / "case.toml"
    f.write_text(CASE)
    assert load_params(str(f)).NY == 160


def test_invalid_sizes_rejected():
    with pytest.raises(ValueError):
        CaseParams(dt=1e-3, dkx=1, dkz=1, NX=15, NY=33, NZ=16, alpha_mesh=2, nu=1e-3).validate()
    with pytest.raises(ValueError):
        CaseParams(dt=1e-3, dkx=1, dkz=1, NX=16, NY=5, NZ=16, alpha_mesh=2, nu=1e-3).validate()


def test_workload_definitions():
    a, b = channel_180(), channel_550()
    assert (a.NX, a.NY, a.NZ, a.NX2) == (128, 129, 128, 192)
    assert (b.NX, b.NY, b.NZ, b.NX2) == (384, 257, 384, 576)
    assert abs(1.0 / a.nu - 2800) < 1e-9 and b.nu == 1e-4


@pytest.fixture(scope="module")
def ic():
    p = CaseParams(dt=0.005, dkx=0.5, dkz=1.5, NX=32, NY=33, NZ=32, alpha_mesh=2.0, nu=1 / 2800.)
    return p, seeded_velocity(p, seed=3)


def test_ic_is_divergence_free(ic):
    p, (u, v, w) = ic
    kx, kz = wavenumbers(p)
    D1 = dy1(p.NY, p.alpha_mesh)
    div = 1j * kx[None, :, None] * u + np.einsum("ij,zxj->zxi", D1, v) + 1j * kz[:, None, None] * w
    assert np.abs(div).max() < 1e-12 * max(np.abs(v).max(), 1e-30) * np.abs(D1).max()


def test_ic_walls_and_hermitian(ic):
    p, (u, v, w) = ic
    assert np.abs(v[:, :, [0, -1]]).max() < 1e-14 * np.abs(v).max()
    # kx = 0 column Hermitian in kz; Nyquist kz row empty
    for k in range(1, p.NZH):
        np.testing.assert_array_equal(v[p.NZ - k, 0], np.conj(v[k, 0]))
    assert np.abs(v[p.NZH]).max() == 0.0
    y, _, _ = grid(p.NY, p.alpha_mesh)
    np.testing.assert_allclose(u[0, 0].real, 1.5 * (1 - y ** 2), atol=1e-15)


def test_ic_rms_and_determinism(ic):
    p, (u, v, w) = ic
    u2, v2, w2 = seeded_velocity(p, seed=3)
    np.testing.assert_array_equal(v, v2)
    # perturbation RMS is 0.1 of the bulk velocity (Parseval, trapezoid in y)
    y, _, _ = grid(p.NY, p.alpha_mesh)
    wy = np.zeros(p.NY)
    dy = np.diff(y)
    wy[:-1] += dy / 2
    wy[1:] += dy / 2
    wy /= wy.sum()
    wx = np.full(p.NXH, 2.0)
    wx[0] = 1
    up = u.copy()
    up[0, 0] = 0
    e = sum((np.abs(f) ** 2 * wx[None, :, None]).sum(axis=(0, 1)) for f in (up, v, w))
    assert abs(np.sqrt((e * wy).sum() / 3) - 0.1) < 1e-12
    assert not np.array_equal(seeded_velocity(p, seed=4)[1], v)
