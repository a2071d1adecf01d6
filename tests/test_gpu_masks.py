"""Integer work of the step on the GPU, checked bit for bit where the
arithmetic allows it: the dealias masks of the transforms (src/FFT.cpp:49-194)
and the wavenumber indexing (src/solver.cpp:25-37).

* The Nyquist-z row (kz index NZH, wavenumber -NZH dkz) is dropped on the way
  to physical space (src/FFT.cpp:86-87): fields with energy only there give a
  Lamb vector that is exactly zero.
* Products whose every wavenumber lies outside the kept modes (|kx| >= NX/2
  or kz outside [-NZ/2, NZ/2)) are truncated on the way back
  (src/FFT.cpp:153-162, 177-188): such a Lamb vector is zero to FFT
  round-off, while a product inside the kept modes lands exactly on the modes
  the product formula gives.
* kz = k dkz for k < NZ/2 and (k - NZ) dkz from index NZ/2 on, kx = i dkx:
  omega_y = i kz u - i kx w of single-signed inputs is one rounded product,
  so it equals numpy's product with those wavenumbers bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("velx", "vely", "velz", "vorx", "vory", "vorz")


def small_params():
    from owt.params import CaseParams
    return CaseParams(dt=0.005, dkx=0.5, dkz=1.5, NX=12, NY=17, NZ=12, alpha_mesh=2.0, nu=1 / 2800.)


def solver(p, precision="fp64"):
    from owt.solver import GpuSolver
    from owt.ic import seeded_velocity
    s = GpuSolver(p, precision=precision)
    s.init_fields(*seeded_velocity(p, seed=1))
    return s


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nyquist_row_never_reaches_physical_space(gpu_lib, precision):
    p = small_params()
    s = solver(p, precision)
    rng = np.random.default_rng(3)
    for n in FIELDS:
        f = np.zeros(p.spectral_shape, np.complex128)
        f[p.NZH] = rng.standard_normal(f[p.NZH].shape) + 1j * rng.standard_normal(f[p.NZH].shape)
        s.set(n, f)
    s.Lamb_vec()
    for n in ("lmbx", "lmby", "lmbz"):
        got = s.get(n)
        assert np.count_nonzero(got) == 0, (n, np.abs(got).max())


def _single_mode(p, kz_mode, kx, amp):
    f = np.zeros(p.spectral_shape, np.complex128)
    k = kz_mode if kz_mode >= 0 else kz_mode + p.NZ
    f[k, kx, :] = amp * (1.0 + 0.25 * np.arange(p.NY))
    return f


def test_truncated_products_vanish_and_kept_ones_land_on_their_modes(gpu_lib):
    """lambda_z = u omega_y with v = w = omega_x = omega_z = 0.  u in mode
    (kx, kz) = (3, 4), omega_y in (3, -3): the products sit at (6, 1) (kx at
    NX/2, dropped) and (0, 7) (kz beyond NZ/2, dropped).  The control pair
    (1, 1) x (1, 1) gives a b at (2, 2) and 2 Re(a conj b) at (0, 0)."""
    p = small_params()
    assert p.NXH == 6 and p.NZH == 6
    s = solver(p)
    a, b = 0.5 - 0.2j, 0.7 + 0.3j
    scale = (1.0 + 0.25 * np.arange(p.NY)) ** 2
    zero = np.zeros(p.spectral_shape, np.complex128)
    for n in FIELDS:
        s.set(n, zero)
    s.set("velx", _single_mode(p, 4, 3, a))
    s.set("vory", _single_mode(p, -3, 3, b))
    s.Lamb_vec()
    lz = s.get("lmbz")
    print("truncated product, largest kept coefficient / |a b|: %.1e" % (np.abs(lz).max() / abs(a * b)))
    assert np.abs(lz).max() <= 1e-14 * abs(a * b) * scale.max()
    for n in ("lmbx", "lmby"):
        assert np.count_nonzero(s.get(n)) == 0
    # control: kept modes
    s.set("velx", _single_mode(p, 1, 1, a))
    s.set("vory", _single_mode(p, 1, 1, b))
    s.Lamb_vec()
    lz = s.get("lmbz")
    want = np.zeros(p.spectral_shape, np.complex128)
    want[2, 2, :] = a * b * scale
    want[0, 0, :] = 2 * (a * np.conj(b)).real * scale
    err = np.abs(lz - want).max() / np.abs(want).max()
    print("kept product vs its formula: %.1e" % err)
    assert err < 1e-14


def test_wavenumber_indexing_is_bit_exact(gpu_lib):
    from owt.params import CaseParams
    p = CaseParams(dt=0.005, dkx=0.5, dkz=1.5, NX=16, NY=17, NZ=20, alpha_mesh=2.0, nu=1 / 2800.)
    s = solver(p)
    rng = np.random.default_rng(9)
    kx = np.arange(p.NXH) * p.dkx
    kidx = np.arange(p.NZ)
    kz = np.where(kidx < p.NZH, kidx, kidx - p.NZ).astype(np.float64) * p.dkz
    assert kz[p.NZH] == -p.NZH * p.dkz
    zero = np.zeros(p.spectral_shape, np.complex128)
    for which in ("velx", "velz"):
        f = rng.standard_normal(p.spectral_shape) + 1j * rng.standard_normal(p.spectral_shape)
        for n in ("velx", "vely", "velz"):
            s.set(n, f if n == which else zero)
        s.get_vor_from_vel()
        oy = s.get("vory")
        if which == "velx":  # omega_y = i kz u
            want = (1j * kz[:, None, None]) * f
        else:  # omega_y = -i kx w
            want = (-1j * kx[None, :, None]) * f
        np.testing.assert_array_equal(oy.real, want.real)
        np.testing.assert_array_equal(oy.imag, want.imag)
