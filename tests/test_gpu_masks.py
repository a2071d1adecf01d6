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
* The stand-alone transforms (owt_fourier2physical / owt_physical2fourier,
  the step's own kernels) against the reference's outputs in
  tests/golden/transform_12x17x12.npz, exact zeros for a Nyquist-only field,
  zeros to round-off for a physical field made of truncated modes only.
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


def test_transform_pair_matches_reference_golden(gpu_lib):
    """Fourier2Physical_dealiased / Physical2Fourier_dealiased on the GPU
    against the reference's own outputs (FFTW replaced by the oracle's FFT
    shim, itself checked against numpy): 1e-13 of the largest value."""
    from conftest import golden
    from owt.params import CaseParams
    g = golden("transform_12x17x12.npz")
    dt, dkx, dkz, NX, NY, NZ, al, nu = g["params"]
    p = CaseParams(dt=dt, dkx=dkx, dkz=dkz, NX=int(NX), NY=int(NY), NZ=int(NZ), alpha_mesh=al, nu=nu)
    s = solver(p)
    phys = s.Fourier2Physical_dealiased(g["spec_in"])
    e1 = float(np.abs(phys - g["phys_out"]).max() / np.abs(g["phys_out"]).max())
    spec = s.Physical2Fourier_dealiased(g["phys_in"])
    e2 = float(np.abs(spec - g["spec_out"]).max() / np.abs(g["spec_out"]).max())
    print(f"transform pair vs reference: backward {e1:.1e}, forward {e2:.1e}")
    assert e1 < 1e-13 and e2 < 1e-13


def test_transform_masks_exact_zeros(gpu_lib):
    """A spectral field with energy only in the kz = -NZ/2 row maps to an
    all-zero physical field, bit for bit (src/FFT.cpp:86-87).  A physical
    field built from truncated modes only (|kx| >= NX/2, and |kz| > NZ/2 with
    |kx| < NX/2) maps to a spectrum that is zero to FFT round-off, and the
    same field plus a kept mode returns exactly that mode to round-off."""
    from owt.params import CaseParams
    p = CaseParams(dt=0.005, dkx=0.5, dkz=1.5, NX=16, NY=9, NZ=20, alpha_mesh=2.0, nu=1 / 2800.)
    s = solver(p)
    rng = np.random.default_rng(4)
    f = np.zeros(p.spectral_shape, np.complex128)
    f[p.NZH] = rng.standard_normal(f[p.NZH].shape) + 1j * rng.standard_normal(f[p.NZH].shape)
    phys = s.Fourier2Physical_dealiased(f)
    assert np.count_nonzero(phys) == 0
    # truncated modes on the 3/2 grid: x index X, z index Z of exp(i 2 pi (X x/NX2 + Z z/NZ2))
    NX2, NZ2 = p.NX2, p.NZ2
    x = np.arange(NX2)[None, :, None]
    z = np.arange(NZ2)[:, None, None]
    yy = (1.0 + np.arange(p.NY))[None, None, :]
    up = np.zeros((NZ2, NX2, p.NY))
    for X, Z in [(p.NXH, 0), (p.NXH + 2, 3), (NX2 // 2, p.NZH + 1), (1, p.NZH + 2), (0, NZ2 // 2)]:
        ph = rng.uniform(0, 2 * np.pi)
        up += np.cos(2 * np.pi * (X * x / NX2 + Z * z / NZ2) + ph) * yy
    spec = s.Physical2Fourier_dealiased(up)
    print("truncated modes only: largest kept coefficient %.1e" % np.abs(spec).max())
    assert np.abs(spec).max() < 1e-14 * np.abs(up).max()
    # plus one kept mode (kx = 2, kz = -3), 2 Re(c e^{i theta}): it comes back as c at (kz index NZ-3, kx 2)
    c = 0.8 - 0.3j
    keep = (c * np.exp(2j * np.pi * (2 * x / NX2 - 3 * z / NZ2))).real * 2 * yy
    spec = s.Physical2Fourier_dealiased(up + keep)
    want = np.zeros(p.spectral_shape, np.complex128)
    want[p.NZ - 3, 2, :] = c * yy[0, 0]
    err = np.abs(spec - want).max() / abs(c)
    print("kept mode recovered to %.1e" % err)
    assert err < 1e-13
