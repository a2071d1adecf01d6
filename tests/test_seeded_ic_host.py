"""CPU checks of the restatement of the device's seeded initial condition
(the checker of owt_init_seeded): the generator's output statistics and the
structure of the field it builds."""
import numpy as np

from owt.operators import dy1, wavenumbers
from owt.params import CaseParams
from seeded_ic_ref import gauss, philox4x32_10, seeded_velocity_device_restated

SMALL = dict(dt=0.005, dkx=0.5, dkz=1.5, NX=16, NY=33, NZ=16, alpha_mesh=2.0, nu=1 / 2800.)


def test_philox_is_a_function_of_counter_and_key_only():
    c = np.arange(1000, dtype=np.uint64)
    a = philox4x32_10(c, c, c, c, 5, 7)
    b = philox4x32_10(c, c, c, c, 5, 7)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    d = philox4x32_10(c, c, c, c, 6, 7)
    assert not np.array_equal(a[0], d[0])
    assert all(int(x.max()) < 2 ** 32 for x in a)


def test_gaussian_draws_have_unit_variance_and_no_correlation():
    modes = np.arange(200000, dtype=np.uint64)
    z = gauss(12345, modes, 0, 0)
    for part in (z.real, z.imag):
        assert abs(part.mean()) < 0.01 and abs(part.var() - 1.0) < 0.01
    assert abs(np.mean(z.real * z.imag)) < 0.01
    z2 = gauss(12345, modes, 1, 0)
    assert abs(np.mean(z.real * z2.real)) < 0.01


def test_restated_field_is_divergence_free_real_and_scaled():
    p = CaseParams(**SMALL)
    u, v, w = seeded_velocity_device_restated(p, seed=9, rms=0.1)
    kx, kz = wavenumbers(p)
    D1 = dy1(p.NY, p.alpha_mesh)
    div = 1j * kx[None, :, None] * u + np.einsum("ij,zxj->zxi", D1, v) + 1j * kz[:, None, None] * w
    div[0, 0] = 0.0
    assert np.abs(div).max() < 1e-12 * np.abs(v).max() * np.abs(kz).max()
    assert not v[..., 0].any() and not v[..., -1].any()
    k = np.arange(1, p.NZH)
    np.testing.assert_array_equal(v[p.NZ - k, 0], np.conj(v[k, 0]))
    assert not v[p.NZH].any()
    np.testing.assert_allclose(u[0, 0].real, 1.5 * (1 - np.tanh(p.alpha_mesh * np.linspace(-1, 1, p.NY)) ** 2
                                                     / np.tanh(p.alpha_mesh) ** 2), atol=1e-14)
