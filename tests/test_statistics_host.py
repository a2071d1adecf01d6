"""The Parseval rules of the statistics against direct averages of the
physical fields, built the way the reference's Fourier2Physical_dealiased
does (src/FFT.cpp:49-128): Nyquist kz row dropped, real part of the x
transform (so a non-Hermitian kx = 0 column enters through its Hermitian part)."""
import numpy as np

from owt.snapshot import statistics_from_fields


def to_physical(u, NX, NZ):
    NZ_, NXH, NY = u.shape
    NZH, NX2, NZ2 = NZ // 2, NX // 2 * 3, NZ // 2 * 3
    zp = np.zeros((NZ2, NXH, NY), complex)
    zp[:NZH] = u[:NZH]
    zp[NZ:NZ + NZH] = u[NZH:]
    zp[NZ] = 0.0
    zi = np.fft.ifft(zp, axis=0) * NZ2
    xp = np.zeros((NZ2, NX2, NY), complex)
    xp[:, :NXH] = zi
    for i in range(1, NXH):
        xp[:, NX + i] = np.conj(zi[:, NXH - i])
    return (np.fft.ifft(xp, axis=1) * NX2).real


def test_parseval_statistics_match_physical_averages():
    rng = np.random.default_rng(3)
    NX, NZ, NY = 12, 8, 9
    shp = (NZ, NX // 2, NY)
    u, v, w = [rng.standard_normal(shp) + 1j * rng.standard_normal(shp) for _ in range(3)]
    st = statistics_from_fields(u, v, w, NZ // 2)
    pu, pv, pw = [to_physical(f, NX, NZ) for f in (u, v, w)]
    mean = lambda f: f.mean(axis=(0, 1))
    np.testing.assert_allclose(st["U"], mean(pu), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(st["u_rms"], np.sqrt(mean(pu ** 2) - mean(pu) ** 2), rtol=1e-11)
    np.testing.assert_allclose(st["w_rms"], np.sqrt(mean(pw ** 2) - mean(pw) ** 2), rtol=1e-11)
    np.testing.assert_allclose(st["uv"], mean(pu * pv) - mean(pu) * mean(pv), rtol=1e-10, atol=1e-12)
