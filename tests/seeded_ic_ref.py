"""Test infrastructure: a numpy restatement of the device's seeded initial
condition (owt_init_seeded), used only as the checker of the GPU generator.

Same construction as the device code: Philox4x32-10 (Salmon et al., SC 2011)
keyed by the seed and counted by (mode, p, series), two 53-bit uniforms per
draw, one Box-Muller pair per complex Chebyshev coefficient; v and omega_y
from the coefficients, u and w from continuity, RMS scaling by Parseval with
trapezoidal weights in y, then the laminar mean profile.  Arrays are
complex128 in the reference layout [z][x][y].
"""
import numpy as np

_M0, _M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
_W0, _W1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
_MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    c0, c1, c2, c3 = (np.asarray(x, np.uint64) & _MASK for x in (c0, c1, c2, c3))
    k0, k1 = np.uint64(k0) & _MASK, np.uint64(k1) & _MASK
    for _ in range(10):
        p0, p1 = c0 * _M0, c2 * _M1  # 32 x 32 -> 64 bits, no overflow
        hi0, lo0 = p0 >> np.uint64(32), p0 & _MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & _MASK
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        k0, k1 = (k0 + _W0) & _MASK, (k1 + _W1) & _MASK
    return c0, c1, c2, c3


def _unit53(hi, lo):
    m = (hi << np.uint64(21)) | (lo >> np.uint64(11))
    return (m.astype(np.float64) + 0.5) * 2.0 ** -53


def gauss(seed, mode, p, series):
    seed = int(seed)
    r = philox4x32_10(mode, np.full_like(mode, p), np.full_like(mode, series), np.zeros_like(mode),
                      seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)
    u1, u2 = _unit53(r[0], r[1]), _unit53(r[2], r[3])
    rad = np.sqrt(-2.0 * np.log(u1))
    th = 6.283185307179586 * u2
    return rad * np.cos(th) + 1j * rad * np.sin(th)


def seeded_velocity_device_restated(p, seed, rms=0.1, degree=5):
    from owt.operators import dy1, grid, wavenumbers
    y, _, _ = grid(p.NY, p.alpha_mesh)
    D1 = dy1(p.NY, p.alpha_mesh)
    kx, kz = wavenumbers(p)
    NZ, NXH, NY = p.spectral_shape
    k = np.arange(NZ)[:, None] * np.ones((1, NXH), int)
    i = np.ones((NZ, 1), int) * np.arange(NXH)[None, :]
    mirror = (i == 0) & (k > p.NZH)
    src = np.where(mirror, (NZ - k) * NXH, k * NXH + i).astype(np.uint64)
    zero = ((k == 0) & (i == 0)) | (k == p.NZH)
    coef = np.zeros((2, degree + 1, NZ, NXH), np.complex128)
    for s in range(2):
        for q in range(degree + 1):
            z = gauss(seed, src, q, s)
            z = np.where(mirror, np.conj(z), z)
            coef[s, q] = np.where(zero, 0.0, z)
    k2 = kx[None, :] ** 2 + kz[:, None] ** 2
    kmin = min(p.dkx, p.dkz)
    amp = np.where(k2 > 0, kmin * kmin / np.where(k2 > 0, k2, 1.0), 0.0)
    T = np.zeros((degree + 1, NY))
    tp, tq = np.ones(NY), y.copy()
    for q in range(degree + 1):
        T[q] = tp
        tp, tq = tq, 2.0 * y * tq - tp
    s1 = 1.0 - y * y
    sv = np.einsum("qzx,qy->zxy", coef[0], T)
    sg = np.einsum("qzx,qy->zxy", coef[1], T)
    v = sv * (amp[:, :, None] * s1 * s1)
    g = sg * (amp[:, :, None] * s1)
    d1v = np.einsum("ij,zxj->zxi", D1, v)
    k2s = np.where(k2 > 0, k2, 1.0)
    ax, az = (kx[None, :] / k2s)[:, :, None], (kz[:, None] / k2s)[:, :, None]
    u = 1j * ax * d1v - 1j * az * g
    w = 1j * ax * g + 1j * az * d1v
    u[0, 0] = 0.0
    w[0, 0] = 0.0
    wx = np.full(NXH, 2.0)
    wx[0] = 1.0
    wy = np.zeros(NY)
    dy = np.diff(y)
    wy[:-1] += dy / 2
    wy[1:] += dy / 2
    wy /= wy.sum()
    e = sum((np.abs(f) ** 2 * wx[None, :, None] * wy[None, None, :]).sum() for f in (u, v, w))
    cur = np.sqrt(e / 3.0)
    sc = rms / cur if cur > 0 else 0.0
    u, v, w = u * sc, v * sc, w * sc
    u[0, 0] = 1.5 * (1 - y ** 2)
    return u, v, w
