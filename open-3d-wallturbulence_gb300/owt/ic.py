"""Seeded initial condition: laminar Poiseuille flow plus a random
divergence-free perturbation.

The reference's own initial condition is a fixed TS-like wave
(src/solver.cpp:336-377); the workloads here need a seeded random state
instead.  Construction, per Fourier mode (kx, kz) != (0, 0):

* amplitudes are complex Gaussian with an energy spectrum falling as k^-2
  (k = |(kx, kz)|, relative to the smallest wavenumber);
* wall-normal shapes: v = (1 - y^2)^2 P(y) and omega_y = (1 - y^2) Q(y) with
  P, Q random Chebyshev series of degree 5, so v, dv/dy and omega_y vanish at
  both walls;
* u and w follow from continuity and the definition of omega_y, with the same
  formulas as the reference's solve_horizontal (src/solver.cpp:532-533):
  u = i kx/k^2 DY1 v - i kz/k^2 g,  w = i kx/k^2 g + i kz/k^2 DY1 v;
* the kx = 0 column is made Hermitian in kz and the Nyquist kz row is zero, so
  the physical field is real;
* the perturbation is scaled to an RMS of ``rms`` times the bulk velocity
  (bulk velocity 1 for the profile 1.5 (1 - y^2)), measured by Parseval's sum
  with trapezoidal weights in y.

The mean mode is the laminar profile u = 1.5 (1 - y^2) as in src/solver.cpp:338-341.
Arrays are complex128 in the reference layout [z][x][y].
"""
import numpy as np

from .operators import dy1, grid, wavenumbers


def seeded_velocity(p, seed=0, rms=0.1, degree=5):
    y, _, _ = grid(p.NY, p.alpha_mesh)
    D1 = dy1(p.NY, p.alpha_mesh)
    kx, kz = wavenumbers(p)
    NZ, NXH, NY = p.spectral_shape
    rng = np.random.default_rng(seed)
    cheb = np.polynomial.chebyshev.chebvander(y, degree)  # NY x (degree+1)

    def rnd():
        return (rng.standard_normal((NZ, NXH, degree + 1)) + 1j * rng.standard_normal((NZ, NXH, degree + 1)))

    a, b = rnd(), rnd()
    K = np.sqrt(kx[None, :] ** 2 + kz[:, None] ** 2)
    kmin = min(p.dkx, p.dkz)
    amp = np.zeros_like(K)
    nz = K > 0
    amp[nz] = (K[nz] / kmin) ** -2.0
    v = amp[:, :, None] * np.einsum("zxp,yp->zxy", a, cheb) * ((1 - y ** 2) ** 2)[None, None, :]
    g = amp[:, :, None] * np.einsum("zxp,yp->zxy", b, cheb) * (1 - y ** 2)[None, None, :]
    # Nyquist kz row (index NZH, wavenumber -NZH*dkz) carries nothing.
    v[p.NZH] = 0.0
    g[p.NZH] = 0.0
    # Hermitian kx = 0 column: mode -kz is the conjugate of mode +kz.
    for k in range(1, p.NZH):
        v[p.NZ - k, 0] = np.conj(v[k, 0])
        g[p.NZ - k, 0] = np.conj(g[k, 0])
    v[0, 0] = 0.0
    g[0, 0] = 0.0
    d1v = np.einsum("ij,zxj->zxi", D1, v)
    K2 = np.where(K > 0, K ** 2, 1.0)
    ikx = 1j * kx[None, :, None] / K2[:, :, None]
    ikz = 1j * kz[:, None, None] / K2[:, :, None]
    u = ikx * d1v - ikz * g
    w = ikx * g + ikz * d1v
    u[0, 0] = 0.0
    w[0, 0] = 0.0
    # RMS by Parseval: kx = 0 counts once, kx > 0 twice (the conjugate half).
    wx = np.full(NXH, 2.0)
    wx[0] = 1.0
    wy = np.zeros(NY)
    dy = np.diff(y)
    wy[:-1] += dy / 2
    wy[1:] += dy / 2
    wy /= wy.sum()
    e = sum((np.abs(f) ** 2 * wx[None, :, None]).sum(axis=(0, 1)) for f in (u, v, w))
    cur = np.sqrt((e * wy).sum() / 3.0)
    s = rms / cur if cur > 0 else 0.0
    u, v, w = u * s, v * s, w * s
    u[0, 0] = 1.5 * (1 - y ** 2)
    return u.astype(np.complex128), v.astype(np.complex128), w.astype(np.complex128)
