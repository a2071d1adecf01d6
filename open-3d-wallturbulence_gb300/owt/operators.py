"""Wall-normal grid, metric and the first-derivative operator in numpy.

Used on the host to build initial conditions (u, w from v and omega_y need
DY1).  Restates src/solver.cpp:57-106 (grid, metric) and src/compdiff.hpp:11-69
(first-derivative compact scheme, 8th order interior, 4th order closures);
DY1 = diag(c11) A1^-1 B1 as src/solver.cpp:178-182.
"""
import numpy as np


def grid(NY, alpha):
    """y = tanh(alpha s)/tanh(alpha) on s uniform in [-1, 1], and dy/ds."""
    s = 2 * np.arange(NY) / (NY - 1.0) - 1.0
    a_s = alpha * s
    y = np.tanh(a_s) / np.tanh(alpha)
    dyds1 = alpha / np.tanh(alpha) * (1.0 / np.cosh(a_s)) ** 2
    return y, s, dyds1


def first_derivative_stencils(N, h):
    A = np.zeros((N, N))
    B = np.zeros((N, N))
    al, be, a, b = 4 / 9, 1 / 36, 40 / 27, 25 / 54
    for i in range(2, N - 2):
        A[i, i - 2:i + 3] = (be, al, 1.0, al, be)
        B[i, i - 2] = -b / (4 * h)
        B[i, i - 1] = -a / (2 * h)
        B[i, i + 1] = a / (2 * h)
        B[i, i + 2] = b / (4 * h)
    for i in (1, N - 2):
        A[i, i - 1:i + 2] = (0.25, 1.0, 0.25)
        B[i, i - 1] = -1.5 / (2 * h)
        B[i, i + 1] = 1.5 / (2 * h)
    A[0, 0], A[0, 1] = 1.0, 3.0
    A[N - 1, N - 1], A[N - 1, N - 2] = 1.0, 3.0
    a0, b0, c0, d0 = -17 / 6, 1.5, 1.5, -1 / 6
    B[0, 0:4] = (a0 / h, b0 / h, c0 / h, d0 / h)
    B[N - 1, N - 1], B[N - 1, N - 2], B[N - 1, N - 3], B[N - 1, N - 4] = -a0 / h, -b0 / h, -c0 / h, -d0 / h
    return A, B


def dy1(NY, alpha):
    y, s, dyds1 = grid(NY, alpha)
    A, B = first_derivative_stencils(NY, 2.0 / (NY - 1.0))
    return (1.0 / dyds1)[:, None] * np.linalg.solve(A, B)


def wavenumbers(p):
    """kx for the NXH stored modes; kz with indices >= NZH wrapped to negative
    (src/solver.cpp:25-37, one rank)."""
    kx = np.arange(p.NXH) * p.dkx
    k = np.arange(p.NZ, dtype=np.float64)
    k[k >= p.NZH] -= p.NZ
    return kx, k * p.dkz
