"""Interior order of the compact finite differences (8: the reference's
schemes, src/compdiff.hpp; 6: the sixth-order option), checked exactly on
polynomials: a scheme of order p for the n-th derivative reproduces the
derivative of every polynomial of degree <= p + n - 1 and no higher."""
import numpy as np
import pytest

# first interior row per derivative: D1 rows 2..N-3, D2 rows 2..N-3 (3..N-4 at
# sixth order, see below), D3/D4 rows 3..N-4
ROWS = {1: 2, 2: 2, 3: 3, 4: 3}
ROWS6 = {1: 2, 2: 3, 3: 3, 4: 3}
ORDERS = {8: {1: 8, 2: 8, 3: 8, 4: 6}, 6: {1: 6, 2: 6, 3: 6, 4: 6}}


@pytest.fixture(scope="module")
def port(port_lib):
    from oracle import PortOracle
    return PortOracle()


def _residual(A, B, n, h, i, k):
    """Row i of A f^(n) - B f for f = ((s - s_i)/h)^k, relative to |B| |f|."""
    N = A.shape[0]
    x = (np.arange(N) - i).astype(float)  # (s - s_i)/h
    f = x ** k
    if k >= n:
        c = np.prod(np.arange(k - n + 1, k + 1, dtype=float))
        fn = c * x ** (k - n) / h ** n
    else:
        fn = np.zeros(N)
    r = A[i] @ fn - B[i] @ f
    return abs(r) / (np.abs(B[i]) @ np.abs(f) + 1e-300)


@pytest.mark.parametrize("order", [8, 6])
def test_interior_stencil_order(port, order):
    N = 33
    port.set_fd_order(order)
    try:
        port.init(0.01, 1.0, 1.0, 8, N, 8, 2.0, 1e-3)
        h = 2.0 / (N - 1)
        for n in (1, 2, 3, 4):
            A, B = port.stencil(n)
            p = ORDERS[order][n]
            first = (ROWS6 if order == 6 else ROWS)[n]
            for i in range(first, N - first):
                for k in range(0, p + n):
                    assert _residual(A, B, n, h, i, k) < 1e-11, (order, n, i, k)
                assert _residual(A, B, n, h, i, p + n) > 1e-6, (order, n, i, "too exact")
    finally:
        port.set_fd_order(8)


def test_boundary_rows_are_the_references(port):
    """Sixth order changes interior rows only.  D2 keeps the reference's rows
    2 and N-3 too: the reference's rows 1 and N-2 are the sixth-order scheme
    centred on nodes 2 and N-3, so a sixth-order row 2 would repeat row 1 and
    make A_2 singular."""
    N = 33
    mats = {}
    for order in (8, 6):
        port.set_fd_order(order)
        port.init(0.01, 1.0, 1.0, 8, N, 8, 2.0, 1e-3)
        mats[order] = [port.stencil(n) for n in (1, 2, 3, 4)]
    port.set_fd_order(8)
    for n in (1, 2, 3, 4):
        e = ROWS6[n]
        rows = list(range(e)) + list(range(N - e, N))
        for q in (0, 1):
            a8, a6 = mats[8][n - 1][q], mats[6][n - 1][q]
            np.testing.assert_array_equal(a8[rows], a6[rows])
    for order in (8, 6):
        for n in (1, 2, 3, 4):
            assert np.linalg.cond(mats[order][n - 1][0]) < 1e4
    # D4 is the same sixth-order scheme in both
    np.testing.assert_array_equal(mats[8][3][0], mats[6][3][0])
    np.testing.assert_array_equal(mats[8][3][1], mats[6][3][1])
