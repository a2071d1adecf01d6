"""The FP64 -> FP32 conversion of the mixed precision's mean-flow terms
(csrc/owt_device.cuh d2f_bits, integer instructions) against the hardware
conversion, on the device through owt_convert_selftest: every result equals
the hardware's except where the documented rules differ (ties rounded away
from zero, subnormal FP32 results flushed to zero), and the sixteen edge
values (zeros, infinities, NaN, the two kinds of tie, the largest float,
overflow, the smallest normal and half of it) land where the rules say."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


def run(lib, n, seed):
    from owt import lib as L
    counts = (C.c_int64 * 4)()
    assert lib.owt_convert_selftest(n, seed, counts) == L.OK, lib.owt_last_error(None).decode()
    return list(counts)


def test_edge_values(gpu_lib):
    from owt import lib as L
    lib = L.load(gpu_lib)
    # one tie with an even kept bit (1 + 2^-24) rounds away from zero, 2^-127
    # is flushed, the other 14 match the hardware
    assert run(lib, 16, 0) == [14, 1, 1, 0]


def test_random_patterns(gpu_lib):
    from owt import lib as L
    lib = L.load(gpu_lib)
    n = 1 << 24
    c = run(lib, n, 12345)
    print("equal/ties/flushed/other:", c)
    assert sum(c) == n and c[3] == 0
    # 1 in 20 samples lies below 2^-126 (14 of the 280 binades drawn)
    assert c[2] > n // 40
