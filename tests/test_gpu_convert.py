"""The FP64 <-> FP32 conversions of the mixed-precision transforms
(csrc/owt_device.cuh d2f_bits / f2d_bits, integer instructions) against the
hardware conversions, on the device through owt_convert_selftest: every
result equals the hardware's except where the documented rules differ
(ties rounded away from zero, subnormal FP32 results flushed to zero), and
the sixteen edge values (zeros, infinities, NaN, the two kinds of tie, the
largest float, overflow, the smallest normal and half of it) land where
the rules say."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


def run(lib, n, seed):
    counts = (C.c_int64 * 7)()
    from owt import lib as L
    assert lib.owt_convert_selftest(n, seed, counts) == L.OK, lib.owt_last_error(None).decode()
    return list(counts)


def test_edge_values(gpu_lib):
    from owt import lib as L
    lib = L.load(gpu_lib)
    c = run(lib, 16, 0)
    # 16 d2f samples: one tie with an even kept bit (1 + 2^-24) rounds away
    # from zero, 2^-127 is flushed, the other 14 match the hardware
    assert c[:4] == [14, 1, 1, 0], c
    assert c[6] == 0 and c[4] + c[5] == 16, c


def test_random_patterns(gpu_lib):
    from owt import lib as L
    lib = L.load(gpu_lib)
    n = 1 << 24
    c = run(lib, n, 12345)
    print("d2f equal/ties/flushed/other:", c[:4], " f2d equal/subnormal/other:", c[4:])
    assert sum(c[:4]) == n and sum(c[4:]) == n
    assert c[3] == 0 and c[6] == 0
    # 1 in 20 doubles lies below 2^-126 (14 of the 280 binades drawn) and 1
    # in 256 float patterns is a subnormal: both rules were exercised
    assert c[2] > n // 40 and c[5] > n // 512
