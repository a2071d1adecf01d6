"""The minimal-channel ensemble definition (host only)."""
import math

from owt.batch import minimal_channels


def test_minimal_channel_ensemble_ranges_and_seed():
    ps = minimal_channels(64, seed=0)
    assert len(ps) == 64
    for p in ps:
        assert 150 <= p.extra["Re_tau"] <= 250
        assert math.pi <= p.extra["Lx"] <= 2 * math.pi and 0.3 * math.pi <= p.extra["Lz"] <= 0.6 * math.pi
        assert p.NX in (32, 48, 64) and p.NY in (65, 97) and p.NZ in (32, 48)
        assert abs(p.dkx - 2 * math.pi / p.extra["Lx"]) < 1e-12
    assert len({(p.NX, p.NY, p.NZ) for p in ps}) > 4        # uneven sizes
    # Re_tau 180 <-> Re_b 2800 (the channel_180 workload) under the same correlation
    assert abs((180 / 0.09) ** (1 / 0.88) / 2 - 2800) / 2800 < 0.05
    assert [p.NX for p in minimal_channels(8, seed=1)] == [p.NX for p in minimal_channels(8, seed=1)]
