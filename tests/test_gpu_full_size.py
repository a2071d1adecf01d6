"""Full-size (Re_tau = 550, 384 x 257 x 384) checks through size-independent
properties, plus the mixed-precision error budget against FP64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CURRENT = ["velx", "vely", "velz", "vorx", "vory", "vorz", "lmbx", "lmby", "lmbz", "Hv", "Hg"]


@pytest.fixture(scope="module")
def big():
    from owt.params import channel_550
    from owt.ic import seeded_velocity
    p = channel_550()
    return p, seeded_velocity(p, seed=0)


def rel2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def test_full_size_step_is_divergence_free_and_real(gpu_lib, big):
    from owt.solver import GpuSolver
    from owt.operators import wavenumbers
    p, (u, v, w) = big
    s = GpuSolver(p)
    s.init_fields(u, v, w)
    s.time_Integration(2)
    uu, vv, ww = s.get("velx"), s.get("vely"), s.get("velz")
    kx, kz = wavenumbers(p)
    div = 1j * kx[None, :, None] * uu + s.dy(1, vv) + 1j * kz[:, None, None] * ww
    scale = np.abs(1j * kx[None, :, None] * uu).max()
    assert np.abs(div).max() < 1e-9 * scale
    # the kx = 0 column stays Hermitian in kz (a real field)
    for k in range(1, p.NZH):
        assert np.abs(vv[p.NZ - k, 0] - np.conj(vv[k, 0])).max() <= 1e-10 * np.abs(vv[:, 0]).max()
    assert np.isfinite(s.friction()).all()


def test_mixed_precision_rhs_error(gpu_lib, big):
    """FP32 transforms and products: one-step RHS error per field vs FP64."""
    from owt.solver import GpuSolver
    p, (u, v, w) = big
    a = GpuSolver(p, precision="fp64")
    b = GpuSolver(p, precision="mixed")
    for s in (a, b):
        s.init_fields(u, v, w)
        s.time_Integration(1)
    errs = {n: rel2(b.get(n), a.get(n)) for n in ("lmbx", "lmby", "lmbz", "Hv", "Hg", "vely", "vory")}
    print("mixed vs fp64 relative L2:", {k: "%.2e" % v for k, v in errs.items()})
    assert max(errs.values()) < 1e-6
