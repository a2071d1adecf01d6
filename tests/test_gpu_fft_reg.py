"""FP32 transforms with register-resident line transforms against the
shared-memory Stockham kernels they replace, on the same mixed-precision
state: the Lamb vector after init_fields and after a step, each against the
FP64 step, is within the 1e-6 bound of the mixed precision and within three
times the Stockham kernels' own error, for every line length with a
two-pass factorisation (576, 192, 96, 72, 48 points); for a length without
one the Stockham kernels serve both arms, so the results are bitwise equal."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


@pytest.mark.parametrize("nx,ny,nz", [(384, 33, 384), (128, 17, 128), (64, 17, 64), (48, 17, 48), (32, 17, 32),
                                      (64, 17, 48), (40, 17, 20)])
def test_register_fp32_transforms_match_stockham(gpu_lib, nx, ny, nz):
    from owt.ic import seeded_velocity
    from owt.params import CaseParams
    from owt.solver import GpuSolver
    p = CaseParams(dt=0.002, dkx=1.0, dkz=2.0, NX=nx, NY=ny, NZ=nz, alpha_mesh=2.2, nu=1e-4)
    vel = seeded_velocity(p, seed=4)
    out = {}
    for arm in ("fp64", "register", "stockham"):
        s = GpuSolver(p, precision="fp64" if arm == "fp64" else "mixed")
        s.use_stockham_fft(arm == "stockham")
        s.init_fields(*vel)
        got = {n: s.get(n) for n in ("lmbx", "lmby", "lmbz")}
        s.time_Integration(1)
        got.update({n + "_1": s.get(n) for n in ("lmbx", "lmby", "lmbz")})
        out[arm] = got
        s.close()
    err = {arm: {n: rel2(out[arm][n], out["fp64"][n]) for n in out["fp64"]} for arm in ("register", "stockham")}
    for arm in err:
        print(f"{nx}x{ny}x{nz} {arm} FP32 transforms vs FP64", {k: f"{v:.1e}" for k, v in err[arm].items()})
    if (3 * nx // 2) in (576, 192, 96, 72, 48) or (3 * nz // 2) in (576, 192, 96, 72, 48):
        for n in out["fp64"]:
            assert err["register"][n] < 1e-6, n
            assert err["register"][n] < 3 * err["stockham"][n] + 1e-8, n
    else:
        for n in out["fp64"]:
            assert np.array_equal(out["register"][n], out["stockham"][n]), n
