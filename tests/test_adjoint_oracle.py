"""CPU checks of the wall-drag gradient's references: the float64 PyTorch
restatement of the step against the CPU port (with and without wall
blowing/suction), and its autodiff gradient against central differences of
the port."""
import numpy as np
import pytest
import torch

SMALL = dict(dt=0.005, dkx=0.5, dkz=1.5, NX=16, NY=33, NZ=16, alpha_mesh=2.0, nu=1 / 2800.)


@pytest.fixture(scope="module")
def setup(port_lib):
    from oracle import PortOracle
    from owt.ic import seeded_velocity
    from owt.params import CaseParams
    from torch_step import TorchChannel
    p = CaseParams(**SMALL)
    port = PortOracle()
    port.set_threads(4)
    port.init(p.dt, p.dkx, p.dkz, p.NX, p.NY, p.NZ, p.alpha_mesh, p.nu)
    vel = seeded_velocity(p, seed=3)
    port.set_velocity(*vel)
    fr = lambda: [port.get_scalar(f"fx_fric_{l}") for l in range(3)] + \
        [port.get_scalar(f"fz_fric_{l}") for l in range(3)]
    st0 = TorchChannel.state_from(port.get, port.get_cvec, fr)
    return p, port, vel, st0, TorchChannel(port, p.dt, p.nu)


def _port_drag(port, vel, vb, vt, nsteps):
    port.set_velocity(*vel)
    port.set_wall_velocity(vb, vt)
    acc = 0.0
    for _ in range(nsteps):
        port.step(1)
        acc += port.get_scalar("fx_fric")
    return acc / nsteps


def test_seeded_wall_field_is_real_zero_mean_with_rms():
    from owt.adjoint import seeded_wall_field
    from owt.params import CaseParams
    p = CaseParams(**SMALL)
    a = seeded_wall_field(p, 4, rms=1e-3)
    NZ, NXH = a.shape
    assert a[0, 0] == 0 and not a[NZ // 2].any()
    np.testing.assert_array_equal(a[NZ - np.arange(1, NZ // 2), 0], np.conj(a[np.arange(1, NZ // 2), 0]))
    # physical field on the NX x NZ grid (Hermitian extension in x)
    full = np.zeros((NZ, p.NX), np.complex128)
    full[:, :NXH] = a
    full[:, p.NX - np.arange(1, NXH)] = np.conj(a[(-np.arange(NZ)) % NZ][:, 1:NXH])
    phys = np.fft.ifft2(full, norm="forward")
    assert np.abs(phys.imag).max() < 1e-15
    assert abs(np.sqrt(np.mean(phys.real ** 2)) - 1e-3) < 1e-15


def test_port_zero_wall_velocity_is_no_slip(setup):
    p, port, vel, _, _ = setup
    z = np.zeros(p.spectral_shape[:2], np.complex128)
    port.set_velocity(*vel)
    port.set_wall_velocity(None, None)
    port.step(2)
    a = port.get("vely")
    port.set_velocity(*vel)
    port.set_wall_velocity(z, z)
    port.step(2)
    np.testing.assert_array_equal(port.get("vely"), a)
    port.set_wall_velocity(None, None)


def test_torch_step_matches_port_with_blowing(setup):
    from owt.adjoint import seeded_wall_field
    p, port, vel, st0, tc = setup
    vb, vt = seeded_wall_field(p, 11), seeded_wall_field(p, 12)
    Jp = _port_drag(port, vel, vb, vt, 3)
    J, st = tc.drag(st0, torch.tensor(vb), torch.tensor(vt), 3)
    assert abs(J.item() - Jp) <= 1e-12 * abs(Jp)
    for name, key in (("vely_0", "v0"), ("vory_0", "g0"), ("Hv_0", "hv0"), ("Hg_0", "hg0")):
        a, b = port.get(name), st[key].numpy()
        assert np.abs(a - b).max() <= 1e-9 * np.abs(a).max(), name
    np.testing.assert_allclose(st["v0"].numpy()[..., 0], vb, atol=1e-16)
    port.set_wall_velocity(None, None)


def test_torch_autodiff_gradient_matches_port_differences(setup):
    from owt.adjoint import seeded_wall_field
    p, port, vel, st0, tc = setup
    vb, vt = seeded_wall_field(p, 11), seeded_wall_field(p, 12)
    tb = torch.tensor(vb, requires_grad=True)
    tt = torch.tensor(vt, requires_grad=True)
    J, _ = tc.drag(st0, tb, tt, 3)
    J.backward()
    eps = 1e-6
    for q in range(2):
        db, dt_ = seeded_wall_field(p, 100 + q, 1.0), seeded_wall_field(p, 200 + q, 1.0)
        fd = (_port_drag(port, vel, vb + eps * db, vt + eps * dt_, 3) -
              _port_drag(port, vel, vb - eps * db, vt - eps * dt_, 3)) / (2 * eps)
        ad = float(np.real(np.vdot(tb.grad.numpy(), db) + np.vdot(tt.grad.numpy(), dt_)))
        assert abs(fd - ad) <= 1e-4 * abs(ad), (q, fd, ad)
    port.set_wall_velocity(None, None)


def test_port_init_clears_wall_velocity(setup):
    """A wall velocity belongs to one grid; re-initialising the port drops it."""
    from owt.adjoint import seeded_wall_field
    p, port, vel, _, _ = setup
    port.set_velocity(*vel)
    port.step(1)
    want = port.get("vely")
    port.set_wall_velocity(seeded_wall_field(p, 1), seeded_wall_field(p, 2))
    port.init(p.dt, p.dkx, p.dkz, p.NX, p.NY, p.NZ, p.alpha_mesh, p.nu)
    port.set_velocity(*vel)
    port.step(1)
    np.testing.assert_array_equal(port.get("vely"), want)
