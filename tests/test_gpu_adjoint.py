"""Wall blowing/suction and the discrete adjoint of the wall drag, on the GPU.

Forward with blowing is checked against the CPU port (which puts the wall
velocity in the same boundary rows as the reference's zeros); the hand-written
adjoint against (a) reverse-mode autodiff through a float64 PyTorch
restatement of the same step (an FP64 reference gradient, no finite-difference
noise) and (b) central finite differences of the GPU forward itself at the
Re_tau=180 size over 200 steps.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SMALL = dict(dt=0.005, dkx=0.5, dkz=1.5, NX=16, NY=33, NZ=16, alpha_mesh=2.0, nu=1 / 2800.)


def _case(**kw):
    from owt.params import CaseParams
    d = dict(SMALL)
    d.update(kw)
    return CaseParams(**d)


def _solver(p, seed=3):
    from owt.ic import seeded_velocity
    from owt.solver import GpuSolver
    s = GpuSolver(p)
    s.init_fields(*seeded_velocity(p, seed=seed))
    return s


def _walls(p, s0=11, s1=12, rms=1e-3):
    from owt.adjoint import seeded_wall_field
    return seeded_wall_field(p, s0, rms), seeded_wall_field(p, s1, rms)


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


def test_blowing_step_matches_oracle(gpu_lib, port_lib):
    from oracle import PortOracle
    from owt.ic import seeded_velocity
    p = _case()
    vb, vt = _walls(p)
    s = _solver(p)
    s.set_wall_velocity(vb, vt)
    port = PortOracle()
    port.init(p.dt, p.dkx, p.dkz, p.NX, p.NY, p.NZ, p.alpha_mesh, p.nu)
    port.set_velocity(*seeded_velocity(p, seed=3))
    port.set_wall_velocity(vb, vt)
    try:
        _blowing_steps(s, port, vb, vt)
    finally:
        port.set_wall_velocity(None, None)


def _blowing_steps(s, port, vb, vt):
    for n in range(3):
        s.time_Integration(1)
        port.step(1)
        for name in ("vely", "vory", "velx", "velz", "Hv", "Hg"):
            a, b = s.get(name), port.get(name)
            err = np.abs(a - b).max() / np.abs(b).max()
            assert err < 1e-10, (n, name, err)
        # the wall rows carry the prescribed velocity
        v = s.get("vely")
        np.testing.assert_allclose(v[..., 0], vb, rtol=0, atol=1e-15)
        np.testing.assert_allclose(v[..., -1], vt, rtol=0, atol=1e-15)
        assert abs(s.friction()[0] - port.get_scalar("fx_fric")) < 1e-12 * abs(port.get_scalar("fx_fric"))


def test_zero_wall_velocity_is_no_slip_bitwise(gpu_lib):
    p = _case()
    a, b = _solver(p), _solver(p)
    z = np.zeros(p.spectral_shape[:2], np.complex128)
    b.set_wall_velocity(z, z)
    a.time_Integration(3)
    b.time_Integration(3)
    np.testing.assert_array_equal(a.get("vely"), b.get("vely"))
    np.testing.assert_array_equal(a.get("Hv"), b.get("Hv"))
    b.set_wall_velocity(None, None)
    bw, tw = b.wall_velocity()
    assert not bw.any() and not tw.any()


def _torch_reference(p, s, vb, vt, nsteps):
    """J and dJ/dvw by autodiff through the float64 torch restatement, from the GPU state."""
    from oracle import PortOracle
    from torch_step import TorchChannel
    port = PortOracle()
    port.init(p.dt, p.dkx, p.dkz, p.NX, p.NY, p.NZ, p.alpha_mesh, p.nu)
    tc = TorchChannel(port, p.dt, p.nu)
    st = TorchChannel.state_from(s.get, s.get_cvec, s.friction)
    vbt = torch.tensor(vb, requires_grad=True)
    vtt = torch.tensor(vt, requires_grad=True)
    J, _ = tc.drag(st, vbt, vtt, nsteps)
    J.backward()
    return J.item(), vbt.grad.numpy(), vtt.grad.numpy()


@pytest.mark.parametrize("nsteps,interval,size", [(6, 4, None), (5, 1, None), (4, 10, None), (4, 2, (20, 21, 40))])
def test_adjoint_matches_autodiff_reference(gpu_lib, port_lib, nsteps, interval, size):
    """The last case has lines with a radix-5 stage (3NX/2, 3NZ/2 = 30, 60)."""
    p = _case() if size is None else _case(NX=size[0], NY=size[1], NZ=size[2])
    vb, vt = _walls(p)
    s = _solver(p)
    s.time_Integration(2)  # start from a state with distinct history levels
    s.set_wall_velocity(vb, vt)
    Jr, gbr, gtr = _torch_reference(p, s, vb, vt, nsteps)
    J = s.drag_forward(nsteps, interval)
    gb, gt = s.drag_backward()
    print(f"N={nsteps} interval={interval}: J {J:.15e} ref {Jr:.15e}; grad rel err bottom "
          f"{_rel(gb, gbr):.2e} top {_rel(gt, gtr):.2e}")
    assert abs(J - Jr) <= 1e-12 * abs(Jr)
    assert _rel(gb, gbr) < 1e-9 and _rel(gt, gtr) < 1e-9


def test_adjoint_restores_state_and_repeats(gpu_lib):
    from owt.lib import OwtError
    p = _case()
    vb, vt = _walls(p)
    s = _solver(p)
    s.set_wall_velocity(vb, vt)
    s.drag_forward(7, 3)
    after = s.get("vely"), s.get("Hg"), s.friction(), s.step
    g1 = s.drag_backward()
    np.testing.assert_array_equal(s.get("vely"), after[0])
    np.testing.assert_array_equal(s.get("Hg"), after[1])
    np.testing.assert_array_equal(s.friction(), after[2])
    assert s.step == after[3]
    g2 = s.drag_backward(2.0)
    np.testing.assert_array_equal(g2[0], 2.0 * g1[0])
    np.testing.assert_array_equal(g2[1], 2.0 * g1[1])
    s.time_Integration(1)
    with pytest.raises(OwtError):
        s.drag_backward()


def test_adjoint_masked_transposed_solve_equals_full_band(gpu_lib):
    """Where the forward's masked v-system solve applies, the adjoint's
    transposed v solve skips the entries outside the same interior masks
    (exact zeros in every factorization the setup check admitted): the
    objective and the gradient are bitwise those of the full-band forward and
    adjoint."""
    p = _case(NY=97)
    vb, vt = _walls(p)
    out = []
    for dense in (False, True):
        s = _solver(p)
        s.force_dense_bands(dense)
        assert s.info("sparse_solve") == (0 if dense else 1)
        s.set_wall_velocity(vb, vt)
        J = s.drag_forward(4, 2)
        out.append((J,) + s.drag_backward())
    assert out[0][0] == out[1][0]
    np.testing.assert_array_equal(out[0][1], out[1][1])
    np.testing.assert_array_equal(out[0][2], out[1][2])


def test_adjoint_graph_and_eager_recompute_agree(gpu_lib):
    p = _case()
    vb, vt = _walls(p)
    out = []
    for graph in (False, True):
        s = _solver(p)
        s.use_graph(graph)
        s.set_wall_velocity(vb, vt)
        J = s.drag_forward(5, 2)
        out.append((J,) + s.drag_backward())
    assert out[0][0] == out[1][0]
    np.testing.assert_array_equal(out[0][1], out[1][1])
    np.testing.assert_array_equal(out[0][2], out[1][2])


def test_wall_drag_autograd_function(gpu_lib):
    from owt.adjoint import wall_drag
    p = _case()
    vb, vt = _walls(p)
    s = _solver(p)
    start = s.checkpoint()
    tb = torch.tensor(vb, requires_grad=True)
    tt = torch.tensor(vt, requires_grad=True)
    J = wall_drag(s, tb, tt, 6, interval=3, start=start)
    (3.0 * J).backward()
    s.restore(start)
    s.set_wall_velocity(vb, vt)
    J2 = s.drag_forward(6, 3)
    gb, gt = s.drag_backward(3.0)
    assert J.item() == J2
    np.testing.assert_array_equal(tb.grad.numpy(), gb)
    np.testing.assert_array_equal(tt.grad.numpy(), gt)


def test_adjoint_fd_channel180(gpu_lib):
    """Re_tau=180, 128x129x128, dt=0.005: the gradient of the 200-step wall
    drag against central differences (eps=1e-6) along 8 seeded directions."""
    from owt.adjoint import seeded_wall_field
    from owt.ic import seeded_velocity
    from owt.params import channel_180
    from owt.solver import GpuSolver
    p = channel_180()
    s = GpuSolver(p)
    s.use_graph(True)
    s.init_fields(*seeded_velocity(p, seed=0))
    start = s.checkpoint()
    vb, vt = seeded_wall_field(p, 1), seeded_wall_field(p, 2)
    nsteps, eps = 200, 1e-6
    s.set_wall_velocity(vb, vt)
    J0 = s.drag_forward(nsteps, 20)
    gb, gt = s.drag_backward()

    def J(db, dt_, sgn):
        s.restore(start)
        s.set_wall_velocity(vb + sgn * eps * db, vt + sgn * eps * dt_)
        return s.drag_forward(nsteps, nsteps)

    worst = 0.0
    for q in range(1, 9):
        db, dt_ = seeded_wall_field(p, 100 + q, 1.0), seeded_wall_field(p, 200 + q, 1.0)
        fd = (J(db, dt_, 1) - J(db, dt_, -1)) / (2 * eps)
        ad = float(np.real(np.vdot(gb, db) + np.vdot(gt, dt_)))
        rel = abs(fd - ad) / abs(ad)
        worst = max(worst, rel)
        print(f"direction {q}: adjoint {ad:.10e}  central difference {fd:.10e}  rel {rel:.2e}")
    print(f"J = {J0:.12e}, worst relative difference {worst:.2e}")
    assert worst <= 1e-5
