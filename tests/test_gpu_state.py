"""Statistics, exact restart and snapshots on the GPU state."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ["velx", "vely", "velz", "vorx", "vory", "vorz", "lmbx", "lmby", "lmbz", "Hv", "Hg",
          "vely_0", "vely_1", "vely_2", "vory_0", "vory_1", "vory_2", "Hv_0", "Hv_1", "Hv_2", "Hg_0", "Hg_1", "Hg_2"]


@pytest.fixture
def run():
    from owt.params import CaseParams
    from owt.ic import seeded_velocity
    from owt.solver import GpuSolver
    p = CaseParams(dt=0.005, dkx=0.5, dkz=1.5, NX=32, NY=33, NZ=24, alpha_mesh=2.0, nu=1 / 2800.)
    s = GpuSolver(p)
    s.init_fields(*seeded_velocity(p, seed=4))
    return p, s


def test_statistics_match_host_parseval(gpu_lib, run):
    from owt.snapshot import statistics_from_fields
    p, s = run
    s.time_Integration(3)
    got = s.statistics()
    want = statistics_from_fields(s.get("velx"), s.get("vely"), s.get("velz"), p.NZH)
    for k in want:
        np.testing.assert_allclose(got[k], want[k], rtol=1e-12, atol=1e-14 * max(1.0, np.abs(want[k]).max()))
    assert got["u_rms"].max() > 0.01 and abs(got["U"].max() - 1.5) < 0.1


@pytest.mark.parametrize("graph", [False, True])
def test_restart_from_checkpoint_is_bitwise(gpu_lib, run, graph):
    p, s = run
    s.use_graph(graph)
    s.time_Integration(4)        # ring head not at its start value
    image = s.checkpoint()
    s.time_Integration(3)
    a = {n: s.get(n) for n in FIELDS}
    fa = s.friction()
    s.restore(image)
    assert s.step == 4
    s.time_Integration(3)
    for n in FIELDS:
        np.testing.assert_array_equal(s.get(n), a[n], err_msg=n)
    np.testing.assert_array_equal(s.friction(), fa)


def test_checkpoint_rejects_other_parameters(gpu_lib, run):
    from owt.lib import OwtError
    from owt.params import CaseParams
    from owt.solver import GpuSolver
    p, s = run
    img = s.checkpoint()
    q = CaseParams(dt=0.004, dkx=0.5, dkz=1.5, NX=32, NY=33, NZ=24, alpha_mesh=2.0, nu=1 / 2800.)
    t = GpuSolver(q)
    with pytest.raises(OwtError):
        t.restore(img)


def test_snapshot_round_trip(gpu_lib, run, tmp_path):
    from owt.snapshot import save_instant_field, load_instant_field
    p, s = run
    s.time_Integration(2)
    path = save_instant_field(s, 2, directory=str(tmp_path / "DATA"))
    assert path.endswith("F-00000002.H5")
    d = load_instant_field(path)
    for n in ("velx", "vely", "velz"):
        np.testing.assert_array_equal(d[n], s.get(n))
        assert d[n].shape == (p.NZ, p.NXH, p.NY)


@pytest.mark.parametrize("graph", [False, True])
def test_smaller_channel_created_later_leaves_larger_one_working(gpu_lib, graph):
    """Kernel shared-memory limits are per function, not per handle: creating a
    smaller channel after a larger one must not break the larger one's step."""
    from owt.params import CaseParams
    from owt.ic import seeded_velocity
    from owt.solver import GpuSolver
    big = CaseParams(dt=0.004, dkx=1.0, dkz=2.0, NX=96, NY=97, NZ=96, alpha_mesh=2.0, nu=1 / 3000.)
    small = CaseParams(dt=0.004, dkx=1.0, dkz=2.0, NX=16, NY=17, NZ=16, alpha_mesh=2.0, nu=1 / 3000.)
    ref = GpuSolver(big)
    ref.use_graph(graph)
    ref.init_fields(*seeded_velocity(big, seed=1))
    ref.time_Integration(2)
    want = ref.get("vely")
    ref.close()
    s = GpuSolver(big)
    s.use_graph(graph)
    s.init_fields(*seeded_velocity(big, seed=1))
    t = GpuSolver(small)
    t.init_fields(*seeded_velocity(small, seed=1))
    t.time_Integration(1)
    s.time_Integration(2)
    np.testing.assert_array_equal(s.get("vely"), want)


def test_batch_step_matches_individual_steps(gpu_lib):
    """Channels of uneven sizes stepped as one graph launch give the same bits
    as stepping each alone."""
    from owt.batch import minimal_channels, Batch
    from owt.ic import seeded_velocity
    from owt.solver import GpuSolver
    ps = minimal_channels(4, seed=2)
    alone, batched = [], []
    for q, p in enumerate(ps):
        for group in (alone, batched):
            s = GpuSolver(p, precision="mixed")
            s.init_fields(*seeded_velocity(p, seed=q))
            group.append(s)
    b = Batch(batched)
    b.step(3)
    b.synchronize()
    for s in alone:
        s.time_Integration(3)
    for a, c in zip(alone, batched):
        assert c.step == 3
        for n in ("vely", "vory", "velx", "Hv", "lmbz"):
            np.testing.assert_array_equal(a.get(n), c.get(n))
        np.testing.assert_array_equal(a.friction(), c.friction())
    # one graph launch of batched kernels: far fewer than one kernel set per channel
    assert b.step_launches <= 12, b.step_launches
    assert "->" in b.tuning_report()
    b.close()


def test_batch_of_66_mixed_channels_matches_individual_steps(gpu_lib):
    """More channels than one launch table holds (64), FP64 and mixed-precision
    channels, sixth-order channels (full-band solve), uneven sizes including
    lines with a radix-5 stage, and one channel with wall blowing/suction:
    every channel's bits equal stepping it alone, and creating the batch
    (which times the mode-kernel variants on the live state) leaves every
    channel's state untouched."""
    from owt.adjoint import seeded_wall_field
    from owt.batch import Batch
    from owt.ic import seeded_velocity
    from owt.params import CaseParams
    from owt.solver import GpuSolver
    sizes = [(16, 33, 16), (16, 17, 24), (24, 33, 16), (20, 25, 40)]  # the last: radix-5 lines
    ps, precs = [], []
    for q in range(66):
        nx, ny, nz = sizes[q % 4]
        ps.append(CaseParams(dt=0.004, dkx=0.5 + 0.01 * q, dkz=1.5, NX=nx, NY=ny, NZ=nz, alpha_mesh=2.0,
                             nu=1 / 2800., fd_order=6 if q % 11 == 3 else 8))
        precs.append("fp64" if q % 3 == 0 else "mixed")
    alone, batched = [], []
    for q, p in enumerate(ps):
        for group in (alone, batched):
            s = GpuSolver(p, precision=precs[q])
            s.init_fields(*seeded_velocity(p, seed=q))
            if q == 5:
                s.set_wall_velocity(seeded_wall_field(p, 1), seeded_wall_field(p, 2))
            group.append(s)
    before = [(s.get("vely"), s.get("velx"), s.get("vory")) for s in batched]
    b = Batch(batched)
    b.synchronize()
    for s, (v, u, g) in zip(batched, before):
        np.testing.assert_array_equal(s.get("vely"), v)
        np.testing.assert_array_equal(s.get("velx"), u)
        np.testing.assert_array_equal(s.get("vory"), g)
    b.step(2)
    b.synchronize()
    for s in alone:
        s.time_Integration(2)
    for q, (a, c) in enumerate(zip(alone, batched)):
        for n in ("vely", "vory", "velx", "velz", "Hv", "Hg"):
            np.testing.assert_array_equal(a.get(n), c.get(n), err_msg=f"channel {q} {n}")
        np.testing.assert_array_equal(a.friction(), c.friction())
    b.close()


def test_state_keep_and_restore_on_device(gpu_lib, run):
    p, s = run
    s.time_Integration(2)
    s.keep_state()
    s.time_Integration(3)
    first = s.get("vely"), s.get("Hg"), s.friction(), s.step
    s.restore_state()
    assert s.step == 2
    s.time_Integration(3)
    np.testing.assert_array_equal(s.get("vely"), first[0])
    np.testing.assert_array_equal(s.get("Hg"), first[1])
    np.testing.assert_array_equal(s.friction(), first[2])
    assert s.step == first[3]


@pytest.mark.parametrize("precision,variant", [("fp64", None), ("mixed", None), ("fp64", "quad"), ("mixed", "quad")])
def test_host_state_step_equals_device_step(gpu_lib, precision, variant):
    """owt_time_integration_host (one step on a host-held state, copies
    overlapped with the device work) gives the bits of uploading the same
    state with the set-field calls and stepping, whatever the receiving
    handle's own ring position: the returned v, omega_y and friction, and the
    handle's state afterwards, on two calls in a row, the first from pageable
    host memory (copy-engine uploads), the second from pinned memory (uploads
    by SM loads).  With a quad-mapping mode kernel the call pipelines the
    uploads with the mode kernel over chunks of Fourier modes; the result is
    the same bits.  Both re-derive the
    DY2 v history of the uploaded v levels, which an uninterrupted run
    carries from its own solves, so against the uninterrupted step they
    agree to the one-step bound (1e-10)."""
    from owt.ic import seeded_velocity
    from owt.params import CaseParams
    from owt.solver import GpuSolver
    # NY = 129: long enough for the masked (sparse) solves the quad mapping serves
    p = CaseParams(dt=0.002, dkx=1.0, dkz=2.0, NX=32, NY=129 if variant else 33, NZ=24, alpha_mesh=2.2, nu=1e-4)
    means_names = ("lmbx_mean_0", "lmbx_mean_1", "lmbx_mean_2", "lmbz_mean_0", "lmbz_mean_1", "lmbz_mean_2",
                   "velx_mean_0", "velx_mean_1", "velx_mean_2", "velz_mean_0", "velz_mean_1", "velz_mean_2")
    a = GpuSolver(p, precision=precision)
    a.init_fields(*seeded_velocity(p, seed=3))
    a.time_Integration(2)
    hist = [a.get(n) for n in GpuSolver.HISTORY]
    means = np.stack([a.get_cvec(n) for n in means_names])
    fric = a.friction()
    c = GpuSolver(p, precision=precision)
    c.init_fields(*seeded_velocity(p, seed=9))
    for n, x in zip(GpuSolver.HISTORY, hist):
        c.set(n, x)
    for n, x in zip(means_names, means):
        c.set_cvec(n, x)
    c.set_friction(fric)
    c.time_Integration(1)
    a.time_Integration(1)
    b = GpuSolver(p, precision=precision)
    b.init_fields(*seeded_velocity(p, seed=9))
    b.time_Integration(1)  # a different ring position than c's (and the autotuner's report)
    if variant == "quad":
        assert b.info("sparse_solve") == 1
        names = [t.split("=")[0] for t in b.tuning_report().split(" -> ")[0].split()]
        assert len(names) == b.info("modes_variants")
        b.force_modes_variant(names.index(next(n for n in names if n.startswith("quad/"))))
    import torch

    def pinned(x):
        t = torch.empty(x.shape + (2,), dtype=torch.float64, pin_memory=True).numpy().view(np.complex128)
        t = t.reshape(x.shape)
        t[...] = x
        return t

    # pageable history (copy-engine uploads), then pinned (uploads by SM loads)
    for h_in in (hist, [pinned(x) for x in hist]):
        v, g, f = b.time_Integration_host(h_in, means, fric)
        np.testing.assert_array_equal(v, c.get("vely"))
        np.testing.assert_array_equal(g, c.get("vory"))
        np.testing.assert_array_equal(f, c.friction())
        for n in ("velx", "vorz", "lmbx", "lmbz", "Hv", "Hg", "vely_1", "Hv_2"):
            np.testing.assert_array_equal(b.get(n), c.get(n))
        for x, y in ((v, a.get("vely")), (g, a.get("vory"))):
            assert np.abs(x - y).max() <= 1e-10 * np.abs(y).max()
