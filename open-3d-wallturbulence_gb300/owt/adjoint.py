"""Wall-drag gradients with respect to wall blowing/suction.

The control is the wall-normal velocity on both walls, v(y=-1) and v(y=+1),
given as spectral wall fields [NZ, NX/2] complex (the layout of one y-line set
of a Field); the objective is the wall drag averaged over N steps,

    J = (1/N) sum_{n=1..N} fx_n ,

fx_n the driving force of step n (src/solver.cpp:306-312): the wall shear
stress averaged over both walls.  ``wall_drag`` exposes J as a differentiable
torch function: its forward runs the GPU step N times from a given state
(``owt_drag_forward``), its backward runs the hand-written discrete-adjoint
step kernels in reverse over the recomputed trajectory (``owt_drag_backward``,
checkpoints every ``interval`` steps).  Gradients follow torch's convention
for a real function of complex inputs, dJ/dRe + i dJ/dIm.
"""
import numpy as np
import torch


def seeded_wall_field(params, seed, rms=1e-3):
    """A seeded Gaussian wall field: complex Gaussian Fourier amplitudes on the
    stored modes, Hermitian on the kx = 0 column (a real physical field), the
    mean mode and the kz Nyquist row zero, scaled to physical RMS ``rms``."""
    rng = np.random.default_rng(seed)
    NZ, NXH = params.NZ, params.NX // 2
    a = rng.standard_normal((NZ, NXH)) + 1j * rng.standard_normal((NZ, NXH))
    a[NZ // 2, :] = 0.0
    a[0, 0] = 0.0
    for k in range(1, NZ // 2):
        a[NZ - k, 0] = np.conj(a[k, 0])
    power = np.sum(np.abs(a[:, 0]) ** 2) + 2.0 * np.sum(np.abs(a[:, 1:]) ** 2)
    return a * (rms / np.sqrt(power))


def _np(t):
    return np.ascontiguousarray(t.detach().cpu().numpy().astype(np.complex128))


class WallDrag(torch.autograd.Function):
    """J(vw_bottom, vw_top) for one GpuSolver; see ``wall_drag``."""

    @staticmethod
    def forward(ctx, vw_bottom, vw_top, solver, nsteps, interval, start):
        if start is not None:
            solver.restore(start)
        solver.set_wall_velocity(_np(vw_bottom), _np(vw_top))
        J = solver.drag_forward(nsteps, interval)
        ctx.solver = solver
        ctx.device = vw_bottom.device
        return torch.tensor(J, dtype=torch.float64, device=vw_bottom.device)

    @staticmethod
    def backward(ctx, gJ):
        gb, gt = ctx.solver.drag_backward(float(gJ))
        dev = ctx.device
        return torch.from_numpy(gb).to(dev), torch.from_numpy(gt).to(dev), None, None, None, None


def wall_drag(solver, vw_bottom, vw_top, nsteps, interval=20, start=None):
    """Differentiable wall drag of ``nsteps`` GPU steps under wall velocities
    ``vw_bottom``, ``vw_top`` (complex128 tensors [NZ, NX/2]).  ``start``: a
    checkpoint image (``GpuSolver.checkpoint()``) restored before the run, so
    that repeated evaluations start from the same state; without it the run
    starts from the solver's current state.  Call backward before the solver
    runs anything else (the reverse sweep replays the recorded run)."""
    return WallDrag.apply(vw_bottom, vw_top, solver, int(nsteps), int(interval), start)
