"""Many independent channels stepped together: one CUDA graph launch per step,
in which every kernel of the step covers all channels at once (the mode kernel
as one persistent launch over every channel's banded solves).

``minimal_channels`` draws the uneven minimal-channel ensemble: Re_tau uniform
in [150, 250] (bulk Reynolds number from Dean's correlation
Re_tau = 0.09 (2 Re_b)^0.88, velocities scaled by the bulk velocity, lengths by
the half-height, so nu = 1/Re_b), Lx in [pi, 2 pi], Lz in [0.3 pi, 0.6 pi],
modes from {32, 48, 64} x {65, 97} x {32, 48}.
"""
import ctypes as C
import math

import numpy as np

from . import lib as _L
from .params import CaseParams


def minimal_channels(n=64, seed=0, dt=0.004, alpha_mesh=2.0):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        re_tau = rng.uniform(150.0, 250.0)
        re_b = (re_tau / 0.09) ** (1.0 / 0.88) / 2.0
        lx = rng.uniform(math.pi, 2 * math.pi)
        lz = rng.uniform(0.3 * math.pi, 0.6 * math.pi)
        nx = int(rng.choice([32, 48, 64]))
        ny = int(rng.choice([65, 97]))
        nz = int(rng.choice([32, 48]))
        out.append(CaseParams(dt=dt, dkx=2 * math.pi / lx, dkz=2 * math.pi / lz, NX=nx, NY=ny, NZ=nz,
                              alpha_mesh=alpha_mesh, nu=1.0 / re_b,
                              extra={"Re_tau": re_tau, "Lx": lx, "Lz": lz}))
    return out


class Batch:
    """Step several initialised GpuSolver handles as one graph launch."""

    def __init__(self, solvers):
        self.L = _L.load()
        self.solvers = list(solvers)
        arr = (C.c_void_p * len(self.solvers))(*[s.h.value for s in self.solvers])
        b = C.c_void_p()
        rc = self.L.owt_batch_create(arr, len(self.solvers), C.byref(b))
        if rc != _L.OK:
            raise _L.OwtError(rc, self.L.owt_last_error(None).decode())
        self.b = b

    def step(self, n=1):
        rc = self.L.owt_batch_step(self.b, int(n))
        if rc != _L.OK:
            raise _L.OwtError(rc, self.L.owt_last_error(None).decode())

    def synchronize(self):
        rc = self.L.owt_batch_synchronize(self.b)
        if rc != _L.OK:
            raise _L.OwtError(rc, self.L.owt_last_error(None).decode())

    @property
    def stream(self):
        v = C.c_void_p()
        rc = self.L.owt_batch_get_stream(self.b, C.byref(v))
        if rc != _L.OK:
            raise _L.OwtError(rc, "owt_batch_get_stream")
        return v.value

    def _count(self, fn):
        v = C.c_int64()
        rc = fn(self.b, C.byref(v))
        if rc != _L.OK:
            raise _L.OwtError(rc, "batch launch count")
        return v.value

    @property
    def launch_count(self):
        """Kernels launched by this batch's steps (and its autotuner)."""
        return self._count(self.L.owt_batch_get_launch_count)

    @property
    def step_launches(self):
        """Kernels in one batch step."""
        return self._count(self.L.owt_batch_get_step_launches)

    def tuning_report(self):
        """Timings of the mode-kernel variants on this batch, and the choice."""
        return self.L.owt_batch_tuning_report(self.b).decode()

    def close(self):
        if getattr(self, "b", None):
            self.L.owt_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
