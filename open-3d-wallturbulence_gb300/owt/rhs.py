"""Right-hand sides of the implicit solves of the next step, from a solver's
state: what time_Integration assembles before its per-mode solves
(src/solver.cpp:569-574), on the host in FP64.  A measurement aid for the
precision study; the GPU step assembles these inside its mode kernel."""
import numpy as np

from .operators import wavenumbers

ALPHA = (3.0, -1.5, 1.0 / 3.0)
BETA = (3.0, -3.0, 1.0)


def implicit_rhs(solver):
    p = solver.params
    kx, kz = wavenumbers(p)
    k2 = (kx[None, :] ** 2 + kz[:, None] ** 2)[:, :, None]
    vs = sum(a * solver.get(f"vely_{l}") for l, a in enumerate(ALPHA))
    hv = sum(b * solver.get(f"Hv_{l}") for l, b in enumerate(BETA))
    sv = hv - (k2 / p.dt) * vs + solver.dy(2, vs) / p.dt
    del hv
    gs = sum(a * solver.get(f"vory_{l}") for l, a in enumerate(ALPHA))
    sg = sum(b * solver.get(f"Hg_{l}") for l, b in enumerate(BETA)) + gs / p.dt
    for x in (sv,):
        x[:, :, [0, 1, -2, -1]] = 0.0
    sg[:, :, [0, -1]] = 0.0
    return sv, sg
