"""GB300-native channel-DNS time step (Open-3D-WallTurbulence method).

Python side of the library: case parameters, seeded initial conditions, the
ctypes binding of the C ABI (``libowt_gpu.so``) and a solver object that keeps
the reference's routine names.  The compute path is the CUDA library; nothing
here computes a time step.
"""
from .params import CaseParams, load_params, channel_180, channel_550  # noqa: F401
from .ic import seeded_velocity  # noqa: F401,E402
