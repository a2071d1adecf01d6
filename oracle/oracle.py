"""Test infrastructure (oracle): ctypes loaders for the CPU oracle libraries.

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use
this module.  Two libraries:

* ``_ref/libowt_ref.so`` -- the reference's own ``src/solver.cpp``,
  ``src/FFT.cpp`` and ``src/parallel.cpp`` built against the shims (exists
  only where the reference sources were present at build time);
* ``_build/libowt_port.so`` -- the project's CPU restatement (``owt_port.cpp``),
  which builds anywhere.

Both speak the reference layout: complex128 interleaved, ``[z][x][y]``.
"""
import ctypes as C
import os
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(HERE, "_ref", "libowt_ref.so")
PORT_LIB = os.path.join(HERE, "_build", "libowt_port.so")

FIELD_NAMES = ["velx", "vely", "velz", "vorx", "vory", "vorz", "lmbx", "lmby", "lmbz", "Hv", "Hg",
               "vely_0", "vely_1", "vely_2", "vory_0", "vory_1", "vory_2",
               "Hv_0", "Hv_1", "Hv_2", "Hg_0", "Hg_1", "Hg_2"]
CVEC_NAMES = ["lmbx_mean_0", "lmbx_mean_1", "lmbx_mean_2", "lmbz_mean_0", "lmbz_mean_1", "lmbz_mean_2",
              "velx_mean_0", "velx_mean_1", "velx_mean_2", "velz_mean_0", "velz_mean_1", "velz_mean_2"]
SCALAR_NAMES = ["fx_fric_0", "fx_fric_1", "fx_fric_2", "fz_fric_0", "fz_fric_1", "fz_fric_2"]

_dp = C.POINTER(C.c_double)


def _ptr(a):
    return a.ctypes.data_as(_dp)


def _cplx_from(buf, shape):
    return buf.view(np.complex128).reshape(shape)


class _Common:
    """Shared accessors; ``prefix`` is ``ref_`` or ``port_``."""

    def __init__(self, path, prefix):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        self.p = prefix
        L = self.lib
        for fn, args in [("init", [C.c_double, C.c_double, C.c_double, C.c_long, C.c_long, C.c_long,
                                   C.c_double, C.c_double]),
                         ("set_velocity", [_dp, _dp, _dp]), ("step", [C.c_int]),
                         ("get_field", [C.c_char_p, _dp]), ("set_field", [C.c_char_p, _dp]),
                         ("get_cvec", [C.c_char_p, _dp]), ("set_cvec", [C.c_char_p, _dp]),
                         ("get_rvec", [C.c_char_p, _dp]), ("get_scalar", [C.c_char_p, _dp]),
                         ("set_scalar", [C.c_char_p, C.c_double]), ("get_dy", [C.c_int, _dp]),
                         ("fourier2physical", [_dp, _dp]), ("physical2fourier", [_dp, _dp]),
                         ("call", [C.c_char_p])]:
            f = getattr(L, prefix + fn)
            f.argtypes = args
            f.restype = C.c_int

    def _chk(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{self.p}{what} failed with status {rc}")

    def init(self, dt, dkx, dkz, NX, NY, NZ, alpha, nu):
        self.NX, self.NY, self.NZ = int(NX), int(NY), int(NZ)
        self.NXH, self.NX2, self.NZ2 = self.NX // 2, self.NX // 2 * 3, self.NZ // 2 * 3
        self._chk(getattr(self.lib, self.p + "init")(dt, dkx, dkz, NX, NY, NZ, alpha, nu), "init")

    @property
    def shape(self):
        return (self.NZ, self.NXH, self.NY)

    def set_velocity(self, u, v, w):
        a = [np.ascontiguousarray(x, dtype=np.complex128) for x in (u, v, w)]
        for x in a:
            assert x.shape == self.shape
        self._chk(getattr(self.lib, self.p + "set_velocity")(*[_ptr(x.view(np.float64)) for x in a]), "set_velocity")

    def step(self, n=1):
        self._chk(getattr(self.lib, self.p + "step")(int(n)), "step")

    def call(self, name):
        self._chk(getattr(self.lib, self.p + "call")(name.encode()), "call " + name)

    def get(self, name):
        out = np.empty(2 * self.NZ * self.NXH * self.NY)
        self._chk(getattr(self.lib, self.p + "get_field")(name.encode(), _ptr(out)), "get_field " + name)
        return _cplx_from(out, self.shape)

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.complex128)
        assert a.shape == self.shape
        self._chk(getattr(self.lib, self.p + "set_field")(name.encode(), _ptr(a.view(np.float64))), "set_field " + name)

    def get_cvec(self, name):
        out = np.empty(2 * self.NY)
        self._chk(getattr(self.lib, self.p + "get_cvec")(name.encode(), _ptr(out)), "get_cvec " + name)
        return out.view(np.complex128).copy()

    def set_cvec(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.complex128)
        self._chk(getattr(self.lib, self.p + "set_cvec")(name.encode(), _ptr(a.view(np.float64))), "set_cvec " + name)

    def get_rvec(self, name, n=None):
        n = n or max(self.NY, self.NXH, self.NZ)
        out = np.zeros(n)
        self._chk(getattr(self.lib, self.p + "get_rvec")(name.encode(), _ptr(out)), "get_rvec " + name)
        if name == "kx_local":
            return out[: self.NXH].copy()
        if name == "kz_local":
            return out[: self.NZ].copy()
        return out[: self.NY].copy()

    def get_scalar(self, name):
        out = np.zeros(1)
        self._chk(getattr(self.lib, self.p + "get_scalar")(name.encode(), _ptr(out)), "get_scalar " + name)
        return float(out[0])

    def set_scalar(self, name, val):
        self._chk(getattr(self.lib, self.p + "set_scalar")(name.encode(), float(val)), "set_scalar " + name)

    def dy(self, which):
        out = np.empty(self.NY * self.NY)
        self._chk(getattr(self.lib, self.p + "get_dy")(int(which), _ptr(out)), "get_dy")
        return out.reshape(self.NY, self.NY)

    def fourier2physical(self, u):
        a = np.ascontiguousarray(u, dtype=np.complex128)
        out = np.empty(self.NZ2 * self.NX2 * self.NY)
        self._chk(getattr(self.lib, self.p + "fourier2physical")(_ptr(a.view(np.float64)), _ptr(out)), "f2p")
        return out.reshape(self.NZ2, self.NX2, self.NY)

    def physical2fourier(self, p):
        a = np.ascontiguousarray(p, dtype=np.float64)
        out = np.empty(2 * self.NZ * self.NXH * self.NY)
        self._chk(getattr(self.lib, self.p + "physical2fourier")(_ptr(a), _ptr(out)), "p2f")
        return _cplx_from(out, self.shape)

    def state(self):
        """Every per-step state array of the reference globals, as a dict."""
        d = {n: self.get(n) for n in FIELD_NAMES}
        d.update({n: self.get_cvec(n) for n in CVEC_NAMES})
        d.update({n: self.get_scalar(n) for n in SCALAR_NAMES})
        return d


class RefOracle(_Common):
    """The reference time step built from its own sources (see Makefile)."""

    def __init__(self, path=REF_LIB):
        super().__init__(path, "ref_")
        self.lib.ref_quiet.argtypes = [C.c_int]
        self.lib.ref_init_fields_builtin.restype = C.c_int

    def init_fields_builtin(self):
        self._chk(self.lib.ref_init_fields_builtin(), "init_fields_builtin")


class PortOracle(_Common):
    """The project's CPU restatement of the reference time step."""

    def __init__(self, path=PORT_LIB):
        super().__init__(path, "port_")
        self.lib.port_set_threads.argtypes = [C.c_int]
        self.lib.port_set_threads.restype = C.c_int
        self.lib.port_init_fields_builtin.restype = C.c_int
        self.lib.port_time_modes.argtypes = [C.c_long, C.c_long]
        self.lib.port_time_modes.restype = C.c_double
        self.lib.port_time_transforms.argtypes = [C.c_long]
        self.lib.port_time_transforms.restype = C.c_double
        self.lib.port_set_wall_velocity.argtypes = [_dp, _dp]
        self.lib.port_set_wall_velocity.restype = C.c_int
        self.lib.port_set_fd_order.argtypes = [C.c_int]
        self.lib.port_set_fd_order.restype = C.c_int
        self.lib.port_get_stencil.argtypes = [C.c_int, _dp, _dp]
        self.lib.port_get_stencil.restype = C.c_int

    def set_fd_order(self, order):
        """Interior compact-FD order (8: the reference's, 6); takes effect at init."""
        self._chk(self.lib.port_set_fd_order(int(order)), "set_fd_order")

    def stencil(self, which):
        """The raw A_n, B_n (n = which) on the uniform s-grid, dense [NY, NY]."""
        a = np.empty(self.NY * self.NY)
        b = np.empty(self.NY * self.NY)
        self._chk(self.lib.port_get_stencil(int(which), _ptr(a), _ptr(b)), "get_stencil")
        return a.reshape(self.NY, self.NY), b.reshape(self.NY, self.NY)

    def set_wall_velocity(self, bottom, top):
        """Wall blowing/suction [NZ, NX/2] complex per wall; None, None: no-slip."""
        if bottom is None:
            self._chk(self.lib.port_set_wall_velocity(None, None), "set_wall_velocity")
            return
        b = np.ascontiguousarray(bottom, dtype=np.complex128).reshape(-1).view(np.float64)
        t = np.ascontiguousarray(top, dtype=np.complex128).reshape(-1).view(np.float64)
        self._chk(self.lib.port_set_wall_velocity(_ptr(b), _ptr(t)), "set_wall_velocity")

    def set_threads(self, n):
        return self.lib.port_set_threads(int(n))

    def init_fields_builtin(self):
        self._chk(self.lib.port_init_fields_builtin(), "init_fields_builtin")


def ref_available():
    return os.path.exists(REF_LIB)
