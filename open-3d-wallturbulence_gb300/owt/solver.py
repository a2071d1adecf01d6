"""GPU channel-DNS solver with the reference's routine names.

The reference is a set of free functions on C++ globals (src/setup.hpp:84-114)
driven by src/main.cpp:63-87.  ``GpuSolver`` keeps those names and their
meaning on one device-resident state:

    s = GpuSolver(params)                      # allocate_var + init_mat + init_fft
    s.init_fields(velx, vely, velz)            # init_fields with a given velocity
    for step in range(NT + 1):
        s.time_Integration()                   # time_Integration
    s.get("vely")                              # the global vely, [z][x][y]

Arrays are numpy complex128 in the reference Field layout [z][x][y].
"""
import ctypes as C

import numpy as np

from . import lib as _L
from .params import CaseParams


class GpuSolver:
    def __init__(self, params: CaseParams, precision="fp64", device=0):
        self.L = _L.load()
        self.params = params
        p = _L.OwtParams(params.dt, params.dkx, params.dkz, params.alpha_mesh, params.nu, params.NX, params.NY,
                         params.NZ, _L.PREC[precision], device, int(getattr(params, "fd_order", 8)))
        h = C.c_void_p()
        rc = self.L.owt_create(C.byref(p), C.byref(h))
        if rc != _L.OK:
            raise _L.OwtError(rc, self.L.owt_last_error(None).decode())
        self.h = h
        self.shape = params.spectral_shape

    # -- plumbing -------------------------------------------------------------
    def _chk(self, rc):
        if rc != _L.OK:
            raise _L.OwtError(rc, self.L.owt_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.owt_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, a):
        a = np.ascontiguousarray(a, dtype=np.complex128)
        if a.shape != self.shape:
            raise ValueError(f"expected shape {self.shape}, got {a.shape}")
        return a

    # -- reference routines -----------------------------------------------------
    def init_fields(self, velx, vely, velz):
        u, v, w = self._c(velx), self._c(vely), self._c(velz)
        self._chk(self.L.owt_init_fields(self.h, *[_L.dptr(x.view(np.float64)) for x in (u, v, w)]))

    def init_seeded(self, seed=0, rms=0.1):
        """init_fields with the laminar + seeded random divergence-free
        velocity generated on the device (owt_init_seeded)."""
        self._chk(self.L.owt_init_seeded(self.h, int(seed), float(rms)))

    def time_Integration(self, nsteps=1):
        self._chk(self.L.owt_time_integration(self.h, int(nsteps)))

    def call(self, routine):
        self._chk(self.L.owt_call(self.h, _L.ROUTINES[routine]))

    def get_vor_from_vel(self):
        self.call("get_vor_from_vel")

    def Lamb_vec(self):
        self.call("Lamb_vec")

    def nonlinear_source(self):
        self.call("nonlinear_source")

    def solve_friction_force(self):
        self.call("solve_friction_force")

    def synchronize(self):
        self._chk(self.L.owt_synchronize(self.h))

    # -- state access -----------------------------------------------------------
    def get(self, name, out=None):
        out = np.empty(self.shape, np.complex128) if out is None else out
        self._chk(self.L.owt_get_field(self.h, _L.FIELDS.index(name), _L.dptr(out.view(np.float64))))
        return out

    def set(self, name, arr):
        a = self._c(arr)
        self._chk(self.L.owt_set_field(self.h, _L.FIELDS.index(name), _L.dptr(a.view(np.float64))))

    def get_cvec(self, name):
        out = np.empty(self.params.NY, np.complex128)
        self._chk(self.L.owt_get_mean(self.h, _L.MEANS.index(name), _L.dptr(out.view(np.float64))))
        return out

    def set_cvec(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.complex128)
        self._chk(self.L.owt_set_mean(self.h, _L.MEANS.index(name), _L.dptr(a.view(np.float64))))

    def friction(self):
        out = np.empty(6)
        self._chk(self.L.owt_get_friction(self.h, _L.dptr(out)))
        return out

    def set_friction(self, vals):
        a = np.ascontiguousarray(vals, dtype=np.float64)
        self._chk(self.L.owt_set_friction(self.h, _L.dptr(a)))

    def get_scalar(self, name):
        names = ["fx_fric_0", "fx_fric_1", "fx_fric_2", "fz_fric_0", "fz_fric_1", "fz_fric_2"]
        return float(self.friction()[names.index(name)])

    def state(self):
        d = {n: self.get(n) for n in _L.FIELDS}
        d.update({n: self.get_cvec(n) for n in _L.MEANS})
        f = self.friction()
        for q, n in enumerate(["fx_fric_0", "fx_fric_1", "fx_fric_2", "fz_fric_0", "fz_fric_1", "fz_fric_2"]):
            d[n] = float(f[q])
        return d

    def dy(self, order, field):
        a = self._c(field)
        out = np.empty(self.shape, np.complex128)
        self._chk(self.L.owt_dy_apply(self.h, int(order), _L.dptr(a.view(np.float64)), _L.dptr(out.view(np.float64))))
        return out

    HISTORY = ("vely_0", "vely_1", "vely_2", "vory_0", "vory_1", "vory_2",
               "Hv_0", "Hv_1", "Hv_2", "Hg_0", "Hg_1", "Hg_2")

    def time_Integration_host(self, hist, means, fric, vely_out=None, vory_out=None):
        """One step on a host-held state (owt_time_integration_host): `hist` the 12
        history fields in HISTORY order ([z][x][y] complex128), `means` the 12
        mean vectors as a (12, NY) complex128 array in the library's order,
        `fric` the six friction values.  Returns (vely, vory, friction)."""
        arrs = [self._c(a) for a in hist]
        if len(arrs) != 12:
            raise ValueError("12 history fields expected")
        m = np.ascontiguousarray(means, dtype=np.complex128)
        if m.shape != (12, self.params.NY):
            raise ValueError(f"means must have shape (12, {self.params.NY})")
        f = np.ascontiguousarray(fric, dtype=np.float64)
        vo = np.empty(self.shape, np.complex128) if vely_out is None else vely_out
        go = np.empty(self.shape, np.complex128) if vory_out is None else vory_out
        fo = np.empty(6)
        ptrs = (_L._dp * 12)(*[_L.dptr(a.view(np.float64)) for a in arrs])
        self._chk(self.L.owt_time_integration_host(self.h, ptrs, _L.dptr(m.view(np.float64)), _L.dptr(f),
                                                   _L.dptr(vo.view(np.float64)), _L.dptr(go.view(np.float64)),
                                                   _L.dptr(fo)))
        return vo, go, fo

    @property
    def physical_shape(self):
        p = self.params
        return (p.NZ2, p.NX2, p.NY)

    def Fourier2Physical_dealiased(self, u):
        """src/FFT.cpp:49-128 on one field: [z][x][y] complex -> [z2][x2][y] real."""
        a = self._c(u)
        out = np.empty(self.physical_shape)
        self._chk(self.L.owt_fourier2physical(self.h, _L.dptr(a.view(np.float64)), _L.dptr(out)))
        return out

    def Physical2Fourier_dealiased(self, up):
        """src/FFT.cpp:130-194 on one field: [z2][x2][y] real -> [z][x][y] complex."""
        a = np.ascontiguousarray(up, dtype=np.float64)
        if a.shape != self.physical_shape:
            raise ValueError(f"expected shape {self.physical_shape}, got {a.shape}")
        out = np.empty(self.shape, np.complex128)
        self._chk(self.L.owt_physical2fourier(self.h, _L.dptr(a), _L.dptr(out.view(np.float64))))
        return out

    def grid(self):
        y = np.empty(self.params.NY)
        self._chk(self.L.owt_get_grid(self.h, _L.dptr(y)))
        return y

    STAT_NAMES = ("U", "V", "W", "u_rms", "v_rms", "w_rms", "uv")

    def statistics(self):
        """Wall-normal profiles of the current velocity (dict of NY arrays)."""
        out = np.empty(7 * self.params.NY)
        self._chk(self.L.owt_statistics(self.h, _L.dptr(out)))
        return {n: out[q * self.params.NY:(q + 1) * self.params.NY].copy() for q, n in enumerate(self.STAT_NAMES)}

    def checkpoint(self):
        """The full state as bytes (exact restart)."""
        n = C.c_int64()
        self._chk(self.L.owt_checkpoint_bytes(self.h, C.byref(n)))
        buf = np.empty(n.value, np.uint8)
        self._chk(self.L.owt_checkpoint_save(self.h, buf.ctypes.data_as(C.c_void_p), n.value))
        return buf

    def restore(self, image):
        buf = np.ascontiguousarray(image, dtype=np.uint8)
        self._chk(self.L.owt_checkpoint_load(self.h, buf.ctypes.data_as(C.c_void_p), buf.size))

    def keep_state(self):
        """Copy the full state to a device-side slot (no host round trip)."""
        self._chk(self.L.owt_state_keep(self.h))

    def restore_state(self):
        """Return to the state saved by keep_state."""
        self._chk(self.L.owt_state_restore(self.h))

    def save_checkpoint(self, path):
        self.checkpoint().tofile(path)

    def load_checkpoint(self, path):
        self.restore(np.fromfile(path, dtype=np.uint8))

    def enqueue_stage(self, stage):
        """Enqueue one stage (0 modes, 1 mean, 2 transforms, 3 nonlinear) for timing."""
        self._chk(self.L.owt_enqueue_stage(self.h, int(stage)))

    def force_dense_bands(self, on=True):
        self._chk(self.L.owt_set_option(self.h, 1, 1 if on else 0))

    def use_stockham_fft(self, on=True):
        """FP32 transforms through the shared-memory Stockham kernels instead of
        the register-transform ones (OWT_OPT_FFT_STOCKHAM), for comparisons."""
        self._chk(self.L.owt_set_option(self.h, 3, 1 if on else 0))

    def use_mean_split(self, on=True):
        """Mixed precision: the mean-flow terms of the Lamb vector formed mode by
        mode beside the FP32 transforms of the fluctuations (the default), or
        the whole fields through FP32 (OWT_OPT_MEAN_SPLIT)."""
        self._chk(self.L.owt_set_option(self.h, 4, 1 if on else 0))

    def set_host_chunks(self, n):
        """Chunks of Fourier modes owt_time_integration_host pipelines its uploads
        over (0: the library's default; OWT_OPT_HOST_CHUNKS)."""
        self._chk(self.L.owt_set_option(self.h, 5, int(n)))

    def force_modes_variant(self, v):
        """Run mode-kernel variant v (-1: the autotuned one)."""
        self._chk(self.L.owt_set_option(self.h, 2, int(v)))

    def tuning_report(self):
        return self.L.owt_tuning_report(self.h).decode()

    def setup_report(self):
        """Wall time of the setup phases of this handle's creation."""
        return self.L.owt_setup_report(self.h).decode()

    def info(self, what):
        codes = {"sparse_solve": 1, "pattern_violations": 2, "device_bytes": 3, "modes_variant": 4,
                 "modes_variants": 5}
        v = C.c_int64()
        self._chk(self.L.owt_get_info(self.h, codes[what], C.byref(v)))
        return v.value

    # -- wall blowing/suction and the wall-drag adjoint ----------------------------
    def set_wall_velocity(self, bottom, top):
        """v on the walls as spectral wall fields [NZ, NX/2] complex (None, None: no-slip)."""
        if bottom is None and top is None:
            self._chk(self.L.owt_set_wall_velocity(self.h, None, None))
            return
        shp = self.shape[:2]
        b = np.ascontiguousarray(bottom, dtype=np.complex128)
        t = np.ascontiguousarray(top, dtype=np.complex128)
        if b.shape != shp or t.shape != shp:
            raise ValueError(f"wall fields must have shape {shp}")
        self._chk(self.L.owt_set_wall_velocity(self.h, _L.dptr(b.view(np.float64)), _L.dptr(t.view(np.float64))))

    def wall_velocity(self):
        shp = self.shape[:2]
        b = np.empty(shp, np.complex128)
        t = np.empty(shp, np.complex128)
        self._chk(self.L.owt_get_wall_velocity(self.h, _L.dptr(b.view(np.float64)), _L.dptr(t.view(np.float64))))
        return b, t

    def drag_forward(self, nsteps, interval=20):
        """Run nsteps steps; returns J = mean over the steps of the driving force fx."""
        J = C.c_double()
        self._chk(self.L.owt_drag_forward(self.h, int(nsteps), int(interval), C.byref(J)))
        return J.value

    def drag_backward(self, grad_objective=1.0):
        """dJ/d(wall velocity) of the last drag_forward, as (bottom, top) [NZ, NX/2] complex."""
        shp = self.shape[:2]
        b = np.empty(shp, np.complex128)
        t = np.empty(shp, np.complex128)
        self._chk(self.L.owt_drag_backward(self.h, float(grad_objective), _L.dptr(b.view(np.float64)),
                                           _L.dptr(t.view(np.float64))))
        return b, t

    def set_precision(self, precision):
        self._chk(self.L.owt_set_precision(self.h, _L.PREC[precision]))

    def use_graph(self, on=True):
        self._chk(self.L.owt_use_graph(self.h, 1 if on else 0))

    @property
    def step(self):
        v = C.c_int64()
        self._chk(self.L.owt_get_step(self.h, C.byref(v)))
        return v.value

    @property
    def launch_count(self):
        v = C.c_int64()
        self._chk(self.L.owt_get_launch_count(self.h, C.byref(v)))
        return v.value

    @property
    def stream(self):
        v = C.c_void_p()
        self._chk(self.L.owt_get_stream(self.h, C.byref(v)))
        return v.value
