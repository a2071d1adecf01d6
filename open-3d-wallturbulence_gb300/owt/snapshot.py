"""Snapshots in the reference's layout.

The reference writes ``./DATA/F-%08d.H5`` every ``save_interval`` steps with
datasets ``velx_real, velx_imag, vely_*, velz_*`` of global shape
[NZ][NXH][NY], float64 (src/IO.cpp:118-156, 198-235).  The same file, names,
shapes and type are written here by ``owt.h5lite`` (the HDF5 file format
written directly: no HDF5 library is installed with this package).
"""
import os

import numpy as np

from . import h5lite


def save_instant_field(solver, id_step, directory="DATA"):
    os.makedirs(directory, exist_ok=True)
    path = os.path.join(directory, "F-%08d.H5" % id_step)
    data = {}
    for name in ("velx", "vely", "velz"):
        f = solver.get(name)
        data[name + "_real"] = np.ascontiguousarray(f.real)
        data[name + "_imag"] = np.ascontiguousarray(f.imag)
    h5lite.write(path, data)
    return path


def load_instant_field(path):
    d = h5lite.read(path)
    return {n: d[n + "_real"] + 1j * d[n + "_imag"] for n in ("velx", "vely", "velz")}


def statistics_from_fields(u, v, w, nz_half):
    """Host restatement of owt_statistics (same Parseval rules), for checks."""
    NZ = u.shape[0]

    def herm(f):
        g = f.copy()
        kk = np.arange(NZ)
        kp = (NZ - kk) % NZ
        g[:, 0] = 0.5 * (f[:, 0] + np.conj(f[kp, 0]))
        return g

    uh, vh, wh = herm(u), herm(v), herm(w)
    wgt = np.full(u.shape[1], 2.0)
    wgt[0] = 1.0
    mask = np.ones(NZ, bool)
    mask[nz_half] = False

    def mean_prod(a, b):
        return (wgt[None, :, None] * (a * np.conj(b)).real)[mask].sum(axis=(0, 1))

    U, V, W = u[0, 0].real, v[0, 0].real, w[0, 0].real
    return {"U": U, "V": V, "W": W,
            "u_rms": np.sqrt(np.maximum(mean_prod(uh, uh) - U * U, 0)),
            "v_rms": np.sqrt(np.maximum(mean_prod(vh, vh) - V * V, 0)),
            "w_rms": np.sqrt(np.maximum(mean_prod(wh, wh) - W * W, 0)),
            "uv": mean_prod(uh, vh) - U * V}
