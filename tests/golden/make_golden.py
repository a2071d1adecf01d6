"""Generate the golden fixtures in this directory from the reference itself.

Run where the reference sources exist (it needs ``oracle/_ref/libowt_ref.so``,
built by ``make -C oracle ref REF_SRC=<reference>/src``): the reference's own src/solver.cpp,
src/FFT.cpp and src/parallel.cpp, compiled unmodified against the oracle's
MPI/FFTW/LAPACK shims.  The fixtures are small .npz files; the tests compare the
CPU restatement (oracle/owt_port.cpp) and the CUDA path against them.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "open-3d-wallturbulence_gb300"))
from oracle import RefOracle  # noqa: E402
from owt.params import CaseParams  # noqa: E402
from owt.ic import seeded_velocity  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
CURRENT = ["velx", "vely", "velz", "vorx", "vory", "vorz", "lmbx", "lmby", "lmbz", "Hv", "Hg"]
MEANS = ["lmbx_mean_0", "lmbz_mean_0", "velx_mean_0", "velz_mean_0"]
FRIC = ["fx_fric_0", "fx_fric_1", "fx_fric_2", "fz_fric_0", "fz_fric_1", "fz_fric_2"]

CFG0_PHYS = dict(dt=0.005, dkx=0.5, dkz=1.5, alpha_mesh=2.0, nu=1.0 / 2800.0)
CFG1_PHYS = dict(dt=0.002, dkx=1.0, dkz=2.0, alpha_mesh=2.2, nu=1.0e-4)


def snap(r, prefix, fields=CURRENT):
    d = {f"{prefix}/{n}": r.get(n) for n in fields}
    d.update({f"{prefix}/{n}": r.get_cvec(n) for n in MEANS})
    d.update({f"{prefix}/{n}": np.array(r.get_scalar(n)) for n in FRIC})
    return d


def params_arr(p):
    return np.array([p.dt, p.dkx, p.dkz, p.NX, p.NY, p.NZ, p.alpha_mesh, p.nu])


def init(r, p):
    r.init(p.dt, p.dkx, p.dkz, p.NX, p.NY, p.NZ, p.alpha_mesh, p.nu)


def make_ops(r, NY, phys):
    p = CaseParams(NX=8, NZ=8, NY=NY, **phys)
    init(r, p)
    d = {"params": params_arr(p)}
    for q in range(1, 5):
        d[f"DY{q}"] = r.dy(q)
    for n in ("y", "c11", "c21", "c22", "c41", "c42", "c43", "c44"):
        d[n] = r.get_rvec(n)
    d["kx"] = r.get_rvec("kx_local")
    d["kz"] = r.get_rvec("kz_local")
    np.savez_compressed(os.path.join(OUT, f"ops_ny{NY}.npz"), **d)


def make_transform(r):
    p = CaseParams(NX=12, NY=17, NZ=12, **CFG0_PHYS)
    init(r, p)
    rng = np.random.default_rng(7)
    u = rng.standard_normal(p.spectral_shape) + 1j * rng.standard_normal(p.spectral_shape)
    phys = rng.standard_normal((p.NZ2, p.NX2, p.NY))
    np.savez_compressed(os.path.join(OUT, "transform_12x17x12.npz"), params=params_arr(p), spec_in=u,
                        phys_out=r.fourier2physical(u), phys_in=phys, spec_out=r.physical2fourier(phys))


def make_steps(r, name, p, seed, nsteps_list, fields=CURRENT):
    init(r, p)
    u, v, w = seeded_velocity(p, seed=seed)
    r.set_velocity(u, v, w)
    d = {"params": params_arr(p), "seed": np.array(seed), "ic/velx": u, "ic/vely": v, "ic/velz": w}
    d.update(snap(r, "step0", fields))
    done = 0
    for n in nsteps_list:
        r.step(n - done)
        done = n
        d.update(snap(r, f"step{n}", fields))
    np.savez_compressed(os.path.join(OUT, name), **d)


def make_builtin(r):
    p = CaseParams(NX=8, NY=17, NZ=8, dt=0.005, dkx=1.0, dkz=1.0, alpha_mesh=2.0, nu=1.0 / 2800.0)
    init(r, p)
    r.init_fields_builtin()
    d = {"params": params_arr(p), "ic/velx": r.get("velx"), "ic/vely": r.get("vely"), "ic/velz": r.get("velz")}
    d.update(snap(r, "step0"))
    r.step(2)
    d.update(snap(r, "step2"))
    np.savez_compressed(os.path.join(OUT, "builtin_8x17x8.npz"), **d)


def _case(which):
    r = RefOracle()
    if which == "ops17":
        make_ops(r, 17, CFG0_PHYS)
    elif which == "ops33":
        make_ops(r, 33, CFG1_PHYS)
    elif which == "transform":
        make_transform(r)
    elif which == "steps12":
        make_steps(r, "steps_12x17x12.npz", CaseParams(NX=12, NY=17, NZ=12, **CFG0_PHYS), 0, [1, 3])
    elif which == "steps16":
        make_steps(r, "steps_16x33x16.npz", CaseParams(NX=16, NY=33, NZ=16, **CFG1_PHYS), 1, [1],
                   fields=["velx", "vely", "vory", "vorz", "lmby", "Hv", "Hg"])
    elif which == "builtin":
        make_builtin(r)


def main():
    # The reference sizes its pencil-exchange buffers once per process
    # (static thread_local vectors, src/parallel.cpp:18-19), so every grid size
    # gets a fresh process.
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    for which in ("ops17", "ops33", "transform", "steps12", "steps16", "builtin"):
        pr = ctx.Process(target=_case, args=(which,))
        pr.start()
        pr.join()
        if pr.exitcode != 0:
            raise SystemExit(f"case {which} failed ({pr.exitcode})")
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)))


if __name__ == "__main__":
    main()
