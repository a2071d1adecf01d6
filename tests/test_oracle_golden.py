"""The CPU oracle restatement (oracle/owt_port.cpp) against golden fixtures
generated from the reference's own solver (tests/golden/make_golden.py).

These pin the oracle: every later GPU parity test trusts it."""
import numpy as np
import pytest

from conftest import golden

CURRENT = ["velx", "vely", "velz", "vorx", "vory", "vorz", "lmbx", "lmby", "lmbz", "Hv", "Hg"]
MEANS = ["lmbx_mean_0", "lmbz_mean_0", "velx_mean_0", "velz_mean_0"]
FRIC = ["fx_fric_0", "fx_fric_1", "fx_fric_2", "fz_fric_0", "fz_fric_1", "fz_fric_2"]
# The restatement follows the reference operation by operation; on the machine
# that made the fixtures it reproduces them bit for bit.  The tolerance allows
# for a different libm or FMA contraction on another host.
TOL = 1e-11


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def make_port(g):
    from oracle import PortOracle
    dt, dkx, dkz, NX, NY, NZ, al, nu = g["params"]
    o = PortOracle()
    o.init(dt, dkx, dkz, int(NX), int(NY), int(NZ), al, nu)
    return o


def check_snapshot(o, g, prefix, fields):
    for n in fields:
        assert rel(o.get(n), g[f"{prefix}/{n}"]) < TOL, (prefix, n)
    for n in MEANS:
        assert rel(o.get_cvec(n), g[f"{prefix}/{n}"]) < TOL, (prefix, n)
    for n in FRIC:
        assert abs(o.get_scalar(n) - float(g[f"{prefix}/{n}"])) <= TOL * abs(float(g[f"{prefix}/{n}"])), (prefix, n)


@pytest.mark.parametrize("ny", [17, 33])
def test_operators_match_reference(port_lib, ny):
    g = golden(f"ops_ny{ny}.npz")
    o = make_port(g)
    for q in range(1, 5):
        assert rel(o.dy(q), g[f"DY{q}"]) < 1e-12
    for n in ("y", "c11", "c21", "c22", "c41", "c42", "c43", "c44"):
        assert rel(o.get_rvec(n), g[n]) < 1e-14
    np.testing.assert_array_equal(o.get_rvec("kx_local"), g["kx"])
    np.testing.assert_array_equal(o.get_rvec("kz_local"), g["kz"])


def test_d3_top_row_quirk_reproduced(port_lib):
    """The reference's 3rd-derivative top wall row does not annihilate
    constants (src/compdiff.hpp:254-258); the oracle keeps that."""
    g = golden("ops_ny33.npz")
    o = make_port(g)
    # DY4 of a constant: nonzero only in rows that see the faulty D3 row
    dy4 = o.dy(4) @ np.ones(33)
    assert abs(dy4[-1]) > 1.0
    assert rel(o.dy(4), g["DY4"]) < 1e-12


def test_transform_pair_matches_reference(port_lib):
    g = golden("transform_12x17x12.npz")
    o = make_port(g)
    assert rel(o.fourier2physical(g["spec_in"]), g["phys_out"]) < 1e-13
    assert rel(o.physical2fourier(g["phys_in"]), g["spec_out"]) < 1e-13


@pytest.mark.parametrize("name,fields,steps", [
    ("steps_12x17x12.npz", CURRENT, [0, 1, 3]),
    ("steps_16x33x16.npz", ["velx", "vely", "vory", "vorz", "lmby", "Hv", "Hg"], [0, 1]),
])
def test_steps_match_reference(port_lib, name, fields, steps):
    g = golden(name)
    o = make_port(g)
    o.set_velocity(g["ic/velx"], g["ic/vely"], g["ic/velz"])
    done = 0
    for s in steps:
        o.step(s - done)
        done = s
        check_snapshot(o, g, f"step{s}", fields)


def test_builtin_initial_condition_matches_reference(port_lib):
    g = golden("builtin_8x17x8.npz")
    o = make_port(g)
    o.init_fields_builtin()
    for n in ("velx", "vely", "velz"):
        assert rel(o.get(n), g[f"ic/{n}"]) < TOL
    check_snapshot(o, g, "step0", CURRENT)
    o.step(2)
    check_snapshot(o, g, "step2", CURRENT)


def test_reference_build_agrees_with_port_when_present(port_lib):
    """Where the reference itself was built (oracle/_ref), it and the port
    agree bit for bit on a fresh random state."""
    import subprocess
    import sys
    import os
    from oracle import ref_available
    if not ref_available():
        pytest.skip("reference sources not present on this host")
    # separate process: the reference sizes its exchange buffers once per process
    code = r'''
import sys, numpy as np
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[2])
from oracle import RefOracle, PortOracle, FIELD_NAMES
from owt.params import CaseParams
from owt.ic import seeded_velocity
p = CaseParams(dt=0.002, dkx=1.0, dkz=2.0, NX=12, NY=13, NZ=12, alpha_mesh=2.2, nu=1e-4)
u, v, w = seeded_velocity(p, seed=5)
r, o = RefOracle(), PortOracle()
for x in (r, o):
    x.init(p.dt, p.dkx, p.dkz, p.NX, p.NY, p.NZ, p.alpha_mesh, p.nu); x.set_velocity(u, v, w); x.step(2)
bad = [n for n in FIELD_NAMES if not np.array_equal(r.get(n), o.get(n))]
print("MISMATCH" if bad else "SAME", bad)
'''
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, "-c", code, os.path.join(root, "oracle"),
                          os.path.join(root, "open-3d-wallturbulence_gb300")], capture_output=True, text=True)
    assert "SAME" in out.stdout, out.stdout + out.stderr
