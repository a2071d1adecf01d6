"""Test infrastructure (oracle): the reference time step restated in PyTorch
float64 on the CPU, for an FP64 reference gradient by automatic
differentiation.

Only tests use this module.  It restates, with torch operations that autograd
can differentiate, the same algorithm as ``owt_port.cpp`` (and the reference):

  source assembly, dense Av / Ag with boundary rows ... src/solver.cpp:561-603
  (wall rows 0 and NY-1 of source_v carry the wall velocity, :593-596)
  solve_horizontal ................................... src/solver.cpp:516-539
  solve_mean + solve_friction_force .................. src/solver.cpp:306-327, 428-514
  Lamb_vec with the dealiased transforms ............. src/solver.cpp:262-304, src/FFT.cpp:49-194
  nonlinear_source ................................... src/solver.cpp:240-260
  history rotation ................................... src/solver.cpp:612-626

The dense DYn matrices, wavenumbers and grid come from the CPU port, so the
two share their discretisation exactly; the solves use explicit inverses of
the per-mode matrices (a different rounding than LU, not a different map).
The objective is the wall-drag functional of the GPU library:
J = (1/N) sum over N steps of the driving force fx of each step.
"""
import numpy as np
import torch

A0, A1, A2 = 3.0, -1.5, 1.0 / 3.0
B0, B1, B2 = 3.0, -3.0, 1.0
G0 = 11.0 / 6.0

FIELD_KEYS = [("v", "vely"), ("g", "vory"), ("hv", "Hv"), ("hg", "Hg")]
MEAN_KEYS = [("U", "velx_mean"), ("W", "velz_mean"), ("Lx", "lmbx_mean"), ("Lz", "lmbz_mean")]


class TorchChannel:
    """One channel's step as a differentiable function of (state, wall velocity)."""

    def __init__(self, port, dt, nu):
        self.NX, self.NY, self.NZ = port.NX, port.NY, port.NZ
        self.NXH, self.NZH = self.NX // 2, self.NZ // 2
        self.NX2, self.NZ2 = self.NX // 2 * 3, self.NZ // 2 * 3
        self.dt, self.nu = float(dt), float(nu)
        N = self.NY
        self.DY = [torch.tensor(port.dy(w), dtype=torch.float64) for w in (1, 2, 3, 4)]
        kx = torch.tensor(port.get_rvec("kx_local"), dtype=torch.float64)
        kz = torch.tensor(port.get_rvec("kz_local"), dtype=torch.float64)
        y = port.get_rvec("y")
        self.Ly = float(y[-1] - y[0])
        self.kx = kx[None, :, None]
        self.kz = kz[:, None, None]
        k2 = kx[None, :] ** 2 + kz[:, None] ** 2
        self.k2 = k2[..., None]
        self.ik2 = torch.where(k2 < 1e-8, torch.zeros_like(k2), 1.0 / torch.where(k2 < 1e-8, torch.ones_like(k2), k2))[..., None]
        self.mean_mask = (k2 < 1e-8)[..., None]
        eye = torch.eye(N, dtype=torch.float64)
        D1, D2, D4 = self.DY[0], self.DY[1], self.DY[3]
        dt_, nu_ = self.dt, self.nu
        k2b = k2[..., None, None]
        Av = -nu_ * D4 + (G0 / dt_ + 2 * nu_ * k2b) * D2 - (nu_ * k2b ** 2 + G0 * k2b / dt_) * eye
        Ag = -nu_ * D2 + (nu_ * k2b + G0 / dt_) * eye
        Av[..., 0, :] = 0.0
        Av[..., 0, 0] = 1.0
        Av[..., 1, :] = D1[0]
        Av[..., N - 2, :] = D1[N - 1]
        Av[..., N - 1, :] = 0.0
        Av[..., N - 1, N - 1] = 1.0
        Ag[..., 0, :] = 0.0
        Ag[..., 0, 0] = 1.0
        Ag[..., N - 1, :] = 0.0
        Ag[..., N - 1, N - 1] = 1.0
        Am = -nu_ * D2 + G0 / dt_ * eye
        Am[0, :] = 0.0
        Am[0, 0] = 1.0
        Am[N - 1, :] = 0.0
        Am[N - 1, N - 1] = 1.0
        self.Av_inv = torch.linalg.inv(Av).to(torch.complex128)
        self.Ag_inv = torch.linalg.inv(Ag).to(torch.complex128)
        self.Am_inv = torch.linalg.inv(Am).to(torch.complex128)
        self.D1c, self.D2c = D1.to(torch.complex128), D2.to(torch.complex128)

    # -- state ------------------------------------------------------------------
    @staticmethod
    def state_from(get, get_cvec, friction):
        """State dict from accessors with the reference names (port or GPU solver)."""
        st = {}
        for k, name in FIELD_KEYS:
            for l in range(3):
                st[f"{k}{l}"] = torch.tensor(get(f"{name}_{l}"))
        for k, name in MEAN_KEYS:
            for l in range(3):
                st[f"{k}{l}"] = torch.tensor(get_cvec(f"{name}_{l}"))
        fr = friction()
        for l in range(3):
            st[f"fx{l}"] = torch.tensor(float(fr[l]), dtype=torch.float64)
            st[f"fz{l}"] = torch.tensor(float(fr[3 + l]), dtype=torch.float64)
        return st

    # -- transforms (src/FFT.cpp:49-194) ----------------------------------------
    def to_phys(self, f):
        NZH, NZ, NZ2, NXH, NX2 = self.NZH, self.NZ, self.NZ2, self.NXH, self.NX2
        z = torch.zeros((1,) + tuple(f.shape[1:]), dtype=f.dtype)
        P = torch.cat([f[:NZH]] + [z] * (NZ2 - NZ + 1) + [f[NZH + 1:]], dim=0)  # Nyquist row dropped
        Pz = torch.fft.ifft(P, dim=0, norm="forward")
        zx = torch.zeros((NZ2, NX2 - 2 * NXH + 1, f.shape[2]), dtype=f.dtype)
        X = torch.cat([Pz, zx, torch.conj(torch.flip(Pz[:, 1:NXH], dims=[1]))], dim=1)
        return torch.fft.ifft(X, dim=1, norm="forward").real

    def to_spec(self, p):
        NZH, NZ, NZ2, NXH, NX2 = self.NZH, self.NZ, self.NZ2, self.NXH, self.NX2
        X = torch.fft.fft(p.to(torch.complex128), dim=1)[:, :NXH] / NX2
        Z = torch.fft.fft(X, dim=0)
        return torch.cat([Z[:NZH], Z[NZ:NZ2]], dim=0) / NZ2

    def dy(self, D, f):
        return f @ D.T

    # -- one step ------------------------------------------------------------------
    def step(self, st, vw_bottom, vw_top):
        dt, nu, N = self.dt, self.nu, self.NY
        vs = A0 * st["v0"] + A1 * st["v1"] + A2 * st["v2"]
        sv = B0 * st["hv0"] + B1 * st["hv1"] + B2 * st["hv2"] - (self.k2 / dt) * vs + self.dy(self.D2c, vs) / dt
        zc = torch.zeros_like(sv[..., :1])
        sv = torch.cat([vw_bottom[..., None], zc, sv[..., 2:N - 2], zc, vw_top[..., None]], dim=-1)
        sg = B0 * st["hg0"] + B1 * st["hg1"] + B2 * st["hg2"] + (A0 * st["g0"] + A1 * st["g1"] + A2 * st["g2"]) / dt
        sg = torch.cat([zc, sg[..., 1:N - 1], zc], dim=-1)
        v = (self.Av_inv @ sv[..., None])[..., 0]
        g = (self.Ag_inv @ sg[..., None])[..., 0]
        # solve_horizontal
        kx, kz, k2, ik2 = self.kx, self.kz, self.k2, self.ik2
        d1v, d2v, d1g = self.dy(self.D1c, v), self.dy(self.D2c, v), self.dy(self.D1c, g)
        u = 1j * kx * ik2 * d1v - 1j * kz * ik2 * g
        w = 1j * kx * ik2 * g + 1j * kz * ik2 * d1v
        ox = 1j * ik2 * (kx * d1g + kz * d2v - kz * k2 * v)
        oz = 1j * ik2 * (kz * d1g - kx * d2v + kx * k2 * v)
        # solve_mean + solve_friction_force
        su = B0 * (st["Lx0"] + st["fx0"]) + B1 * (st["Lx1"] + st["fx1"]) + B2 * (st["Lx2"] + st["fx2"]) + \
            (A0 * st["U0"] + A1 * st["U1"] + A2 * st["U2"]) / dt
        sw = B0 * (st["Lz0"] + st["fz0"]) + B1 * (st["Lz1"] + st["fz1"]) + B2 * (st["Lz2"] + st["fz2"]) + \
            (A0 * st["W0"] + A1 * st["W1"] + A2 * st["W2"]) / dt
        z1 = torch.zeros(1, dtype=torch.complex128)
        su = torch.cat([z1, su[1:N - 1], z1])
        sw = torch.cat([z1, sw[1:N - 1], z1])
        U = self.Am_inv @ su
        W = self.Am_inv @ sw
        dU, dW = self.D1c @ U, self.D1c @ W
        fx = -nu / self.Ly * (dU[N - 1].real - dU[0].real)
        fz = -nu / self.Ly * (dW[N - 1].real - dW[0].real)
        m0 = self.mean_mask
        u = torch.where(m0, U[None, None, :], u)
        w = torch.where(m0, W[None, None, :], w)
        ox = torch.where(m0, dW[None, None, :], ox)
        oz = torch.where(m0, -dU[None, None, :], oz)
        # Lamb_vec
        up, vp, wp = self.to_phys(u), self.to_phys(v), self.to_phys(w)
        oxp, oyp, ozp = self.to_phys(ox), self.to_phys(g), self.to_phys(oz)
        lx = self.to_spec(vp * ozp - wp * oyp)
        ly = self.to_spec(wp * oxp - up * ozp)
        lz = self.to_spec(up * oyp - vp * oxp)
        # nonlinear_source
        hv = -k2 * ly - self.dy(self.D1c, 1j * kx * lx + 1j * kz * lz)
        hg = 1j * kz * lx - 1j * kx * lz
        new = {
            "v0": v, "v1": st["v0"], "v2": st["v1"], "g0": g, "g1": st["g0"], "g2": st["g1"],
            "hv0": hv, "hv1": st["hv0"], "hv2": st["hv1"], "hg0": hg, "hg1": st["hg0"], "hg2": st["hg1"],
            "U0": U, "U1": st["U0"], "U2": st["U1"], "W0": W, "W1": st["W0"], "W2": st["W1"],
            "Lx0": lx[0, 0], "Lx1": st["Lx0"], "Lx2": st["Lx1"], "Lz0": lz[0, 0], "Lz1": st["Lz0"],
            "Lz2": st["Lz1"], "fx0": fx, "fx1": st["fx0"], "fx2": st["fx1"], "fz0": fz, "fz1": st["fz0"],
            "fz2": st["fz1"],
        }
        return new, fx

    def drag(self, st, vw_bottom, vw_top, nsteps):
        """J = mean of fx over nsteps steps, and the final state."""
        J = torch.zeros((), dtype=torch.float64)
        for _ in range(nsteps):
            st, fx = self.step(st, vw_bottom, vw_top)
            J = J + fx
        return J / nsteps, st
