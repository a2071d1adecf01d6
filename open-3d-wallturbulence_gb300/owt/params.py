"""Case parameters: the reference's TOML keys and the sizes it derives.

The reference reads a flat TOML file with the keys ``dt, dkx, dkz, NX, NY, NZ,
alpha_mesh, NT, PX, PZ, save_interval, nu`` (src/IO.cpp:14-25) and derives
``NXH = NX/2``, ``NZH = NZ/2``, ``NX2 = NX/2*3``, ``NZ2 = NZ/2*3``
(src/IO.cpp:27-30).  The case files are ``key = value # comment`` lines, so a
small parser is enough; unknown keys (e.g. ``initial_condition``) are kept but
ignored, as the reference ignores them.
"""
from dataclasses import dataclass, field, asdict

REQUIRED = ("dt", "dkx", "dkz", "NX", "NY", "NZ", "alpha_mesh", "NT", "PX", "PZ", "save_interval", "nu")
INT_KEYS = ("NX", "NY", "NZ", "NT", "PX", "PZ", "save_interval")


@dataclass
class CaseParams:
    dt: float
    dkx: float
    dkz: float
    NX: int
    NY: int
    NZ: int
    alpha_mesh: float
    nu: float
    NT: int = 0
    PX: int = 1
    PZ: int = 1
    save_interval: int = 1
    extra: dict = field(default_factory=dict)
    # interior compact-FD order: 8 = the reference's schemes, 6 = sixth-order
    # tridiagonal interior schemes (not a reference toml key)
    fd_order: int = 8

    @property
    def NXH(self):
        return self.NX // 2

    @property
    def NZH(self):
        return self.NZ // 2

    @property
    def NX2(self):
        return self.NX // 2 * 3

    @property
    def NZ2(self):
        return self.NZ // 2 * 3

    @property
    def spectral_shape(self):
        """Reference Field layout of a spectral field: [z][x][y]."""
        return (self.NZ, self.NXH, self.NY)

    def validate(self):
        if self.NX < 2 or self.NZ < 2 or self.NX % 2 or self.NZ % 2:
            raise ValueError("NX and NZ must be even and >= 2")
        if self.NY < 7:
            raise ValueError("N must be at least 7 for 3rd derivative scheme")
        if self.dt <= 0 or self.nu <= 0:
            raise ValueError("dt and nu must be positive")
        return self

    def as_dict(self):
        return asdict(self)


def _value(tok):
    t = tok.strip()
    if t.startswith('"') and t.endswith('"'):
        return t[1:-1]
    try:
        if any(c in t for c in ".eE") and not t.lower().startswith("0x"):
            return float(t)
        return int(t)
    except ValueError:
        return t


def parse_toml_text(text):
    """Parse the flat ``key = value # comment`` case format."""
    out = {}
    for ln, raw in enumerate(text.splitlines(), 1):
        line = raw.split("#", 1)[0].strip()
        if not line:
            continue
        if line.startswith("["):
            continue
        if "=" not in line:
            raise ValueError(f"line {ln}: expected 'key = value'")
        k, v = line.split("=", 1)
        out[k.strip()] = _value(v)
    return out


def load_params(path_or_text):
    """Read a case file like the reference's ``load_params`` (src/IO.cpp:8-74).

    Unlike the reference, a missing key raises instead of being printed and
    swallowed (src/IO.cpp:36-39), since continuing with unset sizes is never
    what a caller wants.
    """
    if "\n" in path_or_text or "=" in path_or_text:
        d = parse_toml_text(path_or_text)
    else:
        with open(path_or_text) as f:
            d = parse_toml_text(f.read())
    missing = [k for k in REQUIRED if k not in d]
    if missing:
        raise KeyError("missing keys: " + ", ".join(missing))
    kw = {k: (int(d[k]) if k in INT_KEYS else float(d[k])) for k in REQUIRED}
    extra = {k: v for k, v in d.items() if k not in REQUIRED}
    return CaseParams(extra=extra, **kw).validate()


# Workloads used by the tests and the benchmark (sizes and physics of each case).
def channel_180(**kw):
    """Re_tau=180 channel: 128x129x128 modes, Lx=4pi, Lz=4pi/3, tanh factor 2.0, dt=0.005, Re_b=5600."""
    d = dict(dt=0.005, dkx=0.5, dkz=1.5, NX=128, NY=129, NZ=128, alpha_mesh=2.0, nu=1.0 / 2800.0)
    d.update(kw)
    return CaseParams(**d).validate()


def channel_550(**kw):
    """Re_tau=550 channel: 384x257x384 modes, Lx=2pi, Lz=pi, tanh factor 2.2, dt=0.002, nu=1e-4."""
    d = dict(dt=0.002, dkx=1.0, dkz=2.0, NX=384, NY=257, NZ=384, alpha_mesh=2.2, nu=1.0e-4)
    d.update(kw)
    return CaseParams(**d).validate()
