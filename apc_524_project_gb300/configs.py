"""Run configurations: the reference's Input_Info_t plus the seeded loader.

Physical inputs are given in normalised units (c = 1, dx = 1, electron charge
-1 and mass 1). The reference code works in its own unit system and applies
UNIT_ACC in the push and UNIT_RHOJ in the deposit (src/globals.hpp:12,16), so
each species of macro-particle weight w is handed to it as

    charge_ratio = w q / UNIT_RHOJ,   mass_ratio = UNIT_ACC w m / UNIT_RHOJ,

which gives UNIT_ACC * charge/mass = q/m in the push and UNIT_RHOJ * charge =
w q in the deposit: the normalised equations, unchanged reference code. The
weight w is chosen from the electron plasma frequency,
omega_pe^2 = 4 pi (ppc_e / dx^3) w q^2 / m.

The named workloads follow the benchmark configurations of the project:
  langmuir32   32^3 Langmuir oscillation, FP64, Poisson start, 100 steps
  thermal256   256^3 thermal plasma, 2 x 16 ppc, relativistic, sort every 20
  twostream    256 x 128^2 counter-streaming beams, immobile ions
  laser64      64^3 x-injected plane wave, reflecting x, 8 ppc x 2
  laser512     512 x 128^2 laser-plasma, absorbing x
"""
import ctypes as C
import math
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

from . import abi

UNIT_ACC = 0.58668774
UNIT_RHOJ = 4.80320427e-13
PI = 3.14159265358979323846


@dataclass
class Species:
    name: str
    q: float
    m: float
    ppc: float
    vth: float
    drift: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    test: int = 0
    dens_amp: float = 0.0
    dens_k: float = 1.0
    x_range: Optional[Tuple[float, float]] = None  # load only in x0 <= x < x1


@dataclass
class Shape:
    """Transverse Gaussian spot and sine-series envelope of an injected wave
    (emoo_set_wave_shape; no reference counterpart)."""
    waist: float = 0.0                                # 0: plane wave
    center: Optional[Tuple[float, float]] = None      # None: middle of the transverse extent
    t_start: float = 0.0
    window: float = 0.0
    coef: Tuple[float, ...] = ()                      # sine-series coefficients (empty: Gaussian envelope)


@dataclass
class Wave:
    side: int   # -1 x left, +1 x right, ...
    pol: int    # E polarisation 1,2,3
    amp: float
    omega: float
    phase_deg: float = 0.0
    inv_width: float = 0.0
    delay: float = 0.0
    shape: Optional[Shape] = None


@dataclass
class Config:
    name: str
    n: Tuple[int, int, int]
    dx: Tuple[float, float, float] = (1.0, 1.0, 1.0)
    dt: float = 0.5
    steps: int = 100
    species: List[Species] = field(default_factory=list)
    omega_pe: float = 0.5
    weight: Optional[float] = None
    relativity: int = 0
    electrostatic: int = 0
    part_bc: Tuple[str, ...] = ("periodic",) * 6
    field_bc: Tuple[str, ...] = ("periodic",) * 6
    init: str = "poisson"
    E0: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    B0: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    nstep_sort: int = 0
    waves: List[Wave] = field(default_factory=list)
    bound_phi: Tuple[float, ...] = (0.0,) * 6
    bound_A: Tuple[Tuple[float, ...], ...] = ((0.0,) * 6, (0.0,) * 6, (0.0,) * 6)
    seed: int = 12345
    zero_mean: Optional[bool] = None  # default: Poisson start with all-periodic fields
    x0: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    immobile_ions: bool = False  # uniform neutralising background instead of ion particles
    b_noise: float = 0.0         # seeded white-noise amplitude on every B component (two-stream start)

    @property
    def L(self):
        return tuple(self.n[i] * self.dx[i] for i in range(3))

    def macro_weight(self):
        if self.weight is not None:
            return self.weight
        e = self.species[0]
        vol = self.dx[0] * self.dx[1] * self.dx[2]
        return self.omega_pe ** 2 * e.m / (4.0 * PI * (e.ppc / vol) * e.q ** 2)

    def count(self, s: Species) -> int:
        cells = self.n[0] * self.n[1] * self.n[2]
        if s.x_range is not None:
            frac = (s.x_range[1] - s.x_range[0]) / self.L[0]
            cells = int(round(cells * frac))
        return int(round(cells * s.ppc))

    def total_particles(self) -> int:
        return sum(self.count(s) for s in self.species)

    def want_zero_mean(self):
        if self.zero_mean is not None:
            return self.zero_mean
        return self.init == "poisson" and all(b == "periodic" for b in self.field_bc)


def _setstr(arr, s):
    """Copies a NUL-terminated string into a ctypes char-array (an element of
    a 2-D char array; plain struct members are assigned directly)."""
    b = s.encode()
    if len(b) >= abi.NCHAR:
        raise ValueError(f"string too long for a {abi.NCHAR}-char field: {s!r}")
    C.memmove(arr, b + b"\0", len(b) + 1)


def input_info(cfg: Config) -> abi.InputInfo:
    """Input_Info_t as the reference parser + ProcessInfo would leave it."""
    info = abi.InputInfo()
    w = cfg.macro_weight()
    for d in range(3):
        info.nCell[d] = cfg.n[d]
        info.nProc[d] = 1
        info.xyz0[d] = cfg.x0[d]
        info.Lxyz[d] = cfg.L[d]
        info.E0[d] = cfg.E0[d]
        info.B0[d] = cfg.B0[d]
    info.nt = cfg.steps
    info.restart = 0
    info.relativity = cfg.relativity
    info.electrostatic = cfg.electrostatic
    info.nspecies = len(cfg.species)
    info.nstep_fields = 10
    info.nstep_parts = 10
    info.nstep_restart = 100
    info.nstep_sort = cfg.nstep_sort
    info.which_fields = -1
    for i, s in enumerate(cfg.species):
        info.charge_ratio[i] = w * s.q / UNIT_RHOJ
        info.mass_ratio[i] = UNIT_ACC * w * s.m / UNIT_RHOJ
        info.isTestParticle[i] = s.test
        info.dens_frac[i] = cfg.count(s) / max(1, cfg.total_particles())
        info.temp[i] = 0.0
    info.nparticles_tot = cfg.total_particles()
    info.nparticles_domain = cfg.total_particles()
    info.t0 = 0.0
    info.dens_phys = 0.0
    info.super_ratio = 1.0
    info.fields_init = cfg.init.encode()
    info.parts_init = b"random"
    for s in range(6):
        _setstr(info.parts_bound[s], cfg.part_bc[s])
        _setstr(info.fields_bound[s], cfg.field_bc[s])
        info.bound_phi[s] = cfg.bound_phi[s]
        info.bound_Ax[s] = cfg.bound_A[0][s]
        info.bound_Ay[s] = cfg.bound_A[1][s]
        info.bound_Az[s] = cfg.bound_A[2][s]
    info.nwaves = len(cfg.waves)
    for i, wv in enumerate(cfg.waves):
        info.inSide[i] = wv.side
        info.inPolE[i] = wv.pol
        info.peakamps[i] = wv.amp
        info.omegas[i] = wv.omega
        info.phases[i] = wv.phase_deg
        info.invWidths[i] = wv.inv_width
        info.delays[i] = wv.delay
    return info


def rho_background(cfg: Config) -> float:
    """Uniform immobile background (reference rho units) that neutralises the
    deposited species where they are loaded: each macro-particle deposits
    UNIT_RHOJ * charge_ratio / V = w q / V in total, so the background is
    -sum_s w q_s ppc_s / V. Zero unless cfg.immobile_ions."""
    if not cfg.immobile_ions:
        return 0.0
    w = cfg.macro_weight()
    vol = cfg.dx[0] * cfg.dx[1] * cfg.dx[2]
    return -sum(w * s.q * s.ppc for s in cfg.species if not s.test) / vol


def rho_background_xmin(cfg: Config) -> Optional[float]:
    """Where the background starts: the lowest x the deposited species are
    loaded from, when every one of them is loaded in an x range (None: the
    whole box)."""
    sp = [s for s in cfg.species if not s.test]
    if not cfg.immobile_ions or not sp or any(s.x_range is None for s in sp):
        return None
    return cfg.x0[0] + min(s.x_range[0] for s in sp)


def wave_shape(cfg: Config, w: int, coef=None) -> Optional[abi.WaveShape]:
    """emoo_wave_shape of wave w (None when it has no shape); coef, when
    given, replaces the shape's envelope coefficients."""
    sh = cfg.waves[w].shape
    if sh is None:
        return None
    out = abi.WaveShape()
    out.waist = sh.waist
    d = abs(cfg.waves[w].side) - 1
    axes = [a for a in range(3) if a != d]
    center = sh.center if sh.center is not None else tuple(cfg.x0[a] + 0.5 * cfg.L[a] for a in axes)
    out.center[0], out.center[1] = center
    out.t_start = sh.t_start
    out.window = sh.window
    c = list(sh.coef if coef is None else coef)
    if len(c) > abi.NCOEF:
        raise ValueError(f"at most {abi.NCOEF} envelope coefficients")
    out.ncoef = len(c)
    for k, v in enumerate(c):
        out.coef[k] = v
    return out


def apply_wave_shapes(backend, cfg: Config, coefs=None):
    """Hands every shaped wave's shape to a backend (set_wave_shape(w, shape));
    coefs[w], when given, replaces wave w's envelope coefficients."""
    for w, wv in enumerate(cfg.waves):
        if wv.shape is not None:
            backend.set_wave_shape(w, wave_shape(cfg, w, None if coefs is None else coefs[w]))


def gaussian_sine_coefficients(window: float, fwhm: float, ncoef: int = 16):
    """Sine-series coefficients c_k (k = 1..ncoef) of a unit-peak Gaussian
    of the given FWHM centred in [0, window]: with a = 4 ln 2 / fwhm^2 and the
    tails beyond the window neglected,
    c_k = (2 / window) sin(k pi / 2) sqrt(pi / a) exp(-(k pi / window)^2 / (4 a))."""
    a = 4.0 * math.log(2.0) / fwhm ** 2
    return [(2.0 / window) * math.sin(k * PI / 2.0) * math.sqrt(PI / a)
            * math.exp(-(k * PI / window) ** 2 / (4.0 * a)) for k in range(1, ncoef + 1)]


def b_noise_fields(cfg: Config):
    """Seeded white noise of amplitude cfg.b_noise on Bx, By, Bz at the
    physical points ((n+3)^3 arrays, ghosts zero), the same values for B and
    B_tm1 (the two-stream workload's start). Returns None when cfg.b_noise is 0."""
    if not cfg.b_noise:
        return None
    import numpy as np

    rng = np.random.default_rng(cfg.seed ^ 0x5EED0B)
    shape = tuple(v + 3 for v in cfg.n)
    out = []
    for _ in range(3):
        f = np.zeros(shape)
        f[1:cfg.n[0] + 1, 1:cfg.n[1] + 1, 1:cfg.n[2] + 1] = cfg.b_noise * rng.uniform(-1.0, 1.0, cfg.n)
        out.append(f)
    return out


def gen_params(cfg: Config, si: int) -> abi.GenParams:
    s = cfg.species[si]
    g = abi.GenParams()
    g.seed = cfg.seed
    g.species = si
    g.relativistic_gamma = 1 if cfg.relativity else 0
    L = cfg.L
    for d in range(3):
        g.x0[d] = cfg.x0[d]
        g.L[d] = L[d]
        g.vth[d] = s.vth
        g.vdrift[d] = s.drift[d]
    if s.x_range is not None:
        g.x0[0] = cfg.x0[0] + s.x_range[0]
        g.L[0] = s.x_range[1] - s.x_range[0]
    g.dens_amp = s.dens_amp
    g.dens_k = s.dens_k
    return g


# ---------------------------------------------------------------- workloads

def langmuir32():
    """32^3 Langmuir oscillation: FP64, Poisson start, non-relativistic Boris."""
    return Config(
        name="langmuir32", n=(32, 32, 32), dt=0.5, steps=100, omega_pe=0.5,
        species=[Species("e", -1.0, 1.0, 8, 0.05, dens_amp=0.1, dens_k=1.0),
                 Species("i", 1.0, 1836.0, 8, 0.05 / math.sqrt(1836.0))],
        init="poisson", nstep_sort=0, seed=20240101)


def thermal256(n=256):
    """Thermal plasma at scale: 2 x 16 ppc, relativistic push, sort every 20."""
    return Config(
        name=f"thermal{n}", n=(n, n, n), dt=0.5, steps=200, omega_pe=0.5,
        species=[Species("e", -1.0, 1.0, 16, 0.1),
                 Species("i", 1.0, 1836.0, 16, 0.1 / math.sqrt(1836.0))],
        relativity=1, init="constant", nstep_sort=20, seed=20240202)


def twostream(n=(256, 128, 128), steps=1000):
    """Counter-streaming electron beams (drift +-0.3c along x, 16 ppc each,
    v_th = 0.02c) over an immobile neutralising background, relativistic push,
    seeded 1e-4 white noise on B, periodic, sort every 20 steps."""
    return Config(
        name="twostream", n=tuple(n), dt=0.45, steps=steps, omega_pe=0.5,
        species=[Species("beam+", -1.0, 1.0, 16, 0.02, drift=(0.3, 0.0, 0.0)),
                 Species("beam-", -1.0, 1.0, 16, 0.02, drift=(-0.3, 0.0, 0.0))],
        relativity=1, init="constant", nstep_sort=20, seed=20240303, immobile_ions=True, b_noise=1e-4)


def laser64(n=(64, 64, 64), steps=128, ppc=8, a0=0.5, wavelength=16.0, fwhm_steps=40):
    """Differentiation workload: a y-polarised plane wave injected at x-left
    (amplitude a0 omega, omega = 2 pi / wavelength, Gaussian envelope of the
    given FWHM in steps, peak after two FWHM), reflecting particle walls in
    x, periodic y and z, electrons and ions at ppc each (electron v_th =
    0.05c), fields starting at zero. Objective slab x in [48, 56) of 64."""
    dt = 0.5
    omega = 2.0 * PI / wavelength
    fwhm_t = fwhm_steps * dt
    wave = Wave(side=-1, pol=2, amp=a0 * omega, omega=omega, phase_deg=0.0,
                inv_width=math.sqrt(math.log(2.0)) / (0.5 * fwhm_t), delay=2.0 * fwhm_t)
    return Config(
        name="laser64", n=tuple(n), dt=dt, steps=steps, omega_pe=0.3,
        species=[Species("e", -1.0, 1.0, ppc, 0.05), Species("i", 1.0, 1836.0, ppc, 0.05 / math.sqrt(1836.0))],
        relativity=1, init="constant",
        part_bc=("reflecting", "reflecting", "periodic", "periodic", "periodic", "periodic"),
        field_bc=("external", "external", "periodic", "periodic", "periodic", "periodic"),
        waves=[wave], seed=20240505)


def laser512(n=(512, 128, 128), steps=512, ppc=16, a0=1.0, wavelength=20.0, fwhm_steps=60, waist=30.0,
             plasma_x0=64.0, density=0.01, vth=0.01, coef_sigma=0.1, seed=20240606):
    """Laser-plasma at scale: a y-polarised pulse injected at x-left
    (amplitude a0 omega, omega = 2 pi / wavelength) with a transverse Gaussian
    spot of the given waist (1/e field radius) and an envelope of 16
    sine-series coefficients over a window of four FWHM: the coefficients of
    a unit-peak Gaussian of FWHM fwhm_steps dt centred in the window, each
    plus seeded N(0, coef_sigma) noise. External fields and absorbing
    particle walls in x, periodic y and z; electrons at `density` of the
    critical density (omega_pe = sqrt(density) omega) and ppc per cell from
    x = plasma_x0 on, over immobile ions there; relativistic push; sorted by
    cell every 20 steps. The electron temperature is not part of the
    workload's definition; vth sets a cold plasma."""
    import numpy as np

    dt = 0.45
    omega = 2.0 * PI / wavelength
    fwhm_t = fwhm_steps * dt
    window = 4.0 * fwhm_t
    coef = gaussian_sine_coefficients(window, fwhm_t, 16)
    rng = np.random.default_rng(seed)
    coef = [c + coef_sigma * float(z) for c, z in zip(coef, rng.standard_normal(16))]
    shape = Shape(waist=waist, t_start=0.0, window=window, coef=tuple(coef))
    wave = Wave(side=-1, pol=2, amp=a0 * omega, omega=omega, phase_deg=0.0, shape=shape)
    return Config(
        name="laser512", n=tuple(n), dt=dt, steps=steps, omega_pe=math.sqrt(density) * omega,
        species=[Species("e", -1.0, 1.0, ppc, vth, x_range=(plasma_x0, n[0] * 1.0))],
        relativity=1, init="constant",
        part_bc=("absorbing", "absorbing", "periodic", "periodic", "periodic", "periodic"),
        field_bc=("external", "external", "periodic", "periodic", "periodic", "periodic"),
        waves=[wave], seed=seed, immobile_ions=True, nstep_sort=20)


def tiny(name="tiny", n=(6, 5, 4), dx=(1.0, 1.0, 1.0), ppc=3, relativity=0, init="poisson", steps=4,
         part_bc=("periodic",) * 6, field_bc=("periodic",) * 6, waves=(), B0=(0.0, 0.0, 0.0), E0=(0.0, 0.0, 0.0),
         vth=0.08, nstep_sort=0, seed=7, dt=0.45, test_species=False):
    sp = [Species("e", -1.0, 1.0, ppc, vth, dens_amp=0.2, dens_k=1.0),
          Species("i", 1.0, 40.0, ppc, vth / 4)]
    if test_species:
        sp.append(Species("t", -1.0, 1.0, 1, vth, test=1))
    return Config(name=name, n=n, dx=dx, dt=dt, steps=steps, omega_pe=0.6, species=sp, relativity=relativity,
                  init=init, part_bc=part_bc, field_bc=field_bc, waves=list(waves), B0=B0, E0=E0,
                  nstep_sort=nstep_sort, seed=seed)
