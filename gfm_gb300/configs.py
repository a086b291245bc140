"""Synthetic furnace cases (stand-ins for the reference's gd/sbc input files).

The cases follow the benchmark definitions: a rectangular combustion space
4.0 x 2.0 x 1.2 m, one CH4 burner and two air ports on the x=0 wall, a flue on
the x=4 m wall, walls held at 1700 K through the convective wall sink, 4 gray
radiation bands.  Sizes: 48x24x16 cells (case "small") and 192x96x64 cells
(1,179,648 cells, case "large").  Nothing here reproduces an evaluation item;
the openings' positions are this project's choice.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

from .abi import GFM_ADI_MARCH, GFM_PREC_FP64, GfmCaseSpec, GfmInletSpec

# Sweep counts per NELG 1..12 from the shipped relaxation file
# (combustion/relaxfactorc.txt:30-43): u v w p p' fuel co2 h k eps n2 o2
REFERENCE_SWEEPS = (2, 2, 2, 6, 5, 3, 3, 8, 2, 2, 3, 3)

AIR_O2 = 0.2329175       # air composition used by the shipped case0041 inlet
AIR_N2 = 0.7670825


@dataclass
class Inlet:
    y0: float
    y1: float
    z0: float
    z1: float
    t_k: float
    u_ms: float
    yf: float = 0.0
    yo2: float = 0.0
    yn2: float = 0.0
    yco2: float = 0.0
    yh2o: float = 0.0


@dataclass
class FurnaceCase:
    name: str
    nx: int
    ny: int
    nz: int
    lx: float = 4.0
    ly: float = 2.0
    lz: float = 1.2
    inlets: list = field(default_factory=list)
    exit_yz: tuple = (0.8, 1.2, 0.3, 0.9)
    t_init_k: float = 1500.0
    noise_amp: float = 0.01
    seed: int = 20261203
    inlet_jitter: float = 0.0
    t_wall_k: float = 1700.0
    rf_uvw: float = 0.5
    rfl_h: float = 0.7
    rfl_k: float = 0.7
    rfl_eps: float = 0.7
    rfl_species: float = 0.6
    rf_hsource: float = 0.3
    ntimesg: tuple = REFERENCE_SWEEPS
    sigma_k: float = 1.0
    sigma_eps: float = 1.3
    kappa: tuple = (0.1, 0.5, 1.0, 2.0)
    wl_um: tuple = (2.0, 4.0, 8.0, 1000.0)
    pg0: float = 1.01325e5
    q0_jkg: float = 5.0e7
    h_g: float = 10.0
    react: int = 1
    wall_sink: int = 1
    rad_emission: int = 1
    maxgi: int = 2000
    bgcon: float = 1.0e-5
    adi_mode: int = GFM_ADI_MARCH
    precision: int = GFM_PREC_FP64

    @property
    def ncells_box(self) -> int:
        return self.nx * self.ny * self.nz

    def to_spec(self) -> GfmCaseSpec:
        s = GfmCaseSpec()
        s.nx, s.ny, s.nz = self.nx, self.ny, self.nz
        s.lx, s.ly, s.lz = self.lx, self.ly, self.lz
        s.n_inlets = len(self.inlets)
        for i, inl in enumerate(self.inlets):
            s.inlets[i] = GfmInletSpec(inl.y0, inl.y1, inl.z0, inl.z1, inl.t_k,
                                       inl.yf, inl.yo2, inl.yn2, inl.yco2, inl.yh2o, inl.u_ms)
        s.exit_y0, s.exit_y1, s.exit_z0, s.exit_z1 = self.exit_yz
        s.t_init_k, s.noise_amp, s.seed = self.t_init_k, self.noise_amp, self.seed
        s.inlet_jitter, s.t_wall_k = self.inlet_jitter, self.t_wall_k
        s.rf_uvw, s.rfl_h, s.rfl_k, s.rfl_eps = self.rf_uvw, self.rfl_h, self.rfl_k, self.rfl_eps
        s.rfl_species, s.rf_hsource = self.rfl_species, self.rf_hsource
        for i, n in enumerate(self.ntimesg):
            s.ntimesg[i] = n
        s.sigma_k, s.sigma_eps = self.sigma_k, self.sigma_eps
        s.nwl = len(self.kappa)
        for i, (k, w) in enumerate(zip(self.kappa, self.wl_um)):
            s.kappa[i], s.wl_um[i] = k, w
        s.pg0, s.q0_jkg, s.h_g = self.pg0, self.q0_jkg, self.h_g
        s.react, s.wall_sink, s.rad_emission, s.maxgi = self.react, self.wall_sink, self.rad_emission, self.maxgi
        s.bgcon, s.adi_mode, s.precision = self.bgcon, self.adi_mode, self.precision
        return s


def _burner_inlets() -> list:
    # One 0.1 x 0.1 m CH4 burner (300 K, 40 m/s) between two 0.2 x 0.15 m air
    # ports (1500 K, 12 m/s), all on the x=0 wall.  inlets[0] is the pressure
    # reference cell, as the reference requires (Sbc.f90:57-63).
    return [
        Inlet(0.95, 1.05, 0.40, 0.50, 300.0, 40.0, yf=1.0),
        Inlet(0.50, 0.70, 0.375, 0.525, 1500.0, 12.0, yo2=AIR_O2, yn2=AIR_N2),
        Inlet(1.30, 1.50, 0.375, 0.525, 1500.0, 12.0, yo2=AIR_O2, yn2=AIR_N2),
    ]


def small_furnace(**kw) -> FurnaceCase:
    """48 x 24 x 16 cells (18,432): the plain-method small case."""
    return FurnaceCase(name="furnace_48x24x16", nx=48, ny=24, nz=16, inlets=_burner_inlets(), **kw)


def medium_furnace(**kw) -> FurnaceCase:
    """96 x 48 x 32 cells (147,456): the same furnace at half the resolution,
    for kernel captures on a state larger than L2 but a few hundred MB."""
    kw.setdefault("inlet_jitter", 0.05)
    return FurnaceCase(name="furnace_96x48x32", nx=96, ny=48, nz=32, inlets=_burner_inlets(), **kw)


def large_furnace(**kw) -> FurnaceCase:
    """192 x 96 x 64 cells (1,179,648), inlet velocities jittered +-5%."""
    kw.setdefault("inlet_jitter", 0.05)
    return FurnaceCase(name="furnace_192x96x64", nx=192, ny=96, nz=64, inlets=_burner_inlets(), **kw)


def xl_furnace(seed: int = 5, **kw) -> FurnaceCase:
    """384 x 160 x 96 cells (5,898,240) with 10 gray bands whose absorption
    coefficients are drawn log-uniform on 0.05-5 1/m from `seed` (band edges
    geometric from 1.2 to 40 um, the last band open to 1000 um): the
    combustion space of the large coupled configuration, without its melt
    coupling."""
    import random
    rnd = random.Random(seed)
    kappa = tuple(math.exp(rnd.uniform(math.log(0.05), math.log(5.0))) for _ in range(10))
    wl = tuple(1.2 * (40.0 / 1.2) ** (i / 8.0) for i in range(9)) + (1000.0,)
    kw.setdefault("inlet_jitter", 0.05)
    return FurnaceCase(name="furnace_384x160x96", nx=384, ny=160, nz=96, inlets=_burner_inlets(), kappa=kappa,
                       wl_um=wl, **kw)


def furnace_variant(seed: int, nx: int = 48, ny: int = 24, nz: int = 16, aspect: float | None = None,
                    **kw) -> FurnaceCase:
    """A seeded variant of the burner furnace: burner velocity uniform in
    20-60 m/s and air temperature uniform in 1200-1700 K; with `aspect`, the
    box length is aspect x 2.0 m.  Used for the learned p' guess's training
    systems (variants of the 48x24x16 case) and for the batched runs."""
    import random
    rnd = random.Random(seed)
    u = rnd.uniform(20.0, 60.0)
    t_air = rnd.uniform(1200.0, 1700.0)
    inl = _burner_inlets()
    inl[0].u_ms = u
    inl[1].t_k = inl[2].t_k = t_air
    if aspect is not None:
        kw["lx"] = aspect * 2.0
    kw.setdefault("seed", 1000003 * (seed + 1))
    return FurnaceCase(name=f"furnace_{nx}x{ny}x{nz}_v{seed}", nx=nx, ny=ny, nz=nz, inlets=inl, **kw)


def batch_variants(n: int = 64, seed: int = 7) -> list:
    """n furnace variants with grid, box aspect, burner velocity and air
    temperature drawn from a seed: nx in 32..128, ny in 16..64, nz in 12..48
    cells, aspect 1.5-3.0 (all extents even)."""
    import random
    rnd = random.Random(seed)
    out = []
    for i in range(n):
        nx = 2 * rnd.randint(16, 64)
        ny = 2 * rnd.randint(8, 32)
        nz = 2 * rnd.randint(6, 24)
        out.append(furnace_variant(seed * 7919 + i, nx, ny, nz, aspect=rnd.uniform(1.5, 3.0)))
    return out


def tiny_furnace(nx=12, ny=8, nz=6, **kw) -> FurnaceCase:
    """A few hundred cells: every cell can be checked against the oracle quickly."""
    inl = [
        Inlet(0.75, 1.25, 0.3, 0.7, 300.0, 40.0, yf=1.0),
        Inlet(0.25, 0.75, 0.3, 0.7, 1500.0, 12.0, yo2=AIR_O2, yn2=AIR_N2),
    ]
    return FurnaceCase(name=f"furnace_{nx}x{ny}x{nz}", nx=nx, ny=ny, nz=nz, inlets=inl,
                       exit_yz=(0.5, 1.5, 0.3, 0.9), **kw)
