"""Frozen run configurations for the electron PIC-MCC path.

The reference hard-codes its physics in ``boltzmann.py:46-78`` and the kernel
(``electron_kernel_numba.py:13-24``) and takes the rest from ``main.py``'s flags
(-N particles, -g grid points, -bnf, -rsf resample frequency, -dt (dt = tau/dt),
-spc steps per cycle). ``CCPConfig`` carries all of it; ``reference(...)`` reproduces
the reference's settings for its 1/3/5-bin variants, and ``ccp_256`` / ``ccp_1024``
are the 1 Torr argon CCP workloads (256 cells / 2e6 particles / 3 bins and 1024 cells /
2e7 particles / 5 bins).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace
from typing import Optional, Tuple

from . import _lib
from . import xsec as _xs

M_E = 9.10938e-31
J_EV = 6.241509e18
K_B = 1.380649e-23
M_AR = 6.6e-26

# target fractions per energy bin of the reference variants (boltzmann.py:147;
# 3bin/boltzmann.py:147-149; 5bin/boltzmann.py:147-151) and their edges (eV)
REF_BINS = {
    1: ((), (1.0,)),
    3: ((10.0, 15.76), (0.7, 0.2, 0.1)),
    5: ((5.0, 10.0, 15.76, 20.0), (0.4, 0.3, 0.2, 0.07, 0.03)),
}


def gas_sigma_reference():
    """The reference's gas-velocity spread: Tg*1.5*1.17255e11 with Tg = 300/11606 eV
    (boltzmann.py:556-561). 1.17255e11 is e/m of the electron, so this is the thermal
    speed of an electron at the gas temperature, not of an argon atom."""
    return math.sqrt((300.0 / 11606.0) * 1.5 * 1.17255e11)


def gas_sigma_argon(T=300.0):
    return math.sqrt(K_B * T / M_AR)


@dataclass(frozen=True)
class CCPConfig:
    # grid (main.py -g, -bnf); L in cm
    gridpts: int = 256
    L: float = 2.54
    bnf: int = 4
    # gas and drive (boltzmann.py:47-63)
    pressure_torr: float = 0.1
    V0: float = 100.0
    freq: float = 13.56e6
    eps0: float = 5.5263e5
    nn_Di: float = 2.07e18
    nn_mui: float = 4.65e19
    # time (main.py -dt, -spc)
    in_dt: float = 50000.0
    steps_per_cycle: int = 5000
    # particles (main.py -N); capacity per buffer = capacity_factor * Nc, held in segments
    # of 2*seg_half slots (one warp pushes one segment)
    num_particles: int = 200000
    capacity_factor: float = 2.5
    seg_half: int = 2048
    Te_init_eV: float = 0.5           # boltzmann.py:249 (the benchmark CCPs start at 1 eV)
    ne_profile: str = "reference"     # "reference" (boltzmann.py:246-247) or "uniform"
    ne_uniform: float = 1e9           # cm^-3 when ne_profile == "uniform"
    # ES-WPNC (boltzmann.py:147-148, 542, 547, 807, 826, 829)
    bin_edges: Tuple[float, ...] = ()
    bin_fractions: Tuple[float, ...] = (1.0,)
    resample_freq: int = 1
    min_wt: float = 0.1
    split_below: float = 0.5
    merge_at: float = 3.0
    # the resampling step's appended particles go into the free slots of the segments (merged
    # ones are dropped by the next push) instead of a full repack of every particle
    resample_in_place: bool = True
    merge_keep: float = 0.6
    max_ppc_factor: float = 10.0
    # collisions
    xs: str = "reference_fits"        # "reference_fits" (float64 fits), "reference_table", "analytic"
    xs_points: int = 2000
    coll_model: int = _lib.COLL_DIRECT
    gas_velocity: str = "reference"   # "reference", "argon", "off"
    # numerics
    precision: str = "float32"        # particle state: "float32" or "float64"
    autotune: bool = True             # time the push's CTA shapes once at start and keep the fastest
    seed: int = 1
    quirks: int = _lib.QUIRK_SPLIT_WRAP | _lib.QUIRK_DEAD_IONFLAG | _lib.QUIRK_TRIGGER_LAST

    # derived -----------------------------------------------------------------------
    @property
    def N(self):
        return self.gridpts - 1

    @property
    def dx(self):
        return self.L / self.N

    @property
    def nn_cm3(self):
        return 3.22e16 * self.pressure_torr

    @property
    def nn_m3(self):
        return 1e6 * self.nn_cm3

    @property
    def mu_i(self):
        return self.nn_mui / self.nn_cm3

    @property
    def D_i(self):
        return self.nn_Di / self.nn_cm3

    @property
    def tau(self):
        return 1.0 / self.freq

    @property
    def dt(self):
        return self.tau / self.in_dt

    @property
    def nbins(self):
        return len(self.bin_edges) + 1

    def targets(self):
        """Per-bin target particles per cell: int(frac * Nc / N) (boltzmann.py:147)."""
        return [int(f * self.num_particles / self.N) for f in self.bin_fractions]

    def max_ppc(self):
        return [int(self.max_ppc_factor * t) for t in self.targets()]

    def gas_sigma(self):
        return {"reference": gas_sigma_reference(), "argon": gas_sigma_argon(), "off": 0.0}[self.gas_velocity]

    def xs_table(self) -> Optional[_xs.XsTable]:
        if self.xs == "analytic":
            return _xs.analytic_argon(self.xs_points)
        if self.xs == "reference_table":
            return _xs.reference_fits(self.xs_points * 2)
        return None

    def xs_mode(self):
        return _lib.XS_REF_FITS if self.xs == "reference_fits" else _lib.XS_TABLE


def reference(variant_bins=1, **kw):
    """The reference's own settings for its 1bin/3bin/5bin variant (main.py defaults
    unless overridden; 0.1 Torr hard-coded at boltzmann.py:47)."""
    edges, fr = REF_BINS[variant_bins]
    return CCPConfig(bin_edges=edges, bin_fractions=fr, **kw)


# The benchmark CCPs resample with the reference's split indexing and trigger but with the
# energy-conserving merge: the reference's rescale (boltzmann.py:861-869) loses the drift
# part of the energy, and these runs are to conserve weight, momentum and energy per bin.
BENCH_QUIRKS = (_lib.QUIRK_SPLIT_WRAP | _lib.QUIRK_DEAD_IONFLAG | _lib.QUIRK_TRIGGER_LAST
                | _lib.FIX_MERGE_ENERGY)


def ccp_256(**kw):
    """1 Torr argon CCP: 256 cells, 2e6 particles at 1 eV, dt = tau/400, 3 bins with
    edges 4 and 11.5 eV, analytic cross sections, energy-conserving merge."""
    base = dict(gridpts=257, pressure_torr=1.0, in_dt=400.0, steps_per_cycle=400, num_particles=2_000_000,
                Te_init_eV=1.0, ne_profile="uniform", bin_edges=(4.0, 11.5), bin_fractions=(0.7, 0.2, 0.1),
                xs="analytic", resample_freq=50, quirks=BENCH_QUIRKS)
    base.update(kw)
    return CCPConfig(**base)


def ccp_1024(**kw):
    """1 Torr argon CCP scale-up: 1024 cells, 2e7 particles, 5 bins with edges 2, 6,
    11.5, 15.76 eV, analytic cross sections, float32 state, energy-conserving merge."""
    base = dict(gridpts=1025, pressure_torr=1.0, in_dt=400.0, steps_per_cycle=400, num_particles=20_000_000,
                Te_init_eV=1.0, ne_profile="uniform", bin_edges=(2.0, 6.0, 11.5, 15.76),
                bin_fractions=(0.4, 0.3, 0.2, 0.07, 0.03), xs="analytic", resample_freq=50, quirks=BENCH_QUIRKS)
    base.update(kw)
    return CCPConfig(**base)
