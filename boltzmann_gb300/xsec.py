"""Electron-argon cross sections as n*sigma tables on a log energy grid.

The push kernel reads a [3, n] float32 table of n*sigma (m^-1) for (elastic,
excitation, ionization) on ``n`` log-spaced energies between ``emin`` and ``emax`` eV
and interpolates linearly in log2(energy). Sources:

* ``analytic_argon``: elastic 1e-19 m^2 (e/1 eV)^0.3 capped at 1.5e-19 m^2;
  excitation 3e-21 m^2 ln(e/11.5)/(e/11.5) above 11.5 eV; ionization
  3e-20 m^2 ln(e/15.76)/(e/15.76) above 15.76 eV (the benchmark argon set).
* ``reference_fits``: the reference's piecewise log10-quadratic fits for elastic and
  ionization (electron_kernel_numba.py:66-174), no excitation. The kernels can also
  evaluate these fits directly in float64 (``xs_mode = XS_REF_FITS``).
* ``read_lxcat``: tabulated (energy, sigma) pairs in the LXCat text layout.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

E_ION = 15.76
E_EXC = 11.5


@dataclass(frozen=True)
class XsTable:
    sigma: np.ndarray  # [3, n] float64 cross sections, m^2 (elastic, excitation, ionization)
    emin: float
    emax: float
    e_exc: float = E_EXC

    @property
    def n(self):
        return self.sigma.shape[1]

    def energies(self):
        return log_grid(self.emin, self.emax, self.n)

    def nsigma(self, nn_m3):
        """n*sigma in m^-1 as the float32 table the kernels read."""
        return np.ascontiguousarray((self.sigma * nn_m3).astype(np.float32))

    def nu_max(self, nn_m3):
        """Upper bound of n sigma_tot(e) v(e) over the grid (null-collision bound), s^-1."""
        e = self.energies()
        v = np.sqrt(2.0 * e / (9.10938e-31 * 6.241509e18))
        return float(np.max(self.sigma.sum(axis=0) * nn_m3 * v)) * 1.01


def log_grid(emin, emax, n):
    """Energies of the table points: log2-uniform from emin to emax (the kernel's grid)."""
    t = np.arange(n, dtype=np.float64) / (n - 1)
    return np.exp2(math.log2(emin) + t * (math.log2(emax) - math.log2(emin)))


def analytic_argon(n=2000, emin=0.01, emax=1000.0):
    e = log_grid(emin, emax, n)
    el = np.minimum(1e-19 * e ** 0.3, 1.5e-19)
    xe = e / E_EXC
    ex = np.where(e > E_EXC, 3e-21 * np.log(np.maximum(xe, 1.0)) / xe, 0.0)
    xi = e / E_ION
    io = np.where(e > E_ION, 3e-20 * np.log(np.maximum(xi, 1.0)) / xi, 0.0)
    return XsTable(np.stack([el, ex, io]), emin, emax, E_EXC)


# electron_kernel_numba.py:66-174
_EL = [(-0.02704763, -0.23720051, -19.67900951), (-0.08847237, -0.6084786, -20.24111992),
       (-0.37608274, -1.8167778, -21.51414308), (-1.4874467, -4.82420619, -23.55745478),
       (-0.9870356, -4.2206026, -23.44715988), (14.28063581, 18.92275458, -14.70556113),
       (-2.12069169, 0.7555105, -19.71943671), (-0.3585636, 0.79246666, -19.71260274),
       (1.25262128, -0.40002029, -19.48909003), (-2.28332905, 4.89566076, -21.46789173),
       (-1.47508661, 2.82263476, -20.1928456), (-0.11090525, -0.77506081, -17.81752307)]
_EL_E = [0.000780396, 0.006098667, 0.0476269, 0.1015574, 0.1943527, 0.2995781, 1.097156, 2.339524,
         4.988691, 10.63765, 22.68322]
_IO = [(-2149239.99337822, 5150451.29014456, -3085665.64874862), (-227229.83440255, 545171.14839945, -327016.69508374),
       (-20173.68563579, 48599.13254342, -29290.96100603), (-1838.90888364, 4491.58838596, -2763.82866252),
       (-186.98923927, 477.04784782, -324.75732578), (-24.48843901, 69.43965607, -69.145292411),
       (-4.33101714, 14.47124519, -31.66224458), (-0.68345667, 2.6053539, -21.99823511)]
_IO_E = [15.77742, 15.81964, 15.96196, 16.44162, 18.05837, 23.50771, 41.87498]


def reference_fit_sigmas(e):
    """(elastic, ionization) sigma in m^2 from the reference's fits, vectorised."""
    e = np.asarray(e, dtype=np.float64)
    le = np.log10(e)
    k = np.searchsorted(np.array(_EL_E), e, side="right")
    a = np.array([c[0] for c in _EL])[k]
    b = np.array([c[1] for c in _EL])[k]
    c = np.array([c[2] for c in _EL])[k]
    el = 10.0 ** ((a * le + b) * le + c)
    j = np.searchsorted(np.array(_IO_E), e, side="right")
    ai = np.array([c[0] for c in _IO])[j]
    bi = np.array([c[1] for c in _IO])[j]
    ci = np.array([c[2] for c in _IO])[j]
    io = np.where(e > E_ION, 10.0 ** ((ai * le + bi) * le + ci), 0.0)
    return el, io


def reference_fits(n=4000, emin=1e-3, emax=1000.0):
    e = log_grid(emin, emax, n)
    el, io = reference_fit_sigmas(e)
    return XsTable(np.stack([el, np.zeros_like(el), io]), emin, emax, E_EXC)


def read_lxcat(path_or_text, n=2000, emin=0.01, emax=1000.0):
    """Parse an LXCat-style text file (ELASTIC / EXCITATION / IONIZATION blocks, each a
    header, a threshold or mass-ratio line, and a table of "energy(eV) sigma(m2)" rows
    between two lines of dashes) and resample it onto the kernel's log grid.
    Several blocks of the same kind are summed. Values outside a block's table are 0
    below its first energy and held at the last value above its end."""
    text = path_or_text
    if "\n" not in path_or_text:
        with open(path_or_text) as f:
            text = f.read()
    lines = text.splitlines()
    grid = log_grid(emin, emax, n)
    out = np.zeros((3, n))
    kinds = {"ELASTIC": 0, "EFFECTIVE": 0, "EXCITATION": 1, "IONIZATION": 2}
    e_exc = None
    i = 0
    while i < len(lines):
        key = lines[i].strip().upper()
        if key in kinds:
            kind = kinds[key]
            thr = None
            j = i + 1
            # threshold (eV) for excitation / ionization is the first number on line i+2
            try:
                thr = float(lines[i + 2].split()[0])
            except (ValueError, IndexError):
                thr = None
            while j < len(lines) and not lines[j].strip().startswith("-----"):
                j += 1
            j += 1
            rows = []
            while j < len(lines) and not lines[j].strip().startswith("-----"):
                parts = lines[j].split()
                if len(parts) >= 2:
                    rows.append((float(parts[0]), float(parts[1])))
                j += 1
            if rows:
                t = np.array(rows)
                s = np.interp(grid, t[:, 0], t[:, 1], left=0.0, right=t[-1, 1])
                out[kind] += s
                if kind == 1 and thr is not None:
                    e_exc = thr if e_exc is None else min(e_exc, thr)
            i = j + 1
        else:
            i += 1
    return XsTable(out, emin, emax, e_exc if e_exc is not None else E_EXC)
