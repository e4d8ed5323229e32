"""The hybrid CCP step loop on the CPU, built from the oracle's kernels (test
infrastructure: the checker for the GPU solver, never part of the product).

Step order of BoltzmannDSMC.run (boltzmann.py:570-678): every ``resample_freq`` steps
define_particle_bins + _check_for_resampling / _do_resampling (boltzmann.py:894-916,
799-890; the reference's trigger: only the last bin's merge test decides), then
electron_kernel + post_processing (push, collide, deposit, compaction), the host grid
update (ni += ni_src, Te = 2/3 nrg/ne, boltzmann.py:643-647), the clock, the ion fluid
(heavies_kernel_1D.py:4-64) and the Poisson solve (EF_kernel_1D.py:7-44). Float64,
array-of-structures, Philox random numbers keyed by the particle's index (so the stream
differs from the GPU's, which keys by segment slot: the two runs agree statistically).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import oracle as O


class OracleCCP:
    def __init__(self, cfg, x, vx, vy, vz, w, ni, xs_table, seed=7, threads=None):
        self.cfg = cfg
        N = cfg.N
        self.N = N
        self.nn_nodes = N + 1
        n = len(x)
        self.cap = int(8 * max(n, 1))
        self.data, self.tosum = O.soa_to_aos(np.asarray(x, float), np.asarray(vx, float), np.asarray(vy, float),
                                             np.asarray(vz, float), np.asarray(w, float), cap=self.cap)
        self.n = n
        self.dtmp = np.zeros((2 * self.cap, 6))
        self.ttmp = np.zeros((2 * self.cap, 4))
        tab = xs_table
        self.p = O.make_params(N, L=cfg.L, bnf=cfg.bnf, dt=cfg.dt, nn=cfg.nn_m3, rng_mode=1, precision=64, seed=seed,
                               gas_sigma=cfg.gas_sigma(), xs_table=tab.nsigma(cfg.nn_m3), xs_emin=tab.emin,
                               xs_emax=tab.emax, e_exc=tab.e_exc)
        self.ni = np.array(ni, dtype=np.float64)
        self.moments = np.zeros((4, N + 1))
        self.Te = np.zeros(N + 1)
        self.t = 0.0
        self.step_no = 0
        self.rng = np.random.default_rng(seed + 1)
        self.threads = threads or os.cpu_count() or 1
        self.targets = np.asarray(cfg.targets(), dtype=np.int64)
        self.max_ppc = np.asarray(cfg.max_ppc(), dtype=np.int64)
        # deposit of the initial state and the first field solve (boltzmann.py:363-399)
        self.moments = O.deposit(self.p, self.data, self.tosum, self.n)
        self.ni += self.moments[1]
        _, self.E = O.poisson(N, cfg.dx, cfg.eps0, cfg.V0, cfg.freq, 0.0, self.moments[0], self.ni)
        self.ionized = 0.0

    def _resample(self):
        cfg = self.cfg
        d, t, n = self.data, self.tosum, self.n
        edges = list(cfg.bin_edges)
        counts, lists = O.bin_particles(self.p, d[:n, 0], d[:n, 3], d[:n, 4], d[:n, 5], t[:n, 0], edges,
                                        int(self.max_ppc.max()))
        nb = len(edges) + 1
        # the reference's trigger: its last test (the highest bin's merge test) decides
        if not np.any(counts[nb - 1] >= cfg.merge_at * self.targets[nb - 1]):
            return
        u = self.rng.random(4 * int(self.targets.sum()) * self.nn_nodes + 16)
        self.n, _ = O.resample(self.p, d, t, n, nb, self.targets, cfg.min_wt, self.max_ppc, counts, lists, u, flags=1,
                               thr=(cfg.split_below, cfg.merge_at, cfg.merge_keep))

    def step(self):
        cfg = self.cfg
        if self.step_no % cfg.resample_freq == 0:
            self._resample()
        if 2 * self.n > self.cap:
            raise RuntimeError("oracle CCP outgrew its buffers")
        self.p.step = self.step_no
        mom = np.zeros((4, self.N + 1))
        n_new = O.lib().orc_step_omp(ctypes.byref(self.p), self.n, self.cap, self.data, self.tosum, self.dtmp,
                                     self.ttmp, np.ascontiguousarray(self.E), mom, self.threads)
        if n_new < 0:
            raise RuntimeError("oracle step refused")
        self.n = int(n_new)
        self.moments = mom
        self.ionized += mom[1].sum()
        # host grid update, clock, ion fluid, Poisson
        self.ni = self.ni + mom[1]
        with np.errstate(divide="ignore", invalid="ignore"):
            te = (2.0 / 3.0) * mom[3] / mom[0]
        self.Te = np.where(np.isnan(te), 0.0, te)
        self.t += cfg.dt
        self.ni, _, _ = O.fluid(self.N, cfg.dx, cfg.dt, cfg.mu_i, cfg.D_i, self.E, self.ni)
        _, self.E = O.poisson(self.N, cfg.dx, cfg.eps0, cfg.V0, cfg.freq, self.t, mom[0], self.ni)
        self.step_no += 1

    def state(self):
        n = self.n
        return {"x": self.data[:n, 0].copy(), "vx": self.data[:n, 3].copy(), "vy": self.data[:n, 4].copy(),
                "vz": self.data[:n, 5].copy(), "w": self.tosum[:n, 0].copy()}
