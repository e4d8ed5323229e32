"""Independent 0-D electron swarms on one GPU.

A 0-D swarm is the reference's electron push and Monte-Carlo collisions
(electron_kernel_numba.py:7-288) with the spatial part switched off: a uniform field, no
drift, no walls. ``SwarmEnsemble`` advances any number of such swarms together: every
particle stores the index of its swarm in ``x`` (``BZ_ADVECT_ENSEMBLE``), so one push per
step covers all swarms, each particle is kicked by its own swarm's field, and the fused
deposit, the binning and the ES-WPNC resampling (boltzmann.py:799-890) work per swarm
because the swarm takes the place of the grid cell. Resampling targets are per (swarm,
energy bin) (``BZ_PER_KEY_TARGETS``), proportional to each swarm's initial size.

Diagnostics per swarm: mean energy, ionization and excitation rate coefficients from the
push's own deposit (rows 0, 1, 3 and, with ``BZ_MOMENT_EXCITATION``, row 2 of the
moments), and the electron energy distribution on a log grid (``bz_seg_eedf_*``).

``swarm_100td()`` is the single argon swarm at E/N = 100 Td (1e5 particles, float64,
dt = 1e-12 s, one energy bin merged back to its target whenever the count exceeds
twice it); ``ensemble_512()`` the 512-swarm sweep over 10-1000 Td.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Optional, Tuple

import numpy as np
import torch

from . import _lib, kernels as K
from . import xsec as _xs
from .config import K_B, M_AR

TD = 1e-21  # V m^2
KTM = 1.5 * 1.17255e11  # (m/s)^2 per eV of temperature


@dataclass(frozen=True)
class SwarmConfig:
    E_over_N_Td: Tuple[float, ...] = (100.0,)
    counts: Tuple[int, ...] = (100_000,)
    nn: float = 3.22e22            # m^-3
    T_gas: float = 300.0           # K (argon thermal motion; 0 switches it off)
    dt: float = 1e-12              # s
    Te_init_eV: float = 1.0
    precision: str = "float64"
    xs_points: int = 2000
    bin_edges: Tuple[float, ...] = ()
    bin_fractions: Tuple[float, ...] = (1.0,)
    resample_every: int = 1
    split_below: float = 0.5
    merge_at: float = 2.0
    merge_keep: float = 1.0
    max_ppc_factor: float = 10.0
    min_wt: float = 0.1
    resample_in_place: bool = True   # appended particles into free slots instead of a full repack
    capacity_factor: float = 7.0      # slots per initial particle: bins may grow to 3x target, run 0 holds half
    seg_half: int = 2048
    seed: int = 1

    @property
    def n_swarms(self):
        return len(self.counts)

    @property
    def nbins(self):
        return len(self.bin_edges) + 1

    def targets(self):
        """Per (swarm, bin) targets, key order swarm*nbins + bin."""
        return np.array([[int(f * c) for f in self.bin_fractions] for c in self.counts], dtype=np.int32).reshape(-1)


def swarm_100td(**kw):
    """One argon swarm: E/N = 100 Td, n = 3.22e22 m^-3, 1e5 equal-weight particles from an
    isotropic 1 eV Maxwellian, dt = 1e-12 s, float64, one energy bin merged back to the
    1e5 target whenever the count exceeds twice it (checked every 10 steps: at 100 Td the
    count grows by well under 1% in 1e4 steps, so no 10 steps can double it). Segments of
    2 x 256 slots spread the 1e5 particles over ~1000 warps."""
    base = dict(E_over_N_Td=(100.0,), counts=(100_000,), precision="float64", merge_at=2.0, merge_keep=1.0,
                capacity_factor=5.0, resample_every=10, seg_half=256)
    base.update(kw)
    return SwarmConfig(**base)


def ensemble_512(seed=0, n_swarms=512, **kw):
    """512 argon swarms, E/N log-uniform in 10-1000 Td and sizes log-uniform in 1e4-2e5
    (seeded), float32 state, 3-bin ES-WPNC per swarm with edges 4 and 11.5 eV."""
    rng = np.random.default_rng(seed)
    td = np.exp(rng.uniform(math.log(10.0), math.log(1000.0), n_swarms))
    cnt = np.exp(rng.uniform(math.log(1e4), math.log(2e5), n_swarms)).astype(np.int64)
    base = dict(E_over_N_Td=tuple(float(t) for t in td), counts=tuple(int(c) for c in cnt), precision="float32",
                bin_edges=(4.0, 11.5), bin_fractions=(0.7, 0.2, 0.1), merge_at=3.0, merge_keep=0.6,
                resample_every=10)
    base.update(kw)
    return SwarmConfig(**base)


class SwarmEnsemble:
    """S independent swarms advanced by one push per step (see the module docstring)."""

    def __init__(self, cfg: SwarmConfig, device="cuda", xs: Optional[_xs.XsTable] = None):
        self.cfg = cfg
        self.device = device
        self.dtype = torch.float32 if cfg.precision == "float32" else torch.float64
        S = cfg.n_swarms
        self.S = S
        dev = device
        f64 = dict(dtype=torch.float64, device=dev)
        self.xs = xs or _xs.analytic_argon(cfg.xs_points)
        self.xs_t = torch.as_tensor(self.xs.nsigma(cfg.nn), device=dev)
        # field per swarm, V/cm (the push's kick takes V/cm): E = (E/N) N
        self.E = torch.as_tensor(np.asarray(cfg.E_over_N_Td) * TD * cfg.nn / 100.0, dtype=self.dtype, device=dev)
        # particles: swarm index in x, isotropic Maxwellian, weight 1
        n0 = int(sum(cfg.counts))
        g = torch.Generator(device=dev)
        g.manual_seed(int(cfg.seed))
        sw = torch.repeat_interleave(torch.arange(S, device=dev, dtype=torch.float64),
                                     torch.as_tensor(np.asarray(cfg.counts), device=dev))
        v = torch.randn(n0, 3, generator=g, device=dev, dtype=torch.float64) * math.sqrt(cfg.Te_init_eV * KTM)
        cap = int(math.ceil(cfg.capacity_factor * n0))
        half = int(cfg.seg_half)
        nseg = max(1, -(-cap // half))
        self.A = K.SegmentSet(nseg, half, self.dtype, dev)
        self.B = K.SegmentSet(nseg, half, self.dtype, dev)
        self.app = K.ParticleSet(max(cap, 1), self.dtype, dev)
        for f, a in zip(K.ParticleSet.FIELDS, (sw, v[:, 0], v[:, 1], v[:, 2], torch.ones(n0, **f64))):
            getattr(self.app, f)[:n0].copy_(a.to(self.dtype))
        self.app.cnt.zero_()
        self.app.cnt[2] = n0
        del sw, v
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.seg_flags = torch.zeros(1, dtype=torch.int32, device=dev)
        self.ws = K.Workspace(dev)
        K.seg_repack(None, self.A, self.status, self.ws, app=self.app)
        # resampling tables (per swarm and bin)
        nb = cfg.nbins
        self.nb = nb
        nkeys = S * nb
        self.edges = torch.as_tensor(np.asarray(cfg.bin_edges, dtype=np.float64) if nb > 1 else np.zeros(1), device=dev)
        tg = cfg.targets()
        self.targets = torch.as_tensor(tg, device=dev)
        self.max_ppc = torch.as_tensor((cfg.max_ppc_factor * tg).astype(np.int32), device=dev)
        self.perm = torch.zeros(self.A.capacity, dtype=torch.int32, device=dev)
        self.offsets = torch.zeros(nkeys + 1, dtype=torch.int32, device=dev)
        self.bin_counts = torch.zeros(nkeys, dtype=torch.int32, device=dev)
        self.hw_counts = torch.zeros(nkeys, dtype=torch.int32, device=dev)
        self.need = torch.zeros(1, dtype=torch.int32, device=dev)
        # moments of the last step per swarm and running sums
        self.moments = torch.zeros(4, S, **f64)
        self.acc = torch.zeros(4, S, **f64)      # sums over steps of rows 0..3
        self.acc_pre = torch.zeros(S, **f64)     # sum over steps of the pre-push population
        self.steps_acc = 0
        self.step_dev = torch.zeros(1, dtype=torch.int64, device=dev)
        self.particle_steps = torch.zeros(1, dtype=torch.int64, device=dev)
        self.bigstep = 0
        self._graphs = {}
        self._kinds = set()
        self.push_shape = None
        if self.dtype == torch.float32:
            best, times = K.autotune_seg_push(self.params(step_on_device=False), self.A, self.B, self.E, self.status,
                                              self.seg_flags, self.ws, self.moments)
            self.push_shape = {"shape": K.seg_push_shapes()[best], "ms": times}

    # ----------------------------------------------------------------------------------
    def params(self, step_on_device=True):
        cfg = self.cfg
        gas = math.sqrt(K_B * cfg.T_gas / M_AR) if cfg.T_gas > 0 else 0.0
        return K.make_params(
            n_faces=self.S, n_nodes=self.S, bnf=1, advect=_lib.ADVECT_ENSEMBLE, L=float(self.S), dx=1.0, dt=cfg.dt,
            nn=cfg.nn, gas_sigma=gas, e_exc=self.xs.e_exc, xs_mode=_lib.XS_TABLE, xs_table=self.xs_t,
            xs_emin=self.xs.emin, xs_emax=self.xs.emax, flags=_lib.PER_KEY_TARGETS | _lib.MOMENT_EXCITATION,
            seed=cfg.seed, step=self.bigstep, step_ptr=self.step_dev if step_on_device else None)

    def electron_kernel(self):
        """One push + collide of every swarm, deposit per swarm fused in."""
        p = self.params()
        p.flags |= _lib.CLEAR_MOMENTS  # the push clears the moments before it deposits
        K.seg_electron_kernel(p, self.A, self.B, self.E, self.status, self.seg_flags, self.ws,
                              moments=self.moments, n_pushed=self.particle_steps)
        self.A, self.B = self.B, self.A
        # pre-push population = after-push weight minus the children (every ionization
        # adds one particle of its parent's weight; a 0-D swarm loses none)
        self.acc.add_(self.moments)
        self.acc_pre.add_(self.moments[0] - self.moments[1])

    def _repack_if_needed(self):
        K.seg_rebalance(self.A, self.B, self.status, self.ws, only_if=self.seg_flags, clear=self.seg_flags)

    def _resample(self):
        cfg = self.cfg
        p = self.params()
        ed = self.edges[: self.nb - 1] if self.nb > 1 else self.edges[:0]
        # the trigger from the counts first: the sort by key runs only when resampling will
        K.seg_bin_particles(p, self.A, ed, cfg.min_wt, self.perm, self.offsets, self.bin_counts, self.hw_counts,
                            self.status, self.ws, check=(self.targets, cfg.split_below, cfg.merge_at, self.need))
        K.seg_resample(p, self.A, self.app, self.B, self.nb, self.targets, self.max_ppc, cfg.min_wt, cfg.split_below,
                       cfg.merge_at, cfg.merge_keep, self.perm, self.offsets, self.bin_counts, self.hw_counts,
                       self.status, self.seg_flags, self.ws, need=self.need, in_place=cfg.resample_in_place)
        if not cfg.resample_in_place:
            self.A, self.B = self.B, self.A

    def _step_body(self, resample):
        self.electron_kernel()
        if resample:
            self._resample()
        else:
            self._repack_if_needed()
        K.advance_clock(None, self.step_dev, self.cfg.dt)

    def step(self, use_graph=True):
        """One step of every swarm. A step kind (resample or not) runs eagerly the first
        time; after that each (kind, buffer roles) is captured into a CUDA graph once and
        replayed."""
        resample = (self.bigstep + 1) % self.cfg.resample_every == 0
        key = (resample, self.A is self._first_A())
        if use_graph and resample in self._kinds:
            gr = self._graphs.get(key) or self._capture_key(key)
            gr.replay()
            for _ in range(2 if resample and not self.cfg.resample_in_place else 1):
                self.A, self.B = self.B, self.A
        else:
            self._kinds.add(resample)
            self._step_body(resample)
        self.bigstep += 1
        self.steps_acc += 1

    def run(self, num_steps, use_graph=True):
        for _ in range(num_steps):
            self.step(use_graph=use_graph)
        return self

    def capture_all(self):
        """Capture the graphs of every step kind that has run once (both buffer roles)."""
        for resample in sorted(self._kinds):
            for first in (True, False):
                if (resample, first) not in self._graphs:
                    self._capture_key((resample, first))

    def _capture_key(self, key):
        resample, first = key
        swap = (self.A is self._first_A()) != first
        if swap:
            self.A, self.B = self.B, self.A
        g = self._capture(resample)
        if swap:
            self.A, self.B = self.B, self.A
        self._graphs[key] = g
        return g

    def _first_A(self):
        if not hasattr(self, "_A0"):
            self._A0 = self.A
        return self._A0

    def _capture(self, resample):
        lib = _lib.load()
        self.ws.get("seg_push", lib.bz_seg_push_workspace_nodes(self.S))
        self.ws.get("seg_rebalance", lib.bz_seg_repack_workspace(self.A.nseg))
        self.ws.get("seg_bin", lib.bz_seg_bin_workspace(self.A.nseg, self.A.capacity))
        self.ws.get("seg_resample", lib.bz_seg_resample_workspace(self.A.nseg, self.A.capacity, self.S * self.nb))
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream())
        g = torch.cuda.CUDAGraph()
        saved = (self.A, self.B)
        torch.cuda.current_stream().wait_stream(s)
        with torch.cuda.graph(g, stream=s, capture_error_mode="relaxed"):
            self._step_body(resample)
        self.A, self.B = saved
        return g

    # ---------------------------------------------------------------------------------- diagnostics
    def reset_averages(self):
        self.acc.zero_()
        self.acc_pre.zero_()
        self.steps_acc = 0

    def n(self):
        """Particles in all swarms (the step ends with the resampling, whose merges may leave
        emptied slots until the next push: those are not counted)."""
        return self.A.n_live()

    def counts(self):
        """Weight (particle count at weight 1) per swarm after the last step."""
        return self.moments[0].cpu().numpy()

    def mean_energy(self):
        """Time-averaged mean energy per swarm (eV) since the last reset."""
        a = self.acc.cpu().numpy()
        return a[3] / np.maximum(a[0], 1e-300)

    def rate_coefficients(self):
        """Time-averaged ionization and excitation rate coefficients per swarm (m^3/s):
        events per step / (pre-push population x n x dt)."""
        a = self.acc.cpu().numpy()
        pre = self.acc_pre.cpu().numpy()
        den = np.maximum(pre, 1e-300) * self.cfg.nn * self.cfg.dt
        return a[1] / den, a[2] / den

    def eedf(self, nbins=64, emin=0.01, emax=100.0, normalise=True):
        """Electron energy distribution per swarm on nbins log bins over [emin, emax) eV:
        the fraction of each swarm's weight in every bin (or the raw weights)."""
        h = torch.zeros(self.S, nbins, dtype=torch.float64, device=self.device)
        K.seg_eedf(self.params(step_on_device=False), self.A, h, emin, emax)
        h = h.cpu().numpy()
        if normalise:
            h = h / np.maximum(h.sum(axis=1, keepdims=True), 1e-300)
        return h

    def device_status(self):
        return int(self.status.item())
