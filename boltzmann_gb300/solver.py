"""Device-resident hybrid electron PIC-MCC solver with the reference's entry points.

``BoltzmannGB300`` mirrors ``BoltzmannDSMC`` (boltzmann.py:22-916): the same step
order (resample check every ``resample_freq`` steps, push + collide, deposit and
compaction, grid update, ion fluid, Poisson; boltzmann.py:570-678) and the same method
names (electron_kernel, post_processing, bin_particles, _check_for_resampling,
_do_resampling, heavies_kernel_fluid, EF_kernel, run, data_write). Everything runs
on one GPU stream; counts, the step clock and the RF time live in device memory, so a
step is captured once into a CUDA graph and replayed.
"""
from __future__ import annotations

import math
import warnings
import os

import numpy as np
import torch

from . import _lib, kernels as K
from .config import CCPConfig

KTM = 1.5 * 1.17255e11  # (m/s)^2 per eV of temperature (boltzmann.py:263)


class CycleAverages:
    """Cycle averages of the step loop (boltzmann.py:681-701): the fields after every step
    whose number (counted from 1) is not a multiple of steps_per_cycle are summed; after
    the cycle's last step the sums are divided by steps_per_cycle. The reference leaves
    that last step out of the sums and still divides by the full count; so does this."""

    def __init__(self, like):
        self.acc = {k: torch.zeros_like(v) for k, v in like.items()}

    def add(self, fields):
        for k, v in self.acc.items():
            v.add_(fields[k])

    def take(self, spc):
        """The averages of the cycle that just ended; the sums start again from zero."""
        ca = {k: v / spc for k, v in self.acc.items()}
        for v in self.acc.values():
            v.zero_()
        return ca


class BoltzmannGB300:
    def __init__(self, cfg: CCPConfig, device="cuda", capacity=None):
        self.cfg = cfg
        self.device = device
        self.dtype = torch.float32 if cfg.precision == "float32" else torch.float64
        N = cfg.N
        self.N = N
        self.nnodes = N + 1
        dev = device
        f64 = dict(dtype=torch.float64, device=dev)
        # particles: initial condition (boltzmann.py:242-333), spread over the segments
        x, vx, vy, vz, w = self._initial_condition()
        n0 = x.numel()
        cap = capacity or int(math.ceil(cfg.capacity_factor * max(n0, cfg.num_particles)))
        self.capacity = cap
        half = int(cfg.seg_half)
        nseg = max(1, -(-cap // half))
        self.A = K.SegmentSet(nseg, half, self.dtype, dev)
        self.B = K.SegmentSet(nseg, half, self.dtype, dev)
        self.app = K.ParticleSet(max(cap, 1), self.dtype, dev)  # resampling appends, then the IC staging
        for f, a in zip(K.ParticleSet.FIELDS, (x, vx, vy, vz, w)):
            getattr(self.app, f)[:n0].copy_(a.to(self.dtype))
        self.app.cnt.zero_()
        self.app.cnt[2] = n0
        del x, vx, vy, vz, w
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.seg_flags = torch.zeros(1, dtype=torch.int32, device=dev)
        self.ws = K.Workspace(dev)
        K.seg_repack(None, self.A, self.status, self.ws, app=self.app)
        # grid arrays (boltzmann.py:94-109). E, ni, Te and the moments are views of one
        # float64 block so that a host loop moves them with one copy each way: the first
        # 5N+4 values are the reference's per-step host->device block [E, ne, ni, ns, Te]
        # (boltzmann.py:719-741; the ne and ns slots are host-side only, the device reads
        # the deposited moments), followed by the moments [4][N+1] that post_processing
        # returns (ne, ni_src, ns_src, nrg)
        nn = self.nnodes
        self.io = torch.zeros(5 * N + 4 + 4 * nn, **f64)
        self.io_in = 5 * N + 4
        self.E = self.io[0:N]
        self.ni = self.io[2 * N + 1: 3 * N + 2]
        self.Te = self.io[4 * N + 3: 5 * N + 4]
        self.moments = self.io[5 * N + 4:].view(4, nn)
        self.ni.copy_(torch.as_tensor(self._ne_profile(), **f64))
        self.E_push = torch.zeros(N, dtype=self.dtype, device=dev)
        self.V = torch.zeros(N - 1, **f64)
        self.Ji = torch.zeros(N, **f64)
        self.g2 = torch.zeros(self.nnodes, **f64)
        self.chol_d = torch.zeros(max(N - 1, 1), **f64)
        self.chol_l = torch.zeros(max(N - 1, 1), **f64)
        self.poisson_plan = torch.zeros(4 * max(N - 1, 1), **f64)
        self.t = torch.zeros(1, **f64)
        self.step_dev = torch.zeros(1, dtype=torch.int64, device=dev)
        self.brk = torch.zeros(1, dtype=torch.int32, device=dev)
        # cross sections
        tab = cfg.xs_table()
        self.xs = tab
        self.xs_t = None if tab is None else torch.as_tensor(tab.nsigma(cfg.nn_m3), device=dev)
        # ES-WPNC tables (boltzmann.py:538-548)
        nb = cfg.nbins
        self.nb = nb
        nkeys = self.nnodes * nb
        self.edges = torch.as_tensor(np.asarray(cfg.bin_edges, dtype=np.float64).reshape(-1) if nb > 1
                                     else np.zeros(1), device=dev)
        self.targets = torch.as_tensor(np.asarray(cfg.targets(), dtype=np.int32), device=dev)
        self.max_ppc = torch.as_tensor(np.asarray(cfg.max_ppc(), dtype=np.int32), device=dev)
        self.perm = torch.zeros(self.A.capacity, dtype=torch.int32, device=dev)
        self.offsets = torch.zeros(nkeys + 1, dtype=torch.int32, device=dev)
        self.bin_counts = torch.zeros(nkeys, dtype=torch.int32, device=dev)
        self.hw_counts = torch.zeros(nkeys, dtype=torch.int32, device=dev)
        self.need = torch.zeros(1, dtype=torch.int32, device=dev)
        self.bigstep = 0
        self.particle_steps = torch.zeros(1, dtype=torch.int64, device=dev)
        self._graphs = {}
        self._replayed = set()  # graph keys replayed at least once since their capture
        self._kinds = set()
        self._host_io = None
        self._ion_rate = None  # ion-source rate closure per node (set_ion_closure), else None
        self._brk_warned = False
        if N >= 3:
            K.poisson_factor(N, cfg.dx, self.chol_d, self.chol_l, self.poisson_plan)
        # first deposit and field solve (boltzmann.py:363-399)
        K.seg_deposit(self.params(), self.A, self.moments)
        self.ni.add_(self.moments[1])
        self._grid_solves(advance=False)
        # CTA shape of the push, timed on the initial state (A is only read)
        self.push_shape = None
        if cfg.autotune:
            self.retune()

    # ---------------------------------------------------------------------------------
    def _ne_profile(self):
        cfg = self.cfg
        xg = np.linspace(0, cfg.L, self.nnodes)
        if cfg.ne_profile == "uniform":
            return np.full(self.nnodes, cfg.ne_uniform)
        return cfg.pressure_torr * (1e7 + 1e9 * (1 - xg / cfg.L) ** 2 * (xg / cfg.L) ** 2)  # boltzmann.py:247

    def _initial_condition(self):
        """Particles per node at the node position (dx/4 inside at the walls), isotropic
        Maxwellian at Te_init, weight = density / particles per node (boltzmann.py:256-300);
        or, for ne_profile == 'uniform', positions uniform in (0, L)."""
        cfg = self.cfg
        g = torch.Generator(device=self.device)
        g.manual_seed(int(cfg.seed))
        dev = self.device
        ppc = int(sum(cfg.targets()))
        ne = self._ne_profile()
        sig = math.sqrt(cfg.Te_init_eV * KTM)
        if cfg.ne_profile == "uniform":
            n = int(cfg.num_particles)
            x = torch.rand(n, generator=g, device=dev, dtype=torch.float64) * cfg.L
            x = x.clamp(1e-6 * cfg.L, cfg.L * (1 - 1e-6))
            w = torch.full((n,), cfg.ne_uniform * self.nnodes / n, device=dev, dtype=torch.float64)
        else:
            n = ppc * self.nnodes
            xg = torch.linspace(0, cfg.L, self.nnodes, device=dev, dtype=torch.float64)
            xg[0] += cfg.dx / 4.0
            xg[-1] -= cfg.dx / 4.0
            x = xg.repeat_interleave(ppc)
            w = torch.as_tensor(ne / ppc, device=dev).repeat_interleave(ppc)
        v = torch.randn(n, 3, generator=g, device=dev, dtype=torch.float64) * sig
        perm = torch.randperm(n, generator=g, device=dev)  # the reference shuffles (boltzmann.py:315-318)
        return x[perm], v[perm, 0].contiguous(), v[perm, 1].contiguous(), v[perm, 2].contiguous(), w[perm]

    def params(self, step_on_device=True):
        cfg = self.cfg
        tab = self.xs
        return K.make_params(
            n_faces=self.N, n_nodes=self.nnodes, bnf=cfg.bnf, advect=1, L=cfg.L, dx=cfg.dx, dt=cfg.dt,
            nn=cfg.nn_m3, gas_sigma=cfg.gas_sigma(), e_exc=(tab.e_exc if tab else 11.5),
            nu_max=(tab.nu_max(cfg.nn_m3) if tab else 0.0), xs_mode=cfg.xs_mode(), coll_model=cfg.coll_model,
            xs_table=self.xs_t, xs_emin=(tab.emin if tab else 0.01), xs_emax=(tab.emax if tab else 1000.0),
            flags=cfg.quirks, seed=cfg.seed, step=self.bigstep,
            step_ptr=self.step_dev if step_on_device else None)

    # --------------------------------------------------------------------------------- reference entry points
    def electron_kernel(self):
        """Push + collide the current particles; deposit and compaction are fused in
        (electron_kernel_numba.py:291-303 with post_processing_1D.py:40-68). The push
        clears the moments itself before it deposits."""
        p = self.params()
        p.flags |= _lib.CLEAR_MOMENTS
        K.seg_electron_kernel(p, self.A, self.B, self.E_push, self.status, self.seg_flags, self.ws,
                              moments=self.moments, n_pushed=self.particle_steps)
        self.A, self.B = self.B, self.A

    def post_processing(self):
        """Grid moments of the last step: (ne, ni_src, ns_src, nrg) device tensors
        (post_processing_1D.py:40-68 returns them as host arrays)."""
        return self.moments[0], self.moments[1], self.moments[2], self.moments[3]

    def bin_particles(self):
        K.seg_bin_particles(self.params(), self.A, self.edges[: self.nb - 1] if self.nb > 1 else self.edges[:0],
                            self.cfg.min_wt, self.perm, self.offsets, self.bin_counts, self.hw_counts, self.status,
                            self.ws)

    def _check_for_resampling(self):
        """Bin the particles and evaluate the trigger on the device (boltzmann.py:894-916);
        the sort by key runs only when resampling will (_do_resampling evaluates the same
        trigger again and does nothing when it is off)."""
        cfg = self.cfg
        K.seg_bin_particles(self.params(), self.A, self.edges[: self.nb - 1] if self.nb > 1 else self.edges[:0],
                            cfg.min_wt, self.perm, self.offsets, self.bin_counts, self.hw_counts, self.status,
                            self.ws, check=(self.targets, cfg.split_below, cfg.merge_at, self.need))

    def _do_resampling(self):
        cfg = self.cfg
        K.seg_resample(self.params(), self.A, self.app, self.B, self.nb, self.targets, self.max_ppc, cfg.min_wt,
                       cfg.split_below, cfg.merge_at, cfg.merge_keep, self.perm, self.offsets, self.bin_counts,
                       self.hw_counts, self.status, self.seg_flags, self.ws, need=self.need,
                       in_place=cfg.resample_in_place)
        if not cfg.resample_in_place:
            self.A, self.B = self.B, self.A

    def _repack_if_needed(self):
        """Spread the particles evenly again when the last push left a segment above
        half its capacity (decided on the device; through B and back into A in one
        launch, so the buffer roles stay fixed)."""
        K.seg_rebalance(self.A, self.B, self.status, self.ws, only_if=self.seg_flags, clear=self.seg_flags)

    def heavies_kernel_fluid(self):
        cfg = self.cfg
        K.heavies_kernel_fluid(self.N, cfg.dx, cfg.dt, cfg.mu_i, cfg.D_i, self.E, self.ni, self.Ji, self.brk)

    def EF_kernel(self):
        cfg = self.cfg
        K.EF_kernel(self.N, cfg.dx, cfg.eps0, cfg.V0, cfg.freq, 0.0, self.moments[0], self.ni, self.poisson_plan,
                    self.V, self.E, self.E_push if self.dtype == torch.float32 else None, t_dev=self.t)
        if self.dtype == torch.float64:
            self.E_push.copy_(self.E)

    def _grid_solves(self, advance=True):
        """Grid update, clock, ion fluid and Poisson (boltzmann.py:643-678) in one
        cooperative launch over ceil((N-1)/64) CTAs; the first solve (advance=False) is the
        Poisson alone."""
        cfg = self.cfg
        if not advance:
            self.EF_kernel()
            return
        f32 = self.dtype == torch.float32
        K.field_step_coop(self.N, cfg.dx, cfg.dt, cfg.mu_i, cfg.D_i, cfg.eps0, cfg.V0, cfg.freq, self.moments,
                          self.ni, self.Te, self.g2, self.t, self.step_dev, self.poisson_plan, self.V, self.E,
                          self.E_push if f32 else None, self.Ji, self.brk, ws=self.ws)
        if not f32:
            self.E_push.copy_(self.E)

    # --------------------------------------------------------------------------------- stepping
    def _step_body(self, resample):
        if self._host_io is not None:  # _copy_to_GPU (boltzmann.py:719-741)
            self.io[:self.io_in].copy_(self._host_io[:self.io_in], non_blocking=True)
        if resample:
            self._check_for_resampling()
            self._do_resampling()
        else:
            self._repack_if_needed()
        self.electron_kernel()
        if self._ion_rate is not None:
            K.ion_source_closure(self.nnodes, self._ion_rate, self.moments)
        self._grid_solves(advance=True)
        if self._host_io is not None:  # back_to_cpu (post_processing_1D.py:6-24)
            self._host_io.copy_(self.io, non_blocking=True)

    def step(self, use_graph=True):
        """One step of the hybrid loop (boltzmann.py:570-678). With ``use_graph`` a step
        kind (resample or not) runs eagerly the first time, so that every kernel is
        loaded and configured; after that each (kind, which buffer holds the particles)
        is captured into a CUDA graph once and replayed."""
        resample = (self.bigstep % self.cfg.resample_freq) == 0
        key = (resample, self.A is self._first_A())
        if use_graph and resample in self._kinds:
            gr = self._graphs.get(key) or self._capture_key(key)
            gr.replay()
            self._replayed.add(key)
            # the graph swaps A and B internally; mirror the swaps on the host side
            for _ in range(2 if resample and not self.cfg.resample_in_place else 1):
                self.A, self.B = self.B, self.A
        else:
            self._kinds.add(resample)
            self._step_body(resample)
        self.bigstep += 1

    def capture_all(self):
        """Capture the graphs of every step kind that has run once, for both buffer
        roles, so that no capture (which synchronises the device) falls inside a timed
        loop."""
        for resample in sorted(self._kinds):
            for first in (True, False):
                if (resample, first) not in self._graphs:
                    self._capture_key((resample, first))

    def graphs_warm(self):
        """True once every captured step graph has been replayed (a graph's first replay
        also uploads it to the device, a one-off cost)."""
        return all(k in self._replayed for k in self._graphs)

    def attach_host_io(self, host_block):
        """Make every step copy the first ``io_in`` values of a pinned host block (the
        reference's per-step [E, ne, ni, ns, Te], boltzmann.py:719-741) to the device
        before it runs and the whole grid block (those plus the moments) back after it,
        inside the step's graph. ``None`` detaches. Graphs are re-captured."""
        if host_block is not None:
            if not host_block.is_pinned() or host_block.numel() != self.io.numel() or \
                    host_block.dtype != torch.float64:
                raise ValueError(f"host block must be pinned float64 of {self.io.numel()} values")
        self._host_io = host_block
        self._graphs = {}

    def retune(self):
        """Time the push's CTA shapes on the current state (A is only read) and keep the
        fastest; the step graphs, which hold the kernel, are captured again."""
        if self.dtype != torch.float32:
            return
        best, times = K.autotune_seg_push(self.params(step_on_device=False), self.A, self.B, self.E_push,
                                          self.status, self.seg_flags, self.ws, self.moments)
        self.push_shape = {"shape": K.seg_push_shapes()[best], "ms": times}
        self._graphs = {}

    def _capture_key(self, key):
        resample, first = key
        swap = (self.A is self._first_A()) != first
        if swap:
            self.A, self.B = self.B, self.A
        g = self._capture(resample)
        if swap:
            self.A, self.B = self.B, self.A
        self._graphs[key] = g
        self._replayed.discard(key)
        return g

    def _first_A(self):
        if not hasattr(self, "_A0"):
            self._A0 = self.A
        return self._A0

    def _capture(self, resample):
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream())
        g = torch.cuda.CUDAGraph()
        saved = (self.A, self.B)
        with torch.cuda.stream(s):
            self._warm(resample)
        torch.cuda.current_stream().wait_stream(s)
        with torch.cuda.graph(g, stream=s, capture_error_mode="relaxed"):
            self._step_body(resample)
        self.A, self.B = saved
        return g

    def _warm(self, resample):
        """Allocate every workspace the step uses without running the step."""
        lib = _lib.load()
        nkeys = self.nnodes * self.nb
        self.ws.get("seg_push", lib.bz_seg_push_workspace_nodes(self.nnodes))
        self.ws.get("seg_rebalance", lib.bz_seg_repack_workspace(self.A.nseg))
        self.ws.get("field_coop", lib.bz_field_step_coop_workspace(self.N))
        if resample:
            self.ws.get("seg_bin", lib.bz_seg_bin_workspace(self.A.nseg, self.A.capacity))
            self.ws.get("seg_resample", lib.bz_seg_resample_workspace(self.A.nseg, self.A.capacity, nkeys))

    def grid_fields(self):
        """The grid fields the step loop averages over a cycle: ne (this step's deposit),
        ni, Te and E after the step."""
        return {"ne": self.moments[0], "ni": self.ni, "Te": self.Te, "E": self.E}

    def run(self, num_steps, name="", restart_cyclenum=0, use_graph=True, write=False, on_step=None):
        """The step loop (boltzmann.py:565-716), with cycle averages and, when ``write``,
        the reference's per-cycle output files. At every cycle's end the ion production
        total (g2, written as ionprod_total) starts again from zero, as the reference's
        loop resets it (boltzmann.py:713-714). ``on_step(solver)``, when given, is called
        after every step (before that step's averaging and output)."""
        spc = self.cfg.steps_per_cycle
        avg = CycleAverages(self.grid_fields())
        for _ in range(num_steps):
            self.step(use_graph=use_graph)
            if on_step is not None:
                on_step(self)
            if (self.bigstep % spc) != 0:
                avg.add(self.grid_fields())
            else:
                ca = avg.take(spc)
                if not self._brk_warned and int(self.brk.item()):
                    # the reference prints a warning and runs on (heavies_kernel_1D.py:44-46)
                    self._brk_warned = True
                    warnings.warn("an ion density went negative in the fluid update (break flag); the "
                                  "time step is too large for the densities and fields reached", RuntimeWarning)
                if write:
                    from . import io as bzio
                    bzio.data_write(self, name, self.bigstep // spc + restart_cyclenum, ca)
                self.g2.zero_()
        return self

    # --------------------------------------------------------------------------------- learned start-up
    def node_state(self):
        """Per deposit node: reduced field E/N (Td, from the face fields next to the node),
        mean electron energy (eV, from the last deposit), weight fractions in the 64 log
        energy bins of the learned start-up, and the RF phase."""
        from . import surrogate as S
        cfg = self.cfg
        E = np.abs(self.E.detach().cpu().numpy())  # V/cm at the N faces
        En = np.empty(self.nnodes)
        En[0], En[-1] = E[0], E[-1]
        En[1:-1] = 0.5 * (E[:-1] + E[1:])
        td = En * 100.0 / cfg.nn_m3 / 1e-21
        mom = self.moments.detach().cpu().numpy()
        mean = np.where(mom[0] > 0, mom[3] / np.maximum(mom[0], 1e-300), 0.0)
        h = torch.zeros(self.nnodes, S.EEDF_BINS, dtype=torch.float64, device=self.device)
        K.seg_eedf(self.params(step_on_device=False), self.A, h, S.EEDF_EMIN, S.EEDF_EMAX)
        h = h.cpu().numpy()
        f = h / np.maximum(h.sum(axis=1, keepdims=True), 1e-300)
        phase = 2.0 * math.pi * ((cfg.freq * float(self.t.item())) % 1.0)
        return td, mean, f, phase

    def learned_start(self, mlp, seed=None, closure=False, scale_to_mean=True):
        """Redraw every electron's velocity from the surrogate network's steady-state energy
        distribution for its node (features from ``node_state``), each node's energies scaled
        to the network's predicted mean energy unless ``scale_to_mean`` is False (in the
        benchmark's CCP the first 50 steps then averaged 0.8-1.4% below the periodic mean
        energy instead of 1.7-2.1%), then refresh the moments. Positions,
        weights and the field are unchanged; the plain step loop continues from here. With
        ``closure`` the ion source of the following steps is the network's ionization rate
        times the electron density (``set_ion_closure``) instead of the counted
        ionizations. Returns the network's per-node (eedf, k_exc, k_ion, mean energy)."""
        from . import surrogate as S
        td, mean, f, phase = self.node_state()
        out = S.learned_start(mlp, self.params(step_on_device=False), self.A, td, np.maximum(mean, 1e-3),
                              S.bin_fractions(f), phase, seed=self.cfg.seed + 7 if seed is None else seed,
                              device=self.device, scale_to_mean=scale_to_mean)
        self.moments.zero_()
        K.seg_deposit(self.params(step_on_device=False), self.A, self.moments)
        if closure:
            self.set_ion_closure(out[2])
        return out

    def set_ion_closure(self, k_ion=None):
        """Ion source from a rate closure: ni_src = k_ion n_gas dt ne per node (k_ion in m^3/s
        per deposit node, e.g. the learned start-up network's), replacing the counted
        ionizations of the push (post_processing_1D.py:50-55); None restores the counted
        source. The step graphs are captured again."""
        if k_ion is None:
            self._ion_rate = None
        else:
            k = np.broadcast_to(np.asarray(k_ion, dtype=np.float64), (self.nnodes,))
            self._ion_rate = torch.as_tensor(k * self.cfg.nn_m3 * self.cfg.dt, dtype=torch.float64,
                                             device=self.device).contiguous()
        self._graphs = {}

    # --------------------------------------------------------------------------------- diagnostics
    def kernel_launches(self, resample):
        """libbz kernels one step launches (torch's memset of the moments not counted).
        Every step: the push and the fused grid step (grid update, clock, ion fluid,
        Poisson) (2); a plain step adds the conditional rebalance (one cooperative
        kernel); a resampling step adds binning (segment totals, key offsets twice, keys, the
        resampling trigger, then per 8-bit radix pass a histogram, column sums, column scan
        and scatter, which sort nothing when the trigger is off), decide + apply (2) and
        either the placement of the appended particles with its conditional repack (2) or the
        repack of the survivors with them (1)."""
        passes = 2 if self.nnodes * self.nb >= 256 else 1
        tail = 2 if self.cfg.resample_in_place else 1
        return 2 + (5 + 4 * passes + 2 + tail if resample else 1) + (self._ion_rate is not None)

    def snapshot(self):
        """A device copy of the simulation state: the particles (the buffer that holds
        them and its counts), the grid block, the ion fluxes, the potential, the clock, the
        status words and the step index. The Philox step counter and the particle-step
        total are not part of it: a run restored from a snapshot draws new random numbers."""
        return {"first": self.A is self._first_A(), "bigstep": self.bigstep,
                "tensors": [t.clone() for t in self._state_tensors()]}

    def restore(self, snap):
        """Copy a snapshot back into the same device buffers (captured step graphs stay
        valid: their pointers do not change)."""
        if (self.A is self._first_A()) != snap["first"]:
            self.A, self.B = self.B, self.A
        for dst, src in zip(self._state_tensors(), snap["tensors"]):
            dst.copy_(src)
        self.bigstep = snap["bigstep"]

    def _state_tensors(self):
        return [self.A._buf, self.A.counts, self.io, self.E_push, self.V, self.Ji, self.g2, self.t, self.brk,
                self.status, self.seg_flags]

    def n(self):
        return self.A.n()

    def device_status(self):
        return int(self.status.item())

    def ne(self):
        return self.moments[0]
