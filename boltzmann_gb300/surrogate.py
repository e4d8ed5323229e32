"""Learned start-up: a small network that proposes each cell's (or swarm's) electron
energy distribution and rate closure, so that a run starts near its steady state.

The reference starts every run from the plain initial state, electrons at 1 eV
(boltzmann.py:271-312), and has no learned part; this module is the learned start-up of
the hybrid CCP that the benchmark asks for, built on the same kernels:

* training data: batched 0-D swarms (``SwarmEnsemble``) swept over E/N, and plain CCP
  runs, snapshot by snapshot: features of the current state, targets = the steady-state
  distribution and rate coefficients the run settles to;
* the network: ``SurrogateMLP``, 16 inputs -> 4 x 128 GELU -> 80 outputs, trained on the
  GPU by the library's own BF16 tensor-core forward and backward kernels and Adam
  (csrc/bz_mlp.cu), one C call per training step;
* the start-up: ``learned_start`` evaluates the network for every key (swarm or deposit
  node) and redraws the particles' velocities from the predicted distribution
  (``bz_seg_sample_energy``); the plain PIC-MCC run then continues from there and
  checks the surrogate.

Features (9 of BZ_MLP_IN = 16, the rest zero):
  0: log10(E/N in Td) / 3          1: log10(mean energy in eV) / 2
  2, 3: sin and cos of the RF phase (both 0 for a DC field: swarms)
  4..8: weight fractions in the energy bins [0,2), [2,6), [6,11.5), [11.5,15.76), >= 15.76 eV
Outputs (67 of BZ_MLP_OUT = 80):
  0..63: (log10(f_k + 1e-6) + 3) / 3, f_k the weight fraction in log bin k of 64 over
         0.01-100 eV
  64, 65: (log10(k + 1e-20) + 16.5) / 3.5, k the excitation and ionization rate
         coefficients in m^3/s
  66: log10(mean energy in eV) / 2 of the same steady state (the start-up can scale the
      drawn energies so that each key's mean is this output's: ``scale_to_mean``)
"""
from __future__ import annotations

import math
from typing import Optional, Sequence

import numpy as np
import torch

from . import _lib, kernels as K

NIN, NOUT, NPARAM = 16, 80, 62032
LAYERS = ((16, 128), (128, 128), (128, 128), (128, 128), (128, 80))  # (in, out)
EEDF_BINS, EEDF_EMIN, EEDF_EMAX = 64, 0.01, 100.0
BIN_EDGES5 = (2.0, 6.0, 11.5, 15.76)
F_FLOOR, K_FLOOR = 1e-6, 1e-20
N_FEAT, N_TGT = 9, EEDF_BINS + 3
I_MEAN = EEDF_BINS + 2


def eedf_centres():
    le = np.linspace(math.log(EEDF_EMIN), math.log(EEDF_EMAX), EEDF_BINS + 1)
    return np.exp(0.5 * (le[:-1] + le[1:]))


def bin_fractions(eedf):
    """[n, 64] weight fractions -> [n, 5] fractions in the five energy bins (each log bin
    counted in the bin of its centre)."""
    c = eedf_centres()
    b = np.searchsorted(np.asarray(BIN_EDGES5), c, side="right")
    f = np.zeros((len(eedf), 5))
    for k in range(5):
        f[:, k] = eedf[:, b == k].sum(axis=1)
    return f


def features(td, mean_e, phase, fr5):
    td = np.asarray(td, dtype=np.float64).reshape(-1)
    n = len(td)
    x = np.zeros((n, NIN), dtype=np.float32)
    x[:, 0] = np.log10(np.maximum(td, 1e-3)) / 3.0
    x[:, 1] = np.log10(np.maximum(np.broadcast_to(mean_e, (n,)), 1e-3)) / 2.0
    if phase is not None:  # DC (phase None): the zero vector
        ph = np.broadcast_to(np.asarray(phase, dtype=np.float64), (n,))
        x[:, 2] = np.sin(ph)
        x[:, 3] = np.cos(ph)
    x[:, 4:9] = np.broadcast_to(fr5, (n, 5))
    return x


def targets(eedf, k_exc, k_ion, mean_e=None):
    """Network targets; mean_e (eV) defaults to the distribution's own mean (eedf_mean)."""
    n = len(eedf)
    t = np.zeros((n, NOUT), dtype=np.float32)
    t[:, :EEDF_BINS] = (np.log10(np.asarray(eedf) + F_FLOOR) + 3.0) / 3.0
    t[:, EEDF_BINS] = (np.log10(np.maximum(k_exc, 0) + K_FLOOR) + 16.5) / 3.5
    t[:, EEDF_BINS + 1] = (np.log10(np.maximum(k_ion, 0) + K_FLOOR) + 16.5) / 3.5
    m = eedf_mean(eedf) if mean_e is None else np.broadcast_to(np.asarray(mean_e, dtype=np.float64), (n,))
    t[:, I_MEAN] = np.log10(np.maximum(m, 1e-3)) / 2.0
    return t


def decode(y):
    """Network outputs -> (eedf [n,64] normalised, k_exc, k_ion)."""
    y = np.asarray(y, dtype=np.float64)
    f = np.maximum(10.0 ** (3.0 * y[:, :EEDF_BINS] - 3.0) - F_FLOOR, 0.0)
    s = f.sum(axis=1, keepdims=True)
    f = np.where(s > 0, f / np.maximum(s, 1e-300), 1.0 / EEDF_BINS)
    kx = np.maximum(10.0 ** (3.5 * y[:, EEDF_BINS] - 16.5) - K_FLOOR, 0.0)
    ki = np.maximum(10.0 ** (3.5 * y[:, EEDF_BINS + 1] - 16.5) - K_FLOOR, 0.0)
    return f, kx, ki


def decode_mean(y):
    """Network outputs -> the predicted mean energy (eV) [n]."""
    return 10.0 ** (2.0 * np.asarray(y, dtype=np.float64)[:, I_MEAN])


def eedf_mean(eedf):
    """Mean energy (eV) of weight fractions in the 64 log bins, each bin log-uniform (the
    start-up's draw): sum_k f_k (e_k+1 - e_k) / ln(e_k+1 / e_k)."""
    le = np.linspace(math.log(EEDF_EMIN), math.log(EEDF_EMAX), EEDF_BINS + 1)
    e = np.exp(le)
    mk = (e[1:] - e[:-1]) / (le[1:] - le[:-1])
    return np.asarray(eedf, dtype=np.float64) @ mk


def output_weights(eedf_weight=1.0, rate_weight=1.0, mean_weight=1.0):
    w = np.zeros(NOUT, dtype=np.float32)
    w[:EEDF_BINS] = eedf_weight
    w[EEDF_BINS:I_MEAN] = rate_weight
    w[I_MEAN] = mean_weight
    return w


def init_params(seed, scale=1.0):
    """Uniform(-s, s) weights, s = scale sqrt(3 / fan_in), zero biases (float64)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM)
    o = 0
    for ni, no in LAYERS:
        s = scale * math.sqrt(3.0 / ni)
        p[o:o + ni * no] = rng.uniform(-s, s, ni * no)
        o += ni * no + no
    return p


class SurrogateMLP:
    """The network's FP32 parameters, their BF16 copies and the Adam state, on one GPU."""

    def __init__(self, device="cuda", seed=0, params: Optional[np.ndarray] = None):
        assert _lib.load().bz_mlp_param_count() == NPARAM
        self.device = device
        f32 = dict(dtype=torch.float32, device=device)
        p = init_params(seed) if params is None else np.asarray(params)
        self.prm = torch.as_tensor(p.astype(np.float32), device=device).contiguous()
        self.wb = torch.zeros(NPARAM, dtype=torch.int16, device=device)
        self.wt = torch.zeros(NPARAM, dtype=torch.int16, device=device)
        self.grad = torch.zeros(NPARAM, **f32)
        self.m = torch.zeros(NPARAM, **f32)
        self.v = torch.zeros(NPARAM, **f32)
        self.loss = torch.zeros(1, **f32)
        self.step = 0
        self.ws = K.Workspace(device)
        K.mlp_sync(self.prm, self.wb, self.wt)

    def params(self):
        return self.prm.detach().cpu().numpy().astype(np.float64)

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        x = x.to(device=self.device, dtype=torch.float32).contiguous()
        y = torch.empty(x.shape[0], NOUT, dtype=torch.float32, device=self.device)
        K.mlp_forward(self.wb, self.prm, x, y)
        return y

    def train(self, x, t, steps, batch=2048, lr=2e-3, lr_end=2e-5, weight_decay=0.0, seed=0, wcol=None,
              log_every=0):
        """Adam on minibatches drawn uniformly from (x, t) (device tensors [n, 16] and
        [n, 80]), cosine learning-rate decay from lr to lr_end. Returns the losses read
        every ``log_every`` steps (the mean minibatch loss since the previous read)."""
        x = x.to(device=self.device, dtype=torch.float32).contiguous()
        t = t.to(device=self.device, dtype=torch.float32).contiguous()
        wc = torch.as_tensor(output_weights() if wcol is None else wcol, dtype=torch.float32, device=self.device)
        hist = []
        self.loss.zero_()
        for s in range(steps):
            self.step += 1
            lr_s = lr_end + 0.5 * (lr - lr_end) * (1.0 + math.cos(math.pi * s / max(steps - 1, 1)))
            K.mlp_train_step(self.prm, self.grad, self.m, self.v, self.wb, self.wt, x, t, wc, batch, seed, self.step,
                             lr_s, self.loss, self.ws, weight_decay=weight_decay)
            if log_every and (s + 1) % log_every == 0:
                hist.append(float(self.loss.item()) / log_every)
                self.loss.zero_()
        return hist

    def evaluate(self, x, t, wcol=None):
        """Mean loss over (x, t)."""
        y = self.forward(x).double().cpu().numpy()
        tt = np.asarray(t.cpu().numpy() if torch.is_tensor(t) else t, dtype=np.float64)
        w = output_weights() if wcol is None else wcol
        return float(0.5 * np.sum(w * (y - tt) ** 2) / len(y))

    def predict(self, x):
        """(eedf [n,64], k_exc [n], k_ion [n]) for feature rows x [n,16]."""
        return decode(self.forward(torch.as_tensor(np.asarray(x, dtype=np.float32))).cpu().numpy())

    def predict_all(self, x):
        """(eedf [n,64], k_exc [n], k_ion [n], mean energy [n]) for feature rows x [n,16]."""
        y = self.forward(torch.as_tensor(np.asarray(x, dtype=np.float32))).cpu().numpy()
        return decode(y) + (decode_mean(y),)


# ------------------------------------------------------------------------------------ data from swarms
def swarm_state(ens):
    """(mean energy [S], eedf [S,64]) of an ensemble's current particles."""
    mom = ens.moments.cpu().numpy()
    mean = mom[3] / np.maximum(mom[0], 1e-300)
    return mean, ens.eedf(EEDF_BINS, EEDF_EMIN, EEDF_EMAX)


def swarm_dataset(td, counts, steps, snapshot_every, settle_fraction=0.5, seed=1, device="cuda", **kw):
    """Runs one ensemble of swarms at the reduced fields ``td`` (Td) and returns
    (X, T, info): a feature row per swarm per snapshot, and as its target the swarm's
    steady state (the EEDF averaged over the snapshots after ``settle_fraction`` of the
    run; rate coefficients averaged over the same steps)."""
    from .swarm import SwarmConfig, SwarmEnsemble
    td = np.asarray(td, dtype=np.float64)
    S = len(td)
    cfg = SwarmConfig(E_over_N_Td=tuple(float(v) for v in td), counts=tuple(int(c) for c in counts),
                      precision="float32", bin_edges=(4.0, 11.5), bin_fractions=(0.7, 0.2, 0.1), merge_at=3.0,
                      merge_keep=0.6, resample_every=10, seed=seed, **kw)
    ens = SwarmEnsemble(cfg, device=device)
    feats, means, eedfs = [], [], []
    n_snap = steps // snapshot_every
    settle = int(settle_fraction * n_snap)
    for k in range(n_snap):
        if k == settle:
            ens.reset_averages()
        ens.run(snapshot_every)
        mean, f = swarm_state(ens)
        feats.append(features(td, mean, None, bin_fractions(f)))
        means.append(mean)
        eedfs.append(f)
    f_ss = np.mean(eedfs[settle:], axis=0)
    kion, kexc = ens.rate_coefficients()
    tg = targets(f_ss, kexc, kion, np.mean(means[settle:], axis=0))
    X = np.concatenate(feats)
    T = np.concatenate([tg] * n_snap)
    # the initial state is a sample too (what the start-up sees)
    f0 = initial_eedf(cfg.Te_init_eV)
    X = np.concatenate([features(td, 1.5 * cfg.Te_init_eV, None, bin_fractions(f0[None, :])), X])
    T = np.concatenate([tg, T])
    info = {"td": td, "mean_series": np.array(means), "eedf_ss": f_ss, "k_exc": kexc, "k_ion": kion,
            "mean_ss": np.mean(means[settle:], axis=0), "status": ens.device_status()}
    return X, T, info


def initial_eedf(Te_eV=1.0):
    """Weight fractions of an isotropic Maxwellian of temperature Te in the 64 log bins."""
    le = np.linspace(math.log(EEDF_EMIN), math.log(EEDF_EMAX), EEDF_BINS + 1)
    e = np.exp(le)
    # chi-square with 3 degrees of freedom in 2 e / Te: CDF from the regularised gamma P(3/2, e/Te)
    from scipy.special import gammainc
    c = gammainc(1.5, e / Te_eV)
    f = np.diff(c)
    return f / f.sum()


def eedf_cdf(eedf):
    c = np.cumsum(np.asarray(eedf, dtype=np.float64), axis=1)
    c /= np.maximum(c[:, -1:], 1e-300)
    c[:, -1] = 1.0
    return c


def learned_start(mlp: SurrogateMLP, params, segs, td, mean_e, fr5, phase=None, seed=11, device="cuda",
                  scale_to_mean=False):
    """Redraw the velocities of every particle from the network's steady-state EEDF for
    its key (swarm / deposit node): features per key from (td, mean_e, fr5, phase; phase
    None for a DC field). With ``scale_to_mean`` the energies are scaled so that each key's
    mean is the network's predicted mean energy (the CCP solver's start-up does so; on the
    benchmark's held-out swarms it put more starts beyond 5% of the settled mean energy, so
    the swarms' start-up does not). Returns (eedf, k_exc, k_ion, mean energy) per key."""
    x = features(td, mean_e, phase, fr5)
    f, kx, ki, em = mlp.predict_all(x)
    cdf = torch.as_tensor(eedf_cdf(f), dtype=torch.float64, device=device)
    scale = None
    if scale_to_mean:
        scale = torch.as_tensor(np.clip(em / np.maximum(eedf_mean(f), 1e-6), 0.5, 2.0), dtype=torch.float64,
                                device=device)
    K.seg_sample_energy(params, segs, cdf, EEDF_EMIN, EEDF_EMAX, seed, scale=scale)
    return f, kx, ki, em


def steps_to_steady(series, final, tol=0.02, window=5):
    """Index of the first sample at which the moving average of the last ``window``
    samples of ``series`` [n, S] is within tol (relative) of ``final`` [S] (the index of
    the window's last sample); n when it never is."""
    s = np.asarray(series, dtype=np.float64)
    n = len(s)
    k = np.ones(window) / window
    out = np.full(s.shape[1], n)
    for j in range(s.shape[1]):
        ma = np.convolve(s[:, j], k, mode="valid")
        ok = np.nonzero(np.abs(ma / final[j] - 1.0) <= tol)[0]
        if len(ok):
            out[j] = ok[0] + window - 1
    return out


def swarm_relaxation(td, counts, steps, chunk, mlp: Optional[SurrogateMLP] = None, seed=5, device="cuda", **kw):
    """Mean energy per swarm averaged over consecutive chunks of ``chunk`` steps
    ([steps // chunk, S]), from the plain start (1 eV Maxwellian) or, with ``mlp``, from
    the learned start; also returns the ensemble."""
    from .swarm import SwarmConfig, SwarmEnsemble
    td = np.asarray(td, dtype=np.float64)
    cfg = SwarmConfig(E_over_N_Td=tuple(float(v) for v in td), counts=tuple(int(c) for c in counts),
                      precision="float32", bin_edges=(4.0, 11.5), bin_fractions=(0.7, 0.2, 0.1), merge_at=3.0,
                      merge_keep=0.6, resample_every=10, seed=seed, **kw)
    ens = SwarmEnsemble(cfg, device=device)
    if mlp is not None:
        f0 = initial_eedf(cfg.Te_init_eV)
        learned_start(mlp, ens.params(step_on_device=False), ens.A, td, 1.5 * cfg.Te_init_eV,
                      bin_fractions(f0[None, :]), seed=seed + 1000, device=device)
    out = []
    for _ in range(steps // chunk):
        ens.reset_averages()
        ens.run(chunk)
        out.append(ens.mean_energy())
    return np.array(out), ens


# ------------------------------------------------------------------------------------ data from plain CCP runs
def ccp_dataset(cfg, cycles, snaps_per_cycle=8, settle_cycles=None, min_density=1e-3, density_repeat=8,
                device="cuda"):
    """Runs a plain CCP (``BoltzmannGB300``) for ``cycles`` RF cycles and returns (X, T, info):
    per deposit node and snapshot (``snaps_per_cycle`` per cycle), the features of the
    current state; as targets, the node's energy distribution at the same RF phase averaged
    over the last ``settle_cycles`` cycles, and its ionization and excitation rate
    coefficients averaged over those cycles. Nodes whose settled density is below
    ``min_density`` of the largest are left out."""
    import dataclasses
    from .solver import BoltzmannGB300
    cfg = dataclasses.replace(cfg, quirks=cfg.quirks | _lib.MOMENT_EXCITATION)
    sv = BoltzmannGB300(cfg, device=device)
    nn_ = sv.nnodes
    spc = cfg.steps_per_cycle
    every = max(spc // snaps_per_cycle, 1)
    settle_n = settle_cycles or max(cycles // 2, 1)
    settle = cycles - settle_n
    snaps = []
    f_acc = np.zeros((snaps_per_cycle, nn_, EEDF_BINS))
    m_acc = np.zeros((snaps_per_cycle, nn_))
    ev = torch.zeros(3, nn_, dtype=torch.float64, device=device)
    for c in range(cycles):
        for k in range(snaps_per_cycle):
            td, mean, f, phase = sv.node_state()
            snaps.append((k, features(td, np.maximum(mean, 1e-3), phase, bin_fractions(f))))
            if c >= settle:
                f_acc[k] += f
                m_acc[k] += mean
            for _ in range(every):
                sv.step()
                if c >= settle:
                    ev[0].add_(sv.moments[1])
                    ev[1].add_(sv.moments[2])
                    ev[2].add_(sv.moments[0])
    f_ss = f_acc / settle_n
    m_ss = m_acc / settle_n
    e = ev.cpu().numpy()
    den = np.maximum(e[2], 1e-300) * cfg.nn_m3 * cfg.dt
    k_ion, k_exc = e[0] / den, e[1] / den
    keep = e[2] >= min_density * e[2].max()
    # each node's rows repeated in proportion to its electron density (1 .. density_repeat):
    # the fit then weighs nodes as the gap's energy balance does
    rep = np.maximum(1, np.round(density_repeat * e[2] / e[2].max())).astype(int)[keep]
    X = np.concatenate([np.repeat(x[keep], rep, axis=0) for _, x in snaps])
    T = np.concatenate([np.repeat(targets(f_ss[k][keep], k_exc[keep], k_ion[keep], np.maximum(m_ss[k][keep], 1e-3)),
                                  rep, axis=0) for k, _ in snaps])
    info = {"nodes": np.nonzero(keep)[0], "eedf_ss": f_ss, "mean_ss": m_ss, "k_ion": k_ion, "k_exc": k_exc,
            "status": sv.device_status(), "n_end": sv.n()}
    return X, T, info


def steps_to_periodic(series, period, tol=0.02, window=5):
    """Index of the first sample of the first period of ``series`` (1-D, at least two
    periods long) from which the moving average (``window`` samples) of the ratio to the
    same phase one period later is within tol of 1; ``period`` when it never is."""
    s = np.asarray(series, dtype=np.float64)
    r = s[:period] / s[period:2 * period]
    ma = np.convolve(r, np.ones(window) / window, mode="valid")
    ok = np.nonzero(np.abs(ma - 1.0) <= tol)[0]
    return int(ok[0] + window - 1) if len(ok) else period


def ccp_relaxation(cfg, steps, chunk, mlp: Optional[SurrogateMLP] = None, device="cuda", closure=False,
                   ion_flux=False, redraw_after=0):
    """Mean electron energy of a CCP (weight-averaged over the whole gap) per chunk of
    ``chunk`` steps, from the plain start or, with ``mlp``, the learned start (with
    ``closure``, its ion source from the network's rate closure; with ``redraw_after`` > 0
    the learned start is applied once more after that many chunks, from the state the
    fields have reached by then); also returns the solver.
    With ``ion_flux`` it returns (energies, ion fluxes, solver), the ion flux per chunk being
    the mean of |Ji| at the two electrodes (heavies_kernel_1D.py:37-38)."""
    from .solver import BoltzmannGB300
    sv = BoltzmannGB300(cfg, device=device)
    if mlp is not None:
        sv.learned_start(mlp, closure=closure)
    acc = torch.zeros(3, dtype=torch.float64, device=device)
    out, flux = [], []
    for c in range(steps // chunk):
        if mlp is not None and redraw_after and c == redraw_after:
            sv.learned_start(mlp, closure=closure)
        acc.zero_()
        for _ in range(chunk):
            sv.step()
            acc[0].add_(sv.moments[0].sum())
            acc[1].add_(sv.moments[3].sum())
            acc[2].add_(sv.Ji[0].abs() + sv.Ji[-1].abs())
        a = acc.cpu().numpy()
        out.append(a[1] / max(a[0], 1e-300))
        flux.append(0.5 * a[2] / chunk)
    if ion_flux:
        return np.array(out), np.array(flux), sv
    return np.array(out), sv
