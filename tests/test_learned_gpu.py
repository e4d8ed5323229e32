"""The learned start-up against the plain one: a network trained on swarm sweeps (the
library's own BF16 training kernels) proposes each swarm's steady-state energy
distribution; swarms started from it reach their steady mean energy (within 2%) in a
fraction of the steps the plain 1 eV start needs. Held-out reduced fields, same seeds and
particle counts for both starts; the plain run defines the steady state."""
import math

import numpy as np
import pytest
import torch

from boltzmann_gb300 import surrogate as S

pytestmark = pytest.mark.gpu


def trained_surrogate():
    rng = np.random.default_rng(0)
    td = np.exp(rng.uniform(math.log(30.0), math.log(1000.0), 256))
    X, T, info = S.swarm_dataset(td, [10_000] * 256, steps=24_000, snapshot_every=300)
    assert info["status"] == 0
    mlp = S.SurrogateMLP(seed=0)
    hist = mlp.train(torch.as_tensor(X), torch.as_tensor(T), steps=3000, batch=2048, log_every=1000)
    assert hist[-1] < 0.5 * hist[0]
    return mlp, info


def test_learned_start_reaches_steady_state_sooner():
    mlp, _ = trained_surrogate()
    # 150-1000 Td: the plain start settles within the run (slower below, ~1e4 steps at 150 Td)
    td = np.exp(np.random.default_rng(7).uniform(math.log(150.0), math.log(1000.0), 16))
    counts = [30_000] * len(td)
    steps, chunk = 20_000, 100
    plain, ep = S.swarm_relaxation(td, counts, steps, chunk)
    learned, el = S.swarm_relaxation(td, counts, steps, chunk, mlp=mlp)
    assert ep.device_status() == 0 and el.device_status() == 0
    tail = int(0.6 * len(plain))
    final = 0.5 * (plain[tail:].mean(axis=0) + learned[tail:].mean(axis=0))
    # the two starts settle to the same state
    np.testing.assert_allclose(learned[tail:].mean(axis=0), plain[tail:].mean(axis=0), rtol=0.03)
    kp = S.steps_to_steady(plain, final) * chunk
    kl = S.steps_to_steady(learned, final) * chunk
    assert np.median(kl) <= 0.3 * np.median(kp), (kp, kl)
    # the learned start is already within 5% for most swarms
    assert np.mean(np.abs(learned[0] / final - 1) < 0.05) >= 0.75


def test_learned_start_of_the_ccp():
    """A network trained on a plain CCP run (and the swarm sweep) starts a new CCP run
    (another seed) near its periodic electron energy: the plain 1 eV start needs a quarter
    of an RF cycle to heat up. Measured with this small training set (3000 Adam steps):
    plain 19 chunks, learned 9 (0.47x); the benchmark's network (2e4 steps, 2e5 rows)
    reaches 0.22x."""
    from boltzmann_gb300 import config as C
    kw = dict(ne_uniform=1e9, in_dt=4000.0, steps_per_cycle=4000, num_particles=1_000_000)
    Xc, Tc, info = S.ccp_dataset(C.ccp_256(**kw), cycles=2, snaps_per_cycle=16, settle_cycles=1)
    assert info["status"] == 0 and len(Xc) > 0
    rng = np.random.default_rng(0)
    td = np.exp(rng.uniform(math.log(30.0), math.log(1000.0), 128))
    Xs, Ts, _ = S.swarm_dataset(td, [10_000] * 128, steps=12_000, snapshot_every=300)
    mlp = S.SurrogateMLP(seed=0)
    mlp.train(torch.as_tensor(np.concatenate([Xs, Xc])), torch.as_tensor(np.concatenate([Ts, Tc])), steps=3000,
              batch=4096)
    cfg = C.ccp_256(**dict(kw, seed=9))
    per, chunk = 4000 // 50, 50
    plain, sp = S.ccp_relaxation(cfg, 8000, chunk)
    learned, sl = S.ccp_relaxation(cfg, 8000, chunk, mlp=mlp)
    closure, sc = S.ccp_relaxation(cfg, 8000, chunk, mlp=mlp, closure=True)
    assert sp.device_status() == 0 and sl.device_status() == 0 and sc.device_status() == 0
    # the same periodic state in the second cycle
    np.testing.assert_allclose(learned[per:].mean(), plain[per:].mean(), rtol=0.03)
    kp = S.steps_to_periodic(plain, per)
    kl = S.steps_to_periodic(learned, per)
    kc = S.steps_to_periodic(closure, per)
    print("CCP chunks to the periodic state: plain", kp, "learned", kl, "with the rate closure", kc, "first chunk",
          plain[0], learned[0], "periodic", plain[per:].mean(), closure[per:].mean())
    assert kl <= 0.6 * kp, (kp, kl)
    # the network's ion-source rate closure: no slower, and the same periodic energy within 2%
    assert kc <= 0.6 * kp, (kp, kc)
    assert abs(closure[per:].mean() / plain[per:].mean() - 1) < 0.02
    assert abs(learned[0] / plain[per] - 1) < 0.15  # within 15% of the periodic value at once
    assert abs(plain[0] / plain[per] - 1) > 0.5     # the plain start is far from it


def test_energy_redraw_follows_the_tabulated_distribution():
    """bz_seg_sample_energy: per key, the drawn energies follow the tabulated distribution
    (the log-bin fractions to sampling error) times the key's scale; isotropic directions;
    positions and weights untouched."""
    from boltzmann_gb300 import _lib, kernels as K
    nk, per = 4, 100_000
    n = nk * per
    x = np.repeat(np.arange(nk, dtype=np.float64), per)
    w = np.full(n, 2.0)
    seg = K.SegmentSet(-(-n // 2048), 2048, torch.float32)
    seg.load(x, np.zeros(n), np.zeros(n), np.zeros(n), w)
    f = np.stack([S.initial_eedf(1.0), S.initial_eedf(3.0), S.initial_eedf(10.0), np.full(64, 1 / 64)])
    scale = np.array([1.0, 2.0, 0.5, 1.0])
    p = K.make_params(n_faces=nk, n_nodes=nk, bnf=1, advect=_lib.ADVECT_ENSEMBLE, L=float(nk), dx=1.0, dt=1e-12,
                      nn=3.22e22)
    K.seg_sample_energy(p, seg, torch.as_tensor(S.eedf_cdf(f), device="cuda"), S.EEDF_EMIN, S.EEDF_EMAX, 5,
                        scale=torch.as_tensor(scale, device="cuda"))
    o = seg.to_numpy()
    assert np.array_equal(np.sort(o["x"]), x) and np.all(o["w"] == 2.0)
    e = 0.5 * 9.10938e-31 * 6.241509e18 * (o["vx"] ** 2 + o["vy"] ** 2 + o["vz"] ** 2)
    key = o["x"].astype(int)
    for k in range(nk):
        ek = e[key == k]
        np.testing.assert_allclose(ek.mean(), S.eedf_mean(f[k:k + 1])[0] * scale[k], rtol=0.01)
        # the bin fractions of the unscaled energies
        h = np.histogram(np.log(ek / scale[k]), bins=np.linspace(np.log(S.EEDF_EMIN), np.log(S.EEDF_EMAX), 65))[0]
        assert 0.5 * np.abs(h / len(ek) - f[k]).sum() < 0.03  # sampling noise of 1e5 draws in 64 bins: ~0.01
        sp = np.sqrt(o["vx"] ** 2 + o["vy"] ** 2 + o["vz"] ** 2)[key == k]
        assert abs((o["vz"][key == k] / sp).mean()) < 0.01
