"""The learned start-up against the plain one: a network trained on swarm sweeps (the
library's own BF16 training kernels) proposes each swarm's steady-state energy
distribution; swarms started from it reach their steady mean energy (within 2%) in a
fraction of the steps the plain 1 eV start needs. Held-out reduced fields, same seeds and
particle counts for both starts; the plain run judges the steady state."""
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
