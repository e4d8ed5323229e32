"""CPU checks of the surrogate network's oracle and host logic: the float64 network's
analytic gradient against central finite differences, the bfloat16 rounding, and the
feature / target encodings of the learned start-up."""
import math

import numpy as np

from boltzmann_gb300 import surrogate as S
from oracle import mlp as O


def small_case(seed, n=7):
    rng = np.random.default_rng(seed)
    p = S.init_params(seed) + rng.normal(0, 0.05, S.NPARAM)
    x = np.zeros((n, 16))
    x[:, :9] = rng.uniform(-1, 1, (n, 9))
    t = rng.normal(0, 1, (n, 80))
    return p, x, t


def test_layout_matches_the_library_constants():
    assert O.NPARAM == S.NPARAM == 62032
    assert [O.dims(l) for l in range(O.NL)] == list(S.LAYERS)


def test_oracle_gradient_matches_finite_differences():
    p, x, t = small_case(0)
    w = S.output_weights()
    _, g = O.backward(p, x, t, w, exact=True)
    rng = np.random.default_rng(1)
    for i in rng.choice(S.NPARAM, 40, replace=False):
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        num = (O.backward(pp, x, t, w, exact=True)[0] - O.backward(pm, x, t, w, exact=True)[0]) / (2 * h)
        assert abs(g[i] - num) <= 1e-5 * max(abs(num), 1e-3), (i, g[i], num)


def test_bf16_round_to_nearest_even():
    one = 1.0
    ulp = 2.0 ** -7  # bfloat16 spacing at 1
    v = np.array([one, one + ulp / 2, one + 1.5 * ulp, one + ulp / 2 + 2 ** -20, -3.0, 0.0])
    r = O.bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0                 # tie to even
    assert r[2] == one + 2 * ulp       # tie to even (odd neighbour below)
    assert r[3] == one + ulp           # above the tie
    assert r[4] == -3.0 and r[5] == 0.0


def test_bf16_network_is_close_to_the_exact_one():
    p, x, t = small_case(2, n=64)
    w = S.output_weights()
    y, _ = O.forward(p, x)
    y_x, _ = O.forward(p, x, exact=True)
    assert np.linalg.norm(y - y_x) / np.linalg.norm(y_x) < 5e-2
    _, g = O.backward(p, x, t, w)
    _, g_x = O.backward(p, x, t, w, exact=True)
    assert np.linalg.norm(g - g_x) / np.linalg.norm(g_x) < 5e-2


def test_adam_oracle_first_step_moves_by_lr():
    g = np.linspace(-1, 1, S.NPARAM)
    g[g == 0] = 1e-3
    p, m, v = O.adam(np.zeros(S.NPARAM), g, np.zeros(S.NPARAM), np.zeros(S.NPARAM), 1, 1e-3)
    np.testing.assert_allclose(p, -1e-3 * np.sign(g), rtol=1e-4, atol=1e-6)  # eps matters where |g| ~ 1e-5


def test_encodings_round_trip():
    rng = np.random.default_rng(3)
    f = rng.dirichlet(np.ones(S.EEDF_BINS), 5)
    kx = 10.0 ** rng.uniform(-18, -14, 5)
    ki = 10.0 ** rng.uniform(-18, -14, 5)
    t = S.targets(f, kx, ki)
    f2, kx2, ki2 = S.decode(t)
    np.testing.assert_allclose(f2, f, rtol=2e-3, atol=1e-6)
    np.testing.assert_allclose(kx2, kx, rtol=1e-5)
    np.testing.assert_allclose(ki2, ki, rtol=1e-5)
    np.testing.assert_allclose(S.decode_mean(t), S.eedf_mean(f), rtol=1e-5)  # default: the distribution's mean
    m = rng.uniform(0.5, 20.0, 5)
    np.testing.assert_allclose(S.decode_mean(S.targets(f, kx, ki, m)), m, rtol=1e-5)
    assert np.all(t[:, 67:] == 0)
    w = S.output_weights()
    assert w[:67].min() > 0 and np.all(w[67:] == 0)


def test_features_and_bin_fractions():
    f0 = S.initial_eedf(1.0)
    assert abs(f0.sum() - 1) < 1e-12
    c = S.eedf_centres()
    assert abs((f0 * c).sum() - 1.5) < 0.05  # <e> = 3/2 Te
    assert abs(S.eedf_mean(f0[None, :])[0] - 1.5) < 0.02
    fr = S.bin_fractions(f0[None, :])
    assert fr.shape == (1, 5) and abs(fr.sum() - 1) < 1e-12
    assert fr[0, 0] > 0.7  # most of a 1 eV Maxwellian is below 2 eV
    x = S.features([100.0, 10.0], 3.0, math.pi / 2, fr)
    assert x.shape == (2, 16) and x.dtype == np.float32
    np.testing.assert_allclose(x[:, 0], [2 / 3, 1 / 3], rtol=1e-6)
    np.testing.assert_allclose(x[:, 2:4], [[1, 0], [1, 0]], atol=1e-7)
    assert np.all(x[:, 9:] == 0)
    assert np.all(S.features([50.0], 3.0, None, fr)[:, 2:4] == 0)  # DC: no phase
    cdf = S.eedf_cdf(np.vstack([f0, f0]))
    assert np.all(np.diff(cdf, axis=1) >= 0) and np.all(cdf[:, -1] == 1.0)


def test_steps_to_steady():
    n = 100
    t = np.arange(n)
    fast = 5.0 + 0.0 * t
    slow = 5.0 - 4.0 * np.exp(-t / 10.0)
    s = S.steps_to_steady(np.stack([fast, slow], 1), np.array([5.0, 5.0]), tol=0.02, window=1)
    assert s[0] == 0
    # 4 exp(-t/10) <= 0.1  <=>  t >= 10 ln 40 = 36.9
    assert s[1] == 37
    s5 = S.steps_to_steady(np.stack([fast, slow], 1), np.array([5.0, 5.0]), tol=0.02, window=5)
    assert s5[0] == 4 and 37 < s5[1] < 42
    never = S.steps_to_steady(np.stack([slow], 1), np.array([7.0]), tol=0.02)
    assert never[0] == n


def test_steps_to_periodic():
    p = 40
    k = np.arange(3 * p)
    periodic = 5.0 + 0.5 * np.sin(2 * np.pi * k / p)
    assert S.steps_to_periodic(periodic, p, window=1) == 0
    relax = periodic - 4.0 * np.exp(-k / 5.0)
    s = S.steps_to_periodic(relax, p, window=1)
    assert 10 < s < 25
    assert S.steps_to_periodic(periodic * (1 + 0.5 * (k < p)), p) == p
