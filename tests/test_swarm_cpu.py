"""0-D swarm ensemble on the CPU: the oracle's ensemble mode (x holds the swarm index)
against single-swarm runs, the per-key resampling targets, and the swarm configurations."""
import math

import numpy as np
import pytest

from boltzmann_gb300 import swarm, xsec
from oracle import oracle as O


def _case(S=4, per=1500, seed=2):
    rng = np.random.default_rng(seed)
    n = S * per
    x = np.repeat(np.arange(S, dtype=np.float64), per)
    v = rng.normal(0, 1.5e6, (n, 3))
    w = np.ones(n)
    E = np.array([1e-21 * td * 3.22e22 / 100 for td in np.geomspace(30, 900, S)])  # V/cm
    return x, v, w, E


def _params(S, advect, seed=3, moment_exc=0, dt=1e-12):
    tab = xsec.analytic_argon(2000)
    nn = 3.22e22
    p = O.make_params(S, L=float(S), bnf=1, dt=dt, nn=nn, advect=advect, rng_mode=1, precision=64, seed=seed,
                      step=5, gas_sigma=250.0, xs_table=tab.nsigma(nn), xs_emin=tab.emin, xs_emax=tab.emax,
                      e_exc=tab.e_exc, moment_exc=moment_exc)
    p.n_nodes = S  # one node per swarm
    p.dx = 1.0
    return p


def test_oracle_ensemble_equals_single_swarms():
    """Ensemble mode gives every swarm exactly what a lone 0-D swarm in that swarm's field
    gives (same Philox slots), and deposits each swarm into its own node."""
    S = 4
    x, v, w, E = _case(S)
    n = len(x)
    d, t = O.soa_to_aos(x, v[:, 0], v[:, 1], v[:, 2], w, cap=3 * n)
    nni = O.push(_params(S, 2), d, t, n, E)
    assert nni > 0
    mom = O.deposit(_params(S, 2), d, t, n + nni)
    for s in range(S):
        d0, t0 = O.soa_to_aos(x, v[:, 0], v[:, 1], v[:, 2], w, cap=3 * n)
        p0 = _params(S, 0)
        p0.n_faces = 1
        O.push(p0, d0, t0, n, np.array([E[s]]))
        sel = np.nonzero(x == s)[0]
        np.testing.assert_array_equal(d[sel, 3:6], d0[sel, 3:6])
        np.testing.assert_array_equal(t[sel, 3], t0[sel, 3])
        # this swarm's survivors and children land in node s
        ch = n + np.nonzero(d[n:n + nni, 0] == s)[0]
        rows = np.concatenate([sel, ch])
        assert mom[0, s] == pytest.approx(t[rows, 0].sum(), rel=1e-12)
        assert mom[3, s] == pytest.approx((t[rows, 0] * t[rows, 3]).sum(), rel=1e-12)


def test_oracle_excitation_moment():
    S = 3
    x, v, w, E = _case(S, per=3000, seed=5)
    v *= 2.5  # ~15 eV: excitations happen
    n = len(x)
    d, t = O.soa_to_aos(x, v[:, 0], v[:, 1], v[:, 2], w, cap=3 * n)
    p = _params(S, 2, moment_exc=1, dt=2e-10)
    nni = O.push(p, d, t, n, E)
    exc = t[:n, 2].copy()
    mom, _ = O.post(p, d, t, n + nni)
    assert exc.sum() > 10
    for s in range(S):
        assert mom[2, s] == pytest.approx(exc[x == s].sum())


def test_oracle_per_key_targets():
    """bit 4: targets[cell*nb + bin]; a cell whose own target is small merges, one whose
    target is large is left alone."""
    S, per = 2, 4000
    rng = np.random.default_rng(7)
    x = np.repeat(np.arange(S, dtype=np.float64), per)
    v = rng.normal(0, 3e5, (S * per, 3))
    w = np.ones(S * per)
    p = _params(S, 2)
    counts, lists = O.bin_particles(p, x, v[:, 0], v[:, 1], v[:, 2], w, [], 10 * per)
    assert list(counts[0]) == [per, per]
    T = np.array([1000, 4000], dtype=np.int64)  # swarm 0 holds 4x its target, swarm 1 exactly it
    d, t = O.soa_to_aos(x, v[:, 0], v[:, 1], v[:, 2], w, cap=4 * S * per)
    u = np.random.default_rng(1).random(10000)
    na, used = O.resample(p, d, t, S * per, 1, T, 0.1, 10 * T, counts, lists, u, flags=0x10)
    assert na == int(0.6 * 1000) + per
    assert used == int(0.6 * 1000)
    np.testing.assert_allclose(t[:na, 0][d[:na, 0] == 0].sum(), per, rtol=1e-12)  # weight conserved


def test_swarm_configs():
    c = swarm.swarm_100td()
    assert c.n_swarms == 1 and c.counts == (100_000,) and c.precision == "float64" and c.merge_at == 2.0
    assert list(c.targets()) == [100_000]
    e = swarm.ensemble_512(seed=0)
    assert e.n_swarms == 512 and e.nbins == 3
    td, cnt = np.array(e.E_over_N_Td), np.array(e.counts)
    assert td.min() >= 10 and td.max() <= 1000 and cnt.min() >= 10_000 and cnt.max() <= 200_000
    assert 4e4 < cnt.mean() < 9e4  # log-uniform on [1e4, 2e5]: mean ~6.3e4
    tg = e.targets().reshape(512, 3)
    np.testing.assert_array_equal(tg[:, 0], (0.7 * cnt).astype(int))
    assert math.isclose(e.E_over_N_Td[0], swarm.ensemble_512(seed=0).E_over_N_Td[0])
