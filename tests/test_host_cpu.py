"""Host-side logic on the CPU: cross-section tables, the reference's file format, run
configuration, and the OpenMP CPU baseline against the serial oracle."""
import math

import numpy as np
import pytest

from boltzmann_gb300 import config, io as bzio, xsec
from oracle import oracle as O


def test_analytic_argon_values():
    t = xsec.analytic_argon(2000)
    e = t.energies()
    assert e[0] == pytest.approx(0.01) and e[-1] == pytest.approx(1000.0)
    el, ex, io = t.sigma
    k = np.searchsorted(e, 1.0)
    assert el[k] == pytest.approx(1e-19 * e[k] ** 0.3)
    assert el.max() == pytest.approx(1.5e-19)  # cap
    assert np.all(ex[e <= 11.5] == 0) and np.all(io[e <= 15.76] == 0)
    k = np.searchsorted(e, 40.0)
    assert io[k] == pytest.approx(3e-20 * math.log(e[k] / 15.76) / (e[k] / 15.76))
    assert ex[k] == pytest.approx(3e-21 * math.log(e[k] / 11.5) / (e[k] / 11.5))


def test_reference_fit_table_matches_oracle_fits():
    """The tabulated reference fits against the fits evaluated by the oracle (its push at
    one particle with P forced by a tiny dt would be indirect); compare the vectorised
    Python fit with the C restatement through the collision probability instead."""
    e = np.geomspace(0.01, 500, 4000)
    el, io = xsec.reference_fit_sigmas(e)
    assert np.all(np.isfinite(el)) and np.all(el > 0)
    assert np.all(io[e < 15.76] == 0) and np.all(io[e > 15.8] > 0)
    # continuity is not guaranteed by the fits; the table interpolates them to 1e-3 away
    # from the piece edges and the ionization threshold
    tab = xsec.reference_fits(8000)
    te = tab.energies()
    el_t, io_t = xsec.reference_fit_sigmas(te)
    np.testing.assert_allclose(tab.sigma[0], el_t)
    np.testing.assert_allclose(tab.sigma[2], io_t)


def test_read_lxcat_text():
    text = """
ELASTIC
Ar
 1.36e-5
-----------------------------
 0.0   7.5e-20
 1.0   1.5e-20
 100.0 1.0e-19
-----------------------------
EXCITATION
Ar -> Ar*
 11.5
-----------------------------
 11.5 0.0
 20.0 1.0e-21
 100.0 2.0e-21
-----------------------------
IONIZATION
Ar -> Ar^+
 15.76
-----------------------------
 15.76 0.0
 100.0 3.0e-20
-----------------------------
"""
    t = xsec.read_lxcat(text, n=500, emin=0.01, emax=1000.0)
    e = t.energies()
    assert t.e_exc == pytest.approx(11.5)
    k = np.searchsorted(e, 50.0)
    assert t.sigma[2, k] == pytest.approx(np.interp(e[k], [15.76, 100.0], [0, 3e-20]))
    assert t.sigma[1, np.searchsorted(e, 5.0)] == 0.0
    assert t.sigma[0, -1] == pytest.approx(1.0e-19)  # held beyond the table
    assert np.all(t.nsigma(1e22) == (t.sigma * 1e22).astype(np.float32))


def test_reference_file_format_roundtrip(tmp_path):
    name = str(tmp_path / "case_")
    rng = np.random.default_rng(0)
    x, vx, vy, vz = rng.random((4, 100))
    w = rng.random(100)
    w[::7] = 0.0
    bzio.write_particles(name, 3, x, vx, vy, vz, w)
    # data_write_1D.py: headerless little-endian float64, one file per column
    raw = np.fromfile(name + "e_x0_cycle3_mpi0.dat", dtype="<f8")
    np.testing.assert_array_equal(raw, x)
    rx, rvx, rvy, rvz, rw = bzio.read_particles(name, 3)
    keep = w != 0  # boltzmann.py:189 drops w = 0 particles on restart
    np.testing.assert_array_equal(rx, x[keep])
    np.testing.assert_array_equal(rw, w[keep])
    g = rng.random((5, 33))
    bzio.write_grid(name, 3, *g, ca={"ne": g[0], "ni": g[1], "Te": g[2], "E": g[3]})
    np.testing.assert_array_equal(bzio.read_grid(name, 3, "ionprod_total"), g[4])
    np.testing.assert_array_equal(bzio.read_grid(name, 3, "Te_CA"), g[2])


def test_config_matches_reference_constants():
    c = config.reference(5, num_particles=500000, gridpts=1200)
    assert c.N == 1199 and c.dx == pytest.approx(2.54 / 1199)
    assert c.nn_cm3 == pytest.approx(3.22e16 * 0.1)      # boltzmann.py:47-49
    assert c.mu_i == pytest.approx(4.65e19 / (3.22e15))  # boltzmann.py:55
    assert c.targets() == [int(f * 500000 / 1199) for f in (0.4, 0.3, 0.2, 0.07, 0.03)]
    assert c.max_ppc() == [int(10 * t) for t in c.targets()]
    assert config.gas_sigma_reference() == pytest.approx(math.sqrt((300 / 11606) * 1.5 * 1.17255e11))
    b = config.ccp_1024()
    assert b.N == 1024 and b.num_particles == 20_000_000 and b.nbins == 5
    assert b.dt == pytest.approx(1 / 13.56e6 / 400)
    assert b.mu_i * 1e-4 == pytest.approx(0.1444, rel=1e-3)  # 0.14 m^2/(V s) at 1 Torr


def test_omp_step_matches_serial_oracle():
    """The timed CPU baseline (orc_step_omp) gives the serial oracle's particles in the
    same order and the same moments (summation order aside)."""
    rng = np.random.default_rng(1)
    n, N, L = 20_000, 64, 2.54
    x = rng.uniform(0.01, L - 0.01, n)
    v = rng.normal(0, 1.5e6, (n, 3))
    w = rng.uniform(1, 2, n)
    E = rng.uniform(-1000, 1000, N)
    tab = xsec.analytic_argon(2000)
    nn = 3.22e22
    p = O.make_params(N, L=L, dt=1 / 13.56e6 / 400, nn=nn, rng_mode=1, precision=64, seed=5, gas_sigma=6.7e4,
                      xs_table=tab.nsigma(nn), xs_emin=tab.emin, xs_emax=tab.emax, e_exc=tab.e_exc)
    d1, t1 = O.soa_to_aos(x, v[:, 0], v[:, 1], v[:, 2], w, cap=3 * n)
    nni = O.push(p, d1, t1, n, E)
    mom1, n1 = O.post(p, d1, t1, n + nni)
    import ctypes
    d2, t2 = O.soa_to_aos(x, v[:, 0], v[:, 1], v[:, 2], w, cap=3 * n)
    dt_, tt_ = np.zeros((6 * n, 6)), np.zeros((6 * n, 4))
    mom2 = np.zeros((4, N + 1))
    n2 = O.lib().orc_step_omp(ctypes.byref(p), n, 3 * n, d2, t2, dt_, tt_, np.ascontiguousarray(E), mom2, 4)
    assert n2 == n1
    np.testing.assert_allclose(d2[:n2, [0, 3, 4, 5]], d1[:n1, [0, 3, 4, 5]], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(t2[:n2, 0], t1[:n1, 0])
    for j in (0, 1, 3):
        np.testing.assert_allclose(mom2[j], mom1[j], rtol=1e-10, atol=1e-9)
    # the guard: a sample larger than half its buffer is refused, nothing written
    assert O.lib().orc_step_omp(ctypes.byref(p), n, n, d2, t2, dt_, tt_, np.ascontiguousarray(E), mom2, 2) == -1


def test_segment_set_counts_live_particles_apart_from_slots():
    """SegmentSet.n() counts occupied slots, n_live() the particles among them (slots with
    w = 0, which an in-place resampling leaves, are not particles)."""
    import torch
    from boltzmann_gb300 import kernels as K
    s = K.SegmentSet(3, 8, torch.float32, device="cpu")
    s.counts.copy_(torch.tensor([3, 1, 0, 2, 8, 0], dtype=torch.int32))
    s.w.fill_(1.0)
    s.w[1] = 0.0            # segment 0, run 0, slot 1
    s.w[2 * 8 + 8 + 1] = 0.0  # segment 1, run 1, slot 1
    s.w[2 * 8 + 3] = 0.0    # segment 1, run 0, slot 3: not occupied, not counted either way
    assert s.n() == 14
    assert s.n_live() == 12
