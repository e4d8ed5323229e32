"""The device-resident solver: graph replay matches eager stepping, the step loop
keeps its invariants, and the reference-format output round-trips."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from boltzmann_gb300 import config, io as bzio  # noqa: E402
from boltzmann_gb300.solver import BoltzmannGB300  # noqa: E402


def small_cfg(**kw):
    base = dict(gridpts=65, num_particles=60_000, resample_freq=4, steps_per_cycle=1000, in_dt=4000.0)
    base.update(kw)
    return config.ccp_256(**base)


def state(sol):
    return {k: v.copy() for k, v in sol.A.to_numpy().items()}


def test_graph_step_equals_eager_step():
    a = BoltzmannGB300(small_cfg())
    b = BoltzmannGB300(small_cfg())
    for k in range(3):
        a.step(use_graph=True)
        b.step(use_graph=False)
        sa, sb = state(a), state(b)
        assert len(sa["x"]) == len(sb["x"])
        if k == 0:  # identical inputs: bit-identical particles (moments may differ in the last bits)
            for f in sa:
                assert np.array_equal(sa[f], sb[f]), f


@pytest.mark.parametrize("prec", ["float32", "float64"])
def test_step_loop_invariants(prec):
    sol = BoltzmannGB300(small_cfg(precision=prec))
    n0 = sol.n()
    sol.run(24)
    torch.cuda.synchronize()
    assert sol.device_status() == 0
    n = sol.n()
    assert 0.3 * n0 < n < 3 * n0
    s = sol.A.to_numpy()
    assert np.all(s["w"] > 0)
    assert np.all((s["x"] > 0) & (s["x"] < sol.cfg.L))
    for t in (sol.moments, sol.E, sol.ni, sol.Te):
        assert torch.isfinite(t).all()
    assert int(sol.particle_steps.item()) > 20 * 0.3 * n0


def test_reference_format_roundtrip(tmp_path):
    sol = BoltzmannGB300(small_cfg(num_particles=5000, gridpts=33))
    sol.run(2)
    name = str(tmp_path / "run_")
    bzio.data_write(sol, name, 1)
    x, vx, vy, vz, w = bzio.read_particles(name, 1)
    s = sol.A.to_numpy()
    np.testing.assert_array_equal(x, s["x"])
    np.testing.assert_array_equal(w, s["w"])
    ne = bzio.read_grid(name, 1, "ne")
    np.testing.assert_array_equal(ne, sol.moments[0].cpu().numpy())


def test_snapshot_restore_returns_the_state():
    """restore(snapshot()) puts the particles, the grid block, the clock, the status words
    and the step index back into the same buffers, across both buffer roles and a
    resampling step, and the captured step graphs keep running from there."""
    sol = BoltzmannGB300(small_cfg())
    for _ in range(3):
        sol.step()
    sol.capture_all()
    snap = sol.snapshot()
    s0, io0, t0, b0 = state(sol), sol.io.clone(), float(sol.t.item()), sol.bigstep
    for _ in range(5):  # passes a resampling step (every 4) and swaps the buffer roles
        sol.step()
    assert sol.bigstep == b0 + 5 and float(sol.t.item()) != t0
    sol.restore(snap)
    torch.cuda.synchronize()
    assert sol.bigstep == b0 and float(sol.t.item()) == t0
    s1 = state(sol)
    for f in s0:
        np.testing.assert_array_equal(s0[f], s1[f], err_msg=f)
    assert torch.equal(io0, sol.io)
    ps = int(sol.particle_steps.item())
    for _ in range(5):
        sol.step()
    torch.cuda.synchronize()
    assert sol.device_status() == 0 and int(sol.particle_steps.item()) > ps
    assert torch.isfinite(sol.E).all()


def test_run_writes_cycle_files_like_the_reference_loop(tmp_path):
    """solver.run over two short cycles with output: every cycle's *_CA files hold the
    mean the reference's loop forms (the fields after the cycle's first spc-1 steps,
    divided by spc; boltzmann.py:681-701), and ionprod_total holds that cycle's ion
    sources only (the reference resets it every cycle, boltzmann.py:713-714). The fields
    are recorded after every step of the same run through run()'s per-step hook."""
    spc = 5
    sol = BoltzmannGB300(small_cfg(num_particles=20_000, gridpts=33, steps_per_cycle=spc, Te_init_eV=6.0))
    name = str(tmp_path / "run_")
    rec, srcs = [], []

    def record(s):
        rec.append({f: v.cpu().numpy().copy() for f, v in s.grid_fields().items()})
        srcs.append(s.moments[1].cpu().numpy().copy())

    sol.run(2 * spc, name=name, write=True, on_step=record)
    torch.cuda.synchronize()
    assert sol.device_status() == 0 and len(rec) == 2 * spc
    for c in (1, 2):
        steps = rec[(c - 1) * spc: c * spc]
        for f in ("ne", "ni", "Te", "E"):
            exp = np.sum([st[f] for st in steps[:-1]], axis=0) / spc
            got = bzio.read_grid(name, c, f + "_CA")
            np.testing.assert_allclose(got, exp, rtol=1e-12, atol=1e-12 * np.abs(exp).max())
        ion = bzio.read_grid(name, c, "ionprod_total")
        exp = np.sum(srcs[(c - 1) * spc: c * spc], axis=0)
        np.testing.assert_allclose(ion, exp, rtol=1e-12, atol=1e-12 * max(np.abs(exp).max(), 1.0))
        np.testing.assert_array_equal(bzio.read_grid(name, c, "ne"), steps[-1]["ne"])
    assert np.sum(srcs) > 0  # the hot start ionizes


def test_ion_source_rate_closure():
    """set_ion_closure: the ion source of a step is k_ion n_gas dt times the deposited
    electron density of each node (instead of the counted ionizations), both eager and
    graph-replayed; clearing it restores the counted source."""
    sol = BoltzmannGB300(small_cfg(), device="cuda")
    for _ in range(3):
        sol.step()
    k = np.linspace(1e-16, 3e-16, sol.nnodes)
    sol.set_ion_closure(k)
    rate = k * sol.cfg.nn_m3 * sol.cfg.dt
    for use_graph in (False, True, True):
        sol.step(use_graph=use_graph)
        m = sol.moments.cpu().numpy()
        assert m[0].sum() > 0
        np.testing.assert_allclose(m[1], rate * m[0], rtol=1e-15, atol=0)
    assert sol.device_status() == 0
    sol.set_ion_closure(None)
    sol.step()
    m = sol.moments.cpu().numpy()
    assert not np.allclose(m[1], rate * m[0])
