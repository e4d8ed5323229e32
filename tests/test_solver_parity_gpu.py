"""The GPU solver against the oracle's CPU step loop (oracle/ccp.py) on a small 1 Torr
argon CCP: 128 cells, 1e5 electrons at 1 eV, 3-bin ES-WPNC every 50 steps, 400 steps of
tau/4000 (a tenth of an RF cycle, while the sheaths form; at tau/400 this explicit scheme
heats the uniform start within a cycle, which makes a poor statistical test). The two
use different random streams, so they are compared
statistically: the mean of two oracle runs and the mean of eight independent GPU runs must
agree within four standard errors (plus 0.5% for the remaining float32 effects) for the
electron count, the ionizations, the mean energy and the averaged density in eight regions.
"""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from boltzmann_gb300 import config  # noqa: E402
from boltzmann_gb300.solver import BoltzmannGB300  # noqa: E402
from oracle.ccp import OracleCCP  # noqa: E402

STEPS, AVG_FROM, REGIONS = 400, 200, 8


def cfg(seed):
    return config.CCPConfig(gridpts=129, pressure_torr=1.0, in_dt=4000.0, steps_per_cycle=4000, num_particles=100_000,
                            Te_init_eV=1.0, ne_profile="uniform", bin_edges=(4.0, 11.5), bin_fractions=(0.7, 0.2, 0.1),
                            xs="analytic", resample_freq=50, seed=seed, autotune=False)


def observe(moments_per_step, final_weight):
    m = np.array(moments_per_step)  # [steps, 4, nodes]
    ne_avg = m[AVG_FROM:, 0].mean(axis=0)
    reg = ne_avg[: (len(ne_avg) // REGIONS) * REGIONS].reshape(REGIONS, -1).sum(axis=1)
    return {
        "weight": final_weight,
        "ionizations": m[:, 1].sum(),
        "mean_energy": m[AVG_FROM:, 3].sum() / m[AVG_FROM:, 0].sum(),
        **{f"region{k}": reg[k] for k in range(REGIONS)},
    }


def gpu_run(seed):
    sol = BoltzmannGB300(cfg(seed), device="cuda")
    moms = []
    for _ in range(STEPS):
        sol.step()
        moms.append(sol.moments.cpu().numpy().copy())
    assert sol.device_status() == 0
    return sol, observe(moms, float(sol.A.to_numpy()["w"].sum()))


def test_solver_matches_oracle_step_loop_statistically():
    # two oracle runs (different random streams) from the initial state of the seed-0 GPU
    # solver, eight GPU runs with their own seeds; the means must agree within 4 standard
    # errors of the difference (+0.5%), the spread taken from the GPU runs and, for the
    # ionizations (a few hundred events), never below the counting noise
    s0 = BoltzmannGB300(cfg(0), device="cuda")
    st = s0.A.to_numpy("segments")
    w_mean = float(st["w"].mean())
    oracle = []
    for seed in (5, 6):
        orc = OracleCCP(s0.cfg, st["x"], st["vx"], st["vy"], st["vz"], st["w"], s0.ni.cpu().numpy(), s0.xs,
                        seed=seed)
        moms = []
        for _ in range(STEPS):
            orc.step()
            moms.append(orc.moments.copy())
        oracle.append(observe(moms, float(orc.state()["w"].sum())))
    del s0
    runs = [gpu_run(seed)[1] for seed in range(1, 9)]
    for k in oracle[0]:
        g = np.array([r[k] for r in runs])
        o = np.array([r[k] for r in oracle])
        sd = g.std(ddof=1)
        if k == "ionizations":
            sd = max(sd, w_mean * math.sqrt(g.mean() / w_mean))
        lim = 4 * sd * math.sqrt(1 / len(g) + 1 / len(o)) + 0.005 * abs(g.mean())
        assert abs(o.mean() - g.mean()) <= lim, f"{k}: oracle {o}, GPU {g.mean():.6g} +- {sd:.3g}"
    assert min(r["ionizations"] for r in oracle) > 0


def test_tau400_start_heats_in_both_step_loops():
    """At the benchmark's dt = tau/400 the reference's explicit scheme does not settle from
    the uniform 1 eV, 1e9 cm^-3 start: the oracle's CPU step loop (float64, the reference's
    step order) and the GPU solver, from the same particles, agree step by step while both
    heat the electrons, multiply the ions about fivefold and lose every electron within one
    RF cycle (measured: 3.8, 7.4, 9.0 eV at steps 50, 100, 200 in both; ion content x5.1;
    no electron left at step 400) instead of approaching a periodic state. This pins that
    the missing periodic state of that configuration belongs to the scheme, not to this
    implementation."""
    c = config.CCPConfig(gridpts=129, pressure_torr=1.0, in_dt=400.0, steps_per_cycle=400, num_particles=100_000,
                         Te_init_eV=1.0, ne_profile="uniform", bin_edges=(4.0, 11.5), bin_fractions=(0.7, 0.2, 0.1),
                         xs="analytic", resample_freq=50, seed=3, autotune=False)
    g = BoltzmannGB300(c, device="cuda")
    st = g.A.to_numpy("segments")
    ni0 = float(g.ni.sum().item())
    orc = OracleCCP(g.cfg, st["x"], st["vx"], st["vy"], st["vz"], st["w"], g.ni.cpu().numpy(), g.xs, seed=11)
    traces = {"gpu": [], "oracle": []}
    for _ in range(400):
        g.step(use_graph=False)
        orc.step()
        mg, mo = g.moments.cpu().numpy(), orc.moments
        traces["gpu"].append((mg[3].sum() / max(mg[0].sum(), 1e-300), float(g.ni.sum().item()), mg[0].sum()))
        traces["oracle"].append((mo[3].sum() / max(mo[0].sum(), 1e-300), float(orc.ni.sum()), mo[0].sum()))
    for name, tr in traces.items():
        e = np.array([t[0] for t in tr])
        ni = np.array([t[1] for t in tr])
        ne = np.array([t[2] for t in tr])
        print(name, "mean energy at steps 50/100/200/400:", e[[49, 99, 199, 399]], "ion content ratio:", ni[-1] / ni0,
              "electron content at steps 100/200/300/400:", ne[[99, 199, 299, 399]] / ne[0])
        assert e[199] > 2.0 * e[49], name     # heated well beyond the start
        assert ni[-1] > 3.0 * ni0, name       # the ions multiply within the cycle
        assert ne[-1] < 0.05 * ne[0], name    # and the electrons are lost
    eg = np.array([t[0] for t in traces["gpu"]])
    eo = np.array([t[0] for t in traces["oracle"]])
    # the two loops agree on the way up (first half cycle), within 10%
    np.testing.assert_allclose(eg[100:200:20], eo[100:200:20], rtol=0.1)
