"""Output and diagnostics against the reference's own run loop (no GPU).

The fixture tests/golden/cycle.npz was made by running the reference's BoltzmannDSMC.run
(boltzmann.py:565-716) for two short RF cycles through oracle/ref_shim.py: it holds every
step's grid fields as the loop accumulates them and the bytes of every file the
reference's data_write (data_write_1D.py:3-75) wrote. Checked here:

* the cycle averages of the solver's loop (CycleAverages, the arithmetic solver.run
  performs on the device, here on CPU tensors) against the reference's *_CA files;
* the raw float64 files written by boltzmann_gb300.io against the reference's, byte for
  byte, names included;
* the restart reader (boltzmann.py:182-205: the particle files read back, w = 0 entries
  dropped) on the reference's own particle files. The reference's restart branch itself is
  unreachable as shipped (IC_flag = 1 is hard-coded and a restart with it set exits,
  boltzmann.py:151-155), so its reading is restated;
* the ion production total restarting every cycle (boltzmann.py:713-714): the reference's
  ionprod_total file of each cycle is the sum of that cycle's ion sources.
"""
import os

import numpy as np
import torch

from boltzmann_gb300 import io as bzio
from boltzmann_gb300.solver import CycleAverages

G = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cycle.npz"))
SPC, CYCLES = int(G["spc"]), int(G["cycles"])


def ref_file(name):
    return np.frombuffer(G["file_" + name].tobytes(), dtype="<f8")


def test_cycle_averages_match_the_reference_loop():
    rec = {k: G["rec_" + k] for k in ("ne", "ni", "Te", "E")}
    avg = CycleAverages({k: torch.zeros(v.shape[1], dtype=torch.float64) for k, v in rec.items()})
    cycle = 0
    for step in range(1, SPC * CYCLES + 1):
        if step % SPC != 0:
            avg.add({k: torch.as_tensor(v[step - 1]) for k, v in rec.items()})
        else:
            cycle += 1
            ca = avg.take(SPC)
            for k in rec:
                ref = ref_file(f"{k}_CA_cycle{cycle}.dat")
                np.testing.assert_allclose(ca[k].numpy(), ref, rtol=1e-12, atol=0)
    assert cycle == CYCLES


def test_files_match_the_reference_byte_for_byte(tmp_path):
    name = str(tmp_path / "run_")
    for c in range(1, CYCLES + 1):
        ca = {k: ref_file(f"{k}_CA_cycle{c}.dat") for k in ("ne", "ni", "Te", "E")}
        bzio.write_grid(name, c, ref_file(f"ne_cycle{c}.dat"), ref_file(f"ni_cycle{c}.dat"),
                        ref_file(f"Te_cycle{c}.dat"), ref_file(f"E_cycle{c}.dat"),
                        ref_file(f"ionprod_total_cycle{c}.dat"), ca)
        bzio.write_particles(name, c, *(ref_file(f"e_{t}_cycle{c}_mpi0.dat") for t in ("x0", "v0", "v1", "v2", "wt")))
    ours = sorted(f[len("run_"):] for f in os.listdir(tmp_path))
    assert ours == sorted(str(f) for f in G["file_names"])
    for f in ours:
        assert (tmp_path / ("run_" + f)).read_bytes() == G["file_" + f].tobytes(), f


def test_restart_reader_on_the_reference_files(tmp_path):
    name = str(tmp_path / "ref_")
    for f in G["file_names"]:
        (tmp_path / ("ref_" + str(f))).write_bytes(G["file_" + str(f)].tobytes())
    for c in range(1, CYCLES + 1):
        x, vx, vy, vz, w = bzio.read_particles(name, c)
        keep = ref_file(f"e_wt_cycle{c}_mpi0.dat") != 0
        for got, t in zip((x, vx, vy, vz, w), ("x0", "v0", "v1", "v2", "wt")):
            np.testing.assert_array_equal(got, ref_file(f"e_{t}_cycle{c}_mpi0.dat")[keep])
        np.testing.assert_array_equal(bzio.read_grid(name, c, "ni"), ref_file(f"ni_cycle{c}.dat"))


def test_ion_production_restarts_every_cycle():
    src = G["rec_ni_src"]
    assert src.sum() > 0
    for c in range(1, CYCLES + 1):
        np.testing.assert_allclose(ref_file(f"ionprod_total_cycle{c}.dat"), src[(c - 1) * SPC: c * SPC].sum(axis=0),
                                   rtol=1e-12)
