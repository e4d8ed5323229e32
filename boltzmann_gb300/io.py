"""Output and restart files in the reference's raw float64 format.

data_write_1D.py:3-75 writes headerless little-endian float64 arrays once per RF
cycle: grid quantities ``<name>{ne,ni,Te,E,ionprod_total}_cycle<k>.dat``, their cycle
averages ``<name>{ne,ni,Te,E}_CA_cycle<k>.dat`` and the particles
``<name>e_{x0,v0,v1,v2,wt}_cycle<k>_mpi<rank>.dat``. boltzmann.py:157-239 reads the
particle files back (dropping w = 0) for a restart.
"""
from __future__ import annotations

import os

import numpy as np


def _w(path, arr):
    np.ascontiguousarray(np.asarray(arr, dtype="<f8")).tofile(path)


def write_grid(name, cycle, ne, ni, Te, E, ionprod, ca=None):
    c = f"_cycle{cycle}.dat"
    _w(name + "ne" + c, ne)
    _w(name + "ni" + c, ni)
    _w(name + "Te" + c, Te)
    _w(name + "E" + c, E)
    _w(name + "ionprod_total" + c, ionprod)
    if ca is not None:
        for k in ("ne", "ni", "Te", "E"):
            _w(name + k + "_CA" + c, ca[k])


def write_particles(name, cycle, x, vx, vy, vz, w, rank=0):
    c = f"_cycle{cycle}_mpi{rank}.dat"
    for tag, a in (("e_x0", x), ("e_v0", vx), ("e_v1", vy), ("e_v2", vz), ("e_wt", w)):
        _w(name + tag + c, a)


def read_particles(name, cycle, rank=0):
    """boltzmann.py:182-190: the five particle files, w = 0 entries dropped."""
    c = f"_cycle{cycle}_mpi{rank}.dat"
    arr = {tag: np.fromfile(name + tag + c, dtype="<f8") for tag in ("e_x0", "e_v0", "e_v1", "e_v2", "e_wt")}
    keep = arr["e_wt"] != 0
    return tuple(arr[t][keep] for t in ("e_x0", "e_v0", "e_v1", "e_v2", "e_wt"))


def read_grid(name, cycle, key):
    return np.fromfile(name + key + f"_cycle{cycle}.dat", dtype="<f8")


def data_write(solver, name, cycle, ca=None):
    """Write one cycle's files from a BoltzmannGB300 (data_write_1D.py:3-75)."""
    d = os.path.dirname(name)
    if d:
        os.makedirs(d, exist_ok=True)
    cpu = lambda t: t.detach().cpu().numpy().astype(np.float64)
    cam = None if ca is None else {k: cpu(v) for k, v in ca.items()}
    write_grid(name, cycle, cpu(solver.moments[0]), cpu(solver.ni), cpu(solver.Te), cpu(solver.E), cpu(solver.g2),
               cam)
    p = solver.A.to_numpy()
    write_particles(name, cycle, p["x"], p["vx"], p["vy"], p["vz"], p["w"])
