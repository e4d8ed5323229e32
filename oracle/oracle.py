"""ctypes front end of the FP64 C oracle (``bz_oracle.c``).

TEST INFRASTRUCTURE ONLY: used by ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` as the checker and the reported CPU baseline. The
product path (``boltzmann_gb300``) never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liborc.so")

_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("n_faces", ctypes.c_int), ("n_nodes", ctypes.c_int), ("bnf", ctypes.c_int),
        ("L", ctypes.c_double), ("dx", ctypes.c_double), ("dt", ctypes.c_double), ("nn", ctypes.c_double),
        ("xs_mode", ctypes.c_int), ("coll_model", ctypes.c_int), ("advect", ctypes.c_int),
        ("rng_mode", ctypes.c_int), ("precision", ctypes.c_int),
        ("seed", ctypes.c_uint64), ("step", ctypes.c_uint64), ("gas_sigma", ctypes.c_double),
        ("xs_n", ctypes.c_int), ("xs_emin", ctypes.c_double), ("xs_emax", ctypes.c_double),
        ("xs_table", ctypes.c_void_p), ("nu_max", ctypes.c_double), ("e_exc", ctypes.c_double),
        ("moment_exc", ctypes.c_int),
    ]


def build(force=False):
    """Compile bz_oracle.c into liborc.so (gcc, OpenMP)."""
    src = os.path.join(HERE, "bz_oracle.c")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "bz_oracle.h"))):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-o", tmp, src, "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER(OrcParams)
        L.orc_philox.argtypes = [np.ctypeslib.ndpointer(np.uint32), np.ctypeslib.ndpointer(np.uint32),
                                 np.ctypeslib.ndpointer(np.uint32)]
        L.orc_philox_rounds.argtypes = [np.ctypeslib.ndpointer(np.uint32), np.ctypeslib.ndpointer(np.uint32),
                                        np.ctypeslib.ndpointer(np.uint32), ctypes.c_int]
        L.orc_push.argtypes = [P, ctypes.c_int64, _f64p, _f64p, _f64p, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_push.restype = ctypes.c_int64
        L.orc_push_margin.argtypes = [P, ctypes.c_int64, _f64p, _f64p, _f64p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p]
        L.orc_push_margin.restype = ctypes.c_int64
        L.orc_post.argtypes = [P, ctypes.c_int64, _f64p, _f64p, _f64p]
        L.orc_post.restype = ctypes.c_int64
        L.orc_deposit.argtypes = [P, ctypes.c_int64, _f64p, _f64p, _f64p]
        L.orc_bin.argtypes = [P, ctypes.c_int64, _f64p, _f64p, _f64p, _f64p, _f64p, ctypes.c_int, _f64p,
                              ctypes.c_int64, _i64p, _i64p]
        L.orc_resample.argtypes = [P, ctypes.c_int64, _f64p, _f64p, ctypes.c_int, _i64p, ctypes.c_double, _i64p,
                                   _i64p, _i64p, ctypes.c_int64, _f64p, ctypes.c_int64,
                                   ctypes.POINTER(ctypes.c_int64), ctypes.c_int, ctypes.c_void_p]
        L.orc_resample.restype = ctypes.c_int64
        L.orc_eedf.argtypes = [P, ctypes.c_int64, _f64p, _f64p, _f64p, _f64p, _f64p, ctypes.c_int, ctypes.c_double,
                               ctypes.c_double, _f64p]
        L.orc_poisson.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_double, _f64p, _f64p, _f64p, _f64p]
        L.orc_fluid.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                _f64p, _f64p, _f64p]
        L.orc_fluid.restype = ctypes.c_int
        L.orc_step_omp.argtypes = [P, ctypes.c_int64, ctypes.c_int64, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p,
                                   ctypes.c_int]
        L.orc_step_omp.restype = ctypes.c_int64
        _lib = L
    return _lib


def make_params(N, L=2.54, bnf=4, dt=1e-12, nn=3.22e22, xs_mode=0, coll_model=0, advect=1, rng_mode=0,
                precision=32, seed=0, step=0, gas_sigma=0.0, xs_table=None, xs_emin=0.01, xs_emax=1000.0,
                nu_max=0.0, e_exc=11.5, moment_exc=0):
    """Parameters for an N-face / N+1-node grid. ``xs_table`` is an [3, n] float32 n*sigma table."""
    p = OrcParams()
    p.n_faces = N
    p.n_nodes = N + 1
    p.bnf = bnf
    p.L = L
    p.dx = L / N
    p.dt = dt
    p.nn = nn
    p.xs_mode = xs_mode
    p.coll_model = coll_model
    p.advect = advect
    p.rng_mode = rng_mode
    p.precision = precision
    p.seed = seed
    p.step = step
    p.gas_sigma = gas_sigma
    p.nu_max = nu_max
    p.e_exc = e_exc
    p.moment_exc = int(moment_exc)
    p._keep = None
    if xs_table is not None:
        tab = np.ascontiguousarray(xs_table, dtype=np.float32)
        p.xs_n = tab.shape[1]
        p.xs_emin = xs_emin
        p.xs_emax = xs_emax
        p.xs_table = tab.ctypes.data
        p._keep = tab
    return p


def soa_to_aos(x, vx, vy, vz, w, cap=None):
    n = len(x)
    cap = cap or n
    data = np.zeros((cap, 6))
    tosum = np.zeros((cap, 4))
    data[:n, 0] = x
    data[:n, 3] = vx
    data[:n, 4] = vy
    data[:n, 5] = vz
    tosum[:n, 0] = w
    me, jev = 9.10938 * 10 ** (-31), 6.241509 * (10 ** 18)
    tosum[:n, 3] = 0.5 * me * jev * (vx * vx + vy * vy + vz * vz)
    return data, tosum


def push(p, data, tosum, n, E, R=None, gas=None):
    """Run orc_push in place on AoS buffers (capacity >= 2n). Returns the child count."""
    Rp = None if R is None else np.ascontiguousarray(R, dtype=np.float64)
    gp = None if gas is None else np.ascontiguousarray(gas, dtype=np.float64)
    E = np.ascontiguousarray(E, dtype=np.float64)
    return lib().orc_push(ctypes.byref(p), n, data, tosum, E,
                          None if Rp is None else Rp.ctypes.data, None if gp is None else gp.ctypes.data)


def push_margin(p, data, tosum, n, E, R=None, gas=None):
    """orc_push with per-particle decision margins. Returns (children, margin[n])."""
    Rp = None if R is None else np.ascontiguousarray(R, dtype=np.float64)
    gp = None if gas is None else np.ascontiguousarray(gas, dtype=np.float64)
    E = np.ascontiguousarray(E, dtype=np.float64)
    m = np.zeros(n)
    nni = lib().orc_push_margin(ctypes.byref(p), n, data, tosum, E, None if Rp is None else Rp.ctypes.data,
                                None if gp is None else gp.ctypes.data, m.ctypes.data)
    return nni, m


def post(p, data, tosum, n_total):
    mom = np.zeros((4, p.n_nodes))
    nnew = lib().orc_post(ctypes.byref(p), n_total, data, tosum, mom)
    return mom, nnew


def deposit(p, data, tosum, n_total):
    mom = np.zeros((4, p.n_nodes))
    lib().orc_deposit(ctypes.byref(p), n_total, np.ascontiguousarray(data), np.ascontiguousarray(tosum), mom)
    return mom


def bin_particles(p, x, vx, vy, vz, w, edges, max_ppc):
    nb = len(edges) + 1
    counts = np.zeros((nb, p.n_nodes), dtype=np.int64)
    lists = np.zeros((nb, max_ppc, p.n_nodes), dtype=np.int64)
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.float64).reshape(-1) if len(edges) else np.zeros(1))
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    lib().orc_bin(ctypes.byref(p), len(x), f(x), f(vx), f(vy), f(vz), f(w), nb, e, max_ppc, counts, lists)
    return counts, lists


def resample(p, data, tosum, n, nb, targets, min_wt, max_ppc, counts, lists, u, flags=1, thr=None):
    """thr = (split_below, merge_at, merge_keep); None: the reference's (0.5, 3, 0.6).
    flags bit 4 (0x10): targets / max_ppc per (cell, bin) key, index cell*nb + bin."""
    used = ctypes.c_int64(0)
    thr_a = None if thr is None else np.ascontiguousarray(thr, dtype=np.float64)
    targets = np.ascontiguousarray(targets, dtype=np.int64)
    max_ppc = np.ascontiguousarray(max_ppc, dtype=np.int64)
    u = np.ascontiguousarray(u, dtype=np.float64) if len(u) else np.zeros(1)
    na = lib().orc_resample(ctypes.byref(p), n, data, tosum, nb, targets, float(min_wt), max_ppc,
                            np.ascontiguousarray(counts, dtype=np.int64), np.ascontiguousarray(lists, dtype=np.int64),
                            lists.shape[1], u, len(u), ctypes.byref(used), flags,
                            None if thr_a is None else thr_a.ctypes.data_as(ctypes.c_void_p))
    return na, used.value


def eedf(p, x, vx, vy, vz, w, nbins, emin, emax):
    hist = np.zeros((p.n_nodes, nbins))
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    lib().orc_eedf(ctypes.byref(p), len(x), f(x), f(vx), f(vy), f(vz), f(w), int(nbins), float(emin), float(emax),
                   hist)
    return hist


def poisson(N, dx, eps0, V0, freq, t, ne, ni):
    V = np.zeros(N - 1)
    E = np.zeros(N)
    lib().orc_poisson(N, dx, eps0, V0, freq, t, np.ascontiguousarray(ne, dtype=np.float64),
                      np.ascontiguousarray(ni, dtype=np.float64), V, E)
    return V, E


def fluid(N, dx, dt, mu_i, D_i, E, ni):
    ni = np.array(ni, dtype=np.float64)
    Ji = np.zeros(N)
    brk = lib().orc_fluid(N, dx, dt, mu_i, D_i, np.ascontiguousarray(E, dtype=np.float64), ni, Ji)
    return ni, Ji, brk


def philox(ctr, key, rounds=10):
    out = np.zeros(4, dtype=np.uint32)
    lib().orc_philox_rounds(np.asarray(ctr, dtype=np.uint32), np.asarray(key, dtype=np.uint32), out, int(rounds))
    return out
