"""Generate the golden vectors under ``tests/golden`` from the reference itself.

Runs the reference's own Python source (jfabell/boltzmann, variants ``1bin``,
``3bin``, ``5bin``) on the CPU through ``oracle/ref_shim.py`` and stores inputs,
every random number the reference drew, and its outputs as small ``.npz`` files.
Needs the reference checkout (``BZ_REFERENCE_ROOT``, default ``/root/reference``);
the fixtures are committed so that tests never need it.

All particle inputs are float32-representable (x, v, w, E, gas velocities) and all
uniforms are odd multiples of 2**-24, so the float32 CUDA kernels and the float64
reference see exactly the same input values.

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref_shim as rs  # noqa: E402

M_E = 9.10938 * 10 ** (-31)
J_EV = 6.241509 * (10 ** 18)
L = 2.54
TAU = 1.0 / 13.56e6

# Energy boundaries of the reference's cross-section fits (electron_kernel_numba.py:104-114, 156-162)
ELASTIC_EDGES = [0.000780396, 0.006098667, 0.0476269, 0.1015574, 0.1943527, 0.2995781,
                 1.097156, 2.339524, 4.988691, 10.63765, 22.68322]
ION_EDGES = [15.76, 15.77742, 15.81964, 15.96196, 16.44162, 18.05837, 23.50771, 41.87498]


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def quant_uniform(u):
    """Odd multiples of 2**-24 in (0,1): exact in float32, and so is 1-u."""
    k = np.floor(np.asarray(u) * (1 << 23)).astype(np.int64)
    return (k + 0.5) / float(1 << 23)


def speed_for_energy(eps):
    return np.sqrt(2.0 * np.asarray(eps) / (M_E * J_EV))


def iso_dirs(rng, n):
    c = rng.uniform(-1, 1, n)
    s = np.sqrt(1 - c * c)
    ph = rng.uniform(0, 2 * np.pi, n)
    return np.stack([s * np.cos(ph), s * np.sin(ph), c], axis=1)


def engineered_state(rng, n_rand, N, Te_eV=5.0, include_edges=True):
    """Particles: Maxwellian bulk + σ-boundary energies + wall crossers + dead + cell edges."""
    dx = L / N
    xs, vs, ws, gas_zero = [], [], [], []
    # bulk
    x = rng.uniform(0.02, L - 0.02, n_rand)
    sig = math.sqrt(Te_eV / (M_E * J_EV))
    v = rng.normal(0.0, sig, (n_rand, 3))
    xs.append(x); vs.append(v); ws.append(rng.uniform(0.5e5, 2.0e5, n_rand)); gas_zero.append(np.zeros(n_rand, bool))
    if include_edges:
        # energies at the σ-fit piece boundaries and the ionization threshold, both sides
        edges = np.array(ELASTIC_EDGES + ION_EDGES)
        eps = np.concatenate([edges * (1 - 2e-6), edges, edges * (1 + 2e-6), edges * (1 + 1e-3)])
        eps = np.concatenate([eps, np.geomspace(1e-3, 900.0, 200)])
        ne = len(eps)
        v = speed_for_energy(eps)[:, None] * iso_dirs(rng, ne)
        xs.append(rng.uniform(0.1, L - 0.1, ne)); vs.append(v); ws.append(rng.uniform(1e4, 1e5, ne)); gas_zero.append(np.ones(ne, bool))
        # wall crossers: close to a wall, fast outward
        nw = 120
        side = rng.integers(0, 2, nw)
        x = np.where(side == 0, rng.uniform(1e-5, 5e-3, nw), L - rng.uniform(1e-5, 5e-3, nw))
        v = rng.normal(0.0, sig, (nw, 3))
        v[:, 0] = np.where(side == 0, -1, 1) * speed_for_energy(rng.uniform(5, 80, nw))
        xs.append(x); vs.append(v); ws.append(rng.uniform(1e4, 1e5, nw)); gas_zero.append(np.zeros(nw, bool))
        # dead particles (w = 0) at the reference's parking spot and elsewhere
        nd = 40
        x = np.where(np.arange(nd) % 2 == 0, 1e-8, rng.uniform(0.1, L - 0.1, nd))
        v = rng.normal(0.0, sig, (nd, 3)) * (np.arange(nd) % 3 != 0)[:, None]
        xs.append(x); vs.append(v); ws.append(np.zeros(nd)); gas_zero.append(np.zeros(nd, bool))
        # cell-edge positions: x at k*dx and (k+1/2)*dx, slow so they stay near the edge
        k = rng.integers(1, N - 1, 120)
        half = (np.arange(120) % 2) * 0.5
        x = (k + half) * dx
        v = rng.normal(0.0, sig * 0.01, (120, 3))
        xs.append(x); vs.append(v); ws.append(rng.uniform(1e4, 1e5, 120)); gas_zero.append(np.zeros(120, bool))
    x = f32(np.concatenate(xs))
    v = f32(np.concatenate(vs))
    w = f32(np.concatenate(ws))
    gz = np.concatenate(gas_zero)
    return x, v, w, gz


def run_push(ns, x, v, w, E, gas, nn_m3, dt, N, bnf, seed):
    """electron_kernel (electron_kernel_numba.py:291-303) then post_processing
    (post_processing_1D.py:40-68) exactly as the step loop calls them
    (boltzmann.py:592-630)."""
    cp = ns.cupy
    Nc = len(x)
    Nmax = 3 * Nc + 16
    dx = L / N
    data = cp.zeros((Nmax, 6))
    tosum = cp.zeros((Nmax, 4))
    collct = cp.zeros((Nmax, 4))
    data[0:Nc, 0] = x
    data[0:Nc, 3:6] = v
    tosum[0:Nc, 0] = w
    tosum[0:Nc, 3] = 0.5 * M_E * J_EV * (v[:, 0] * v[:, 0] + (v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2]))
    forE = cp.zeros(Nmax).astype(int)
    curr = cp.zeros(Nmax).astype(int)
    forE[0:Nc] = (data[0:Nc, 0] / dx).astype(int)
    curr[0:Nc] = ((data[0:Nc, 0] + 0.5 * dx) / dx).astype(int)
    R = cp.zeros((Nmax, 7))
    gas_v = cp.zeros((Nmax, 3))
    gas_v[0:Nc, :] = gas
    count = cp.zeros(1).astype(int)
    g0 = cp.zeros(Nmax)
    g2 = cp.zeros(Nmax)
    E_d = cp.array(E)
    numba_cuda = ns.numba.cuda
    d = numba_cuda.to_device
    # the launcher draws R[0:Nc,:] = cp.random.rand(Nc, 7); quantise its stream
    rs.DRAWS.reset(seed)
    gen = rs.DRAWS.gen

    class _QGen:
        def random(self, shape=None):
            return quant_uniform(gen.random(shape))

        def standard_normal(self, shape):
            return gen.standard_normal(shape)

        def permutation(self, n):
            return gen.permutation(n)

    rs.DRAWS.gen = _QGen()
    ns.electron.electron_kernel(Nc, d(data), d(tosum), d(collct), d(E_d), R, d(R), d(curr), d(forE),
                                nn_m3, 1, dt, d(count), d(g0), d(g2), d(gas_v), 1024, 64)
    nni = int(count[0])
    R_used = np.array(R[0:Nc, :])
    post_data = np.array(data[0:Nc + nni, :])
    post_tosum = np.array(tosum[0:Nc + nni, :])
    # post_processing with the reference's buffers
    big_N = bnf * (N + 1)
    RN = N + 1
    bufs = [cp.zeros((big_N, 4)) for _ in range(3)]
    nps = [np.zeros((big_N, 4)) for _ in range(3)]
    temp_x = cp.zeros(Nmax)
    grid = [np.zeros(N + 1) for _ in range(8)]
    out = ns.post.post_processing(bufs[0], nps[0], bufs[1], nps[1], bufs[2], nps[2], data, tosum, collct, True,
                                  Nc, Nc, nni, *grid, big_N, RN, L, dx, temp_x)
    ne, ni_src, ns_src, nrg = out[0], out[1], out[2], out[3]
    Nnew = out[8]
    return dict(
        x=x, v=v, w=w, E=np.asarray(E), gas=np.asarray(gas), R=R_used, nn=nn_m3, dt=dt, N=N, L=L, bnf=bnf,
        forE=np.array(forE[0:Nc]), nni=nni, k_data=post_data, k_tosum=post_tosum,
        ne=np.array(ne), ni_src=np.array(ni_src), ns_src=np.array(ns_src), nrg=np.array(nrg), Nnew=Nnew,
        c_data=np.array(data[0:Nnew, :]), c_tosum=np.array(tosum[0:Nnew, :]),
    )


def case_push(ns, name, nn_m3, dt, Te, seed, n_rand=2000, N=64, bnf=4, efield=3000.0, gas_sigma=None):
    rng = np.random.default_rng(seed)
    x, v, w, gz = engineered_state(rng, n_rand, N, Te_eV=Te)
    E = f32(rng.uniform(-efield, efield, N))
    if gas_sigma is None:
        gas_sigma = math.sqrt((300.0 / 11606.0) * 1.5 * 1.17255e11)  # boltzmann.py:556-558
    gas = f32(rng.normal(0.0, gas_sigma, (len(x), 3)))
    gas[gz] = 0.0
    d = run_push(ns, x, v, w, E, gas, nn_m3, dt, N, bnf, seed)
    np.savez_compressed(os.path.join(HERE, name), **d)
    print(name, "Nc", len(x), "nni", d["nni"], "Nnew", d["Nnew"])


# ------------------------------------------------------------------------------------------
# binning
# ------------------------------------------------------------------------------------------

BIN_EDGES = {"1bin": [], "3bin": [10.0, 15.76], "5bin": [5.0, 10.0, 15.76, 20.0]}


def case_bins(variant, seed, N=48, n=4000, max_ppc=60):
    ns = rs.load_variant(variant)
    cp = ns.cupy
    rng = np.random.default_rng(seed)
    dx = L / N
    x = rng.uniform(0.0, L, n)
    x[:200] = (rng.integers(0, N + 1, 200) + 0.5) * dx  # on cell edges (int((x+dx/2)/dx) boundaries)
    x[200:260] = rng.uniform(0, 0.3 * dx, 60)  # a crowded first cell to overflow max_ppc
    x = f32(np.clip(x, 1e-6, L - 1e-6))
    eps = rng.exponential(8.0, n)
    edges = BIN_EDGES[variant]
    if edges:
        eps[260:260 + 4 * len(edges)] = np.repeat(edges, 4) * np.tile([1 - 1e-7, 1.0, 1 + 1e-7, 1 + 1e-6], len(edges))
    v = speed_for_energy(eps)[:, None] * iso_dirs(rng, n)
    v = f32(v)
    w = f32(rng.uniform(1e3, 1e5, n))
    w[rng.integers(0, n, 50)] = 0.0  # dead particles are not binned
    e_kernel = 0.5 * M_E * J_EV * (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2])
    # energy column as the reference holds it at binning time: (eps*w)/w from post_processing
    e_col = np.where(w > 0, (e_kernel * w) / np.where(w > 0, w, 1.0), e_kernel)
    tosum = cp.zeros((n, 4))
    tosum[:, 0] = w
    tosum[:, 3] = e_col
    curr = cp.zeros(n).astype(int)
    curr[:] = ((x + 0.5 * dx) / dx).astype(int)
    nb = len(edges) + 1
    tables = [cp.zeros((max_ppc, N + 1)).astype(int) for _ in range(nb)]
    counts = [cp.zeros(N + 1).astype(int) for _ in range(nb)]
    d = ns.numba.cuda.to_device
    # argument order of each variant's bin_particles: 1bin (LE) bin_particles.py:24-25;
    # 3bin (HE, ME, LE) 3bin/kernels/bin_particles.py:39-40; 5bin (HE, ME1, ME2, ME3, LE)
    # 5bin/kernels/bin_particles.py:51-54. Our bins are ordered low -> high energy.
    order = {1: [0], 3: [2, 1, 0], 5: [4, 1, 2, 3, 0]}[nb]
    ns.bins.bin_particles(tosum, *[d(tables[k]) for k in order], *[d(counts[k]) for k in order], d(curr), n, N,
                          *([max_ppc] * nb), 64)
    np.savez_compressed(os.path.join(HERE, f"bins_{variant}.npz"), x=x, v=v, w=w, N=N, L=L,
                        edges=np.array(edges, dtype=np.float64), max_ppc=max_ppc,
                        counts=np.stack([np.array(c) for c in counts]),
                        tables=np.stack([np.array(t) for t in tables]))
    print("bins", variant, "counts total", int(sum(np.array(c).sum() for c in counts)))


# ------------------------------------------------------------------------------------------
# resampling (ES-WPNC) through the reference class itself
# ------------------------------------------------------------------------------------------

def case_resample(variant, seed, gridpts=17, Nc_arg=1600):
    ns = rs.load_variant(variant)
    cp = ns.cupy
    rs.DRAWS.reset(seed)
    b = ns.BoltzmannDSMC(1, "golden_", 0, Nc_arg, gridpts, 4, 1, False, 1, 50000.0, 1 << 30)
    rng = np.random.default_rng(seed)
    N = b.N
    dx = b.dx
    edges = BIN_EDGES[variant]
    nb = len(edges) + 1
    names = {1: ["LE"], 3: ["LE", "ME", "HE"], 5: ["LE", "ME1", "ME2", "ME3", "HE"]}[nb]
    T = np.array([int(getattr(b, "tt" + nm)) for nm in names])
    # per (cell, bin) population: mix of empty, too few, normal, too many, overflow
    bin_lo = [0.0] + edges
    bin_hi = edges + [60.0]
    xs, vs, ws = [], [], []
    for cc in range(N + 1):
        for k in range(nb):
            kind = rng.integers(0, 6)
            t = max(int(T[k]), 1)
            if kind == 0:
                m = 0
            elif kind == 1:
                m = int(rng.integers(1, max(2, int(0.5 * t))))   # split
            elif kind == 2:
                m = int(rng.integers(max(1, int(0.5 * t)) + 1, 3 * t))  # none
            elif kind in (3, 4):
                m = int(rng.integers(3 * t, 6 * t + 1))  # merge
            else:
                m = int(rng.integers(10 * t + 1, 12 * t + 2))  # merge beyond max_ppc
            if m == 0:
                continue
            lo = max(cc - 0.49, 0.001) * dx
            hi = min(cc + 0.49, N - 0.001) * dx
            xs.append(rng.uniform(lo, hi, m))
            eps = rng.uniform(bin_lo[k] + 0.01, bin_hi[k] - 0.01, m)
            dirs = iso_dirs(rng, m)
            drift = np.array([2e5, -1e5, 5e4]) * rng.uniform(0, 1)
            vs.append(speed_for_energy(eps)[:, None] * dirs + drift)
            wk = rng.uniform(0.5, 2.0, m) * 1e4
            wk[rng.uniform(0, 1, m) < 0.15] = 0.05  # below min_wt_allow: never split
            ws.append(wk)
    x = f32(np.concatenate(xs))
    v = f32(np.concatenate(vs))
    w = f32(np.concatenate(ws))
    perm = rng.permutation(len(x))
    x, v, w = x[perm], v[perm], w[perm]
    n = len(x)
    Nmax = b.Nmax_list[0]
    assert Nmax > 3 * n, (Nmax, n)
    data = b.big_data_ar_list[0]
    tosum = b.big_tosum_ar_list[0]
    data[:] = 0.0
    tosum[:] = 0.0
    data[0:n, 0] = x
    data[0:n, 3:6] = v
    tosum[0:n, 0] = w
    e_kernel = 0.5 * M_E * J_EV * (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2])
    tosum[0:n, 3] = (e_kernel * w) / w
    b.big_curr_xbins_list[0][:] = 0
    b.big_curr_xbins_list[0][0:n] = ((data[0:n, 0] + 0.5 * dx) / dx).astype(int)
    b.Nc_list[0] = n
    rs.DRAWS.reset(seed + 1)
    gen = rs.DRAWS.gen

    class _QGen:
        def random(self, shape=None):
            return quant_uniform(gen.random(shape))

    rs.DRAWS.gen = _QGen()
    b.need_to_resample = False
    b._check_for_resampling()
    need = bool(b.need_to_resample)
    counts = np.stack([np.array(getattr(b, "bin_write_inds_" + nm + "_ar")) for nm in names])
    rs.DRAWS.draws = []
    b._do_resampling()
    draws = rs.DRAWS.draws
    # split draws are 'choice_uniform', merge draws are 'rand', in processing order
    kinds = np.array([0 if d[0] == "choice_uniform" else 1 for d in draws], dtype=np.int32)
    lens = np.array([len(d[1]) for d in draws], dtype=np.int64)
    flat = np.concatenate([d[1] for d in draws]) if draws else np.zeros(0)
    Na = b.Nc_list[0]
    np.savez_compressed(
        os.path.join(HERE, f"resample_{variant}.npz"),
        x=x, v=v, w=w, N=N, L=L, edges=np.array(edges, dtype=np.float64), targets=T,
        min_wt=b.min_wt_allow, need=need, counts=counts,
        draw_kind=kinds, draw_len=lens, draw_u=flat,
        out_n=Na, out_data=np.array(data[0:Na, :]), out_tosum=np.array(tosum[0:Na, :]),
        out_curr=np.array(b.big_curr_xbins_list[0][0:Na]), out_forE=np.array(b.big_forE_xbins_list[0][0:Na]),
    )
    print("resample", variant, "n", n, "need", need, "->", Na, "draw groups", len(draws))


# ------------------------------------------------------------------------------------------
# field solve and ion fluid (next-row kernels)
# ------------------------------------------------------------------------------------------

def case_field(seed, gridpts=65):
    ns = rs.load_variant("1bin")
    rng = np.random.default_rng(seed)
    rs.DRAWS.reset(seed)
    b = ns.BoltzmannDSMC(1, "golden_", 0, 640, gridpts, 4, 1, False, 1, 50000.0, 1 << 30)
    N = b.N
    ne = rng.uniform(0.5e8, 2e8, N + 1)
    ni = ne * rng.uniform(0.9, 1.1, N + 1)
    t = 3.3e-8
    E0 = np.zeros(N)
    V0a = np.zeros(N - 1)
    Va, Ea = ns.ef.EF_kernel(E0, ne, ni, t, V0a, np.zeros(N - 1), b.Vc_diag, b.Vc_lower_diag, np.zeros(N + 1),
                             N, b.dx, b.epsilon, b.V0, b.freq)
    ni2 = ni.copy()
    Ji = np.zeros(N)
    ns2 = np.zeros(N + 1)
    ni2, ns2, brk = ns.heavies.heavies_kernel_fluid(0, Ea.copy(), ni2, np.zeros(N + 1), Ji, ns2, np.zeros(N + 1),
                                                    np.zeros(N), b.dx, b.dt_big, b.mu_i, b.D_i, b.D_s, N)
    np.savez_compressed(os.path.join(HERE, "field.npz"), N=N, L=L, dx=b.dx, ne=ne, ni=ni, t=t, eps0=b.epsilon,
                        V0=b.V0, freq=b.freq, V=np.array(Va), E=np.array(Ea), dt=b.dt_big, mu_i=b.mu_i,
                        D_i=b.D_i, ni_out=np.array(ni2), Ji=np.array(Ji), brk=brk)
    print("field N", N)


# ------------------------------------------------------------------------------------------
# the step loop's cycle averages and per-cycle output files (BoltzmannDSMC.run)
# ------------------------------------------------------------------------------------------

def case_cycle(seed, gridpts=9, Nc_arg=96, spc=3, cycles=2):
    """The reference's own run loop (boltzmann.py:565-716) for two short RF cycles: every
    step's grid fields as the loop accumulates them (recorded around its EF_kernel call),
    and the bytes of every file its data_write (data_write_1D.py:3-75) wrote."""
    import tempfile
    ns = rs.load_variant("1bin")
    rs.DRAWS.reset(seed)
    tmp = tempfile.mkdtemp(prefix="bz_cycle_")
    name = os.path.join(tmp, "ref_")
    steps = spc * cycles
    b = ns.BoltzmannDSMC(steps, name, 0, Nc_arg, gridpts, 4, 1, False, 1000, 400.0, spc)
    # two thirds of the electrons at 40 eV, so that the short run ionizes (the ion
    # production file then has something to reset between cycles)
    rng = np.random.default_rng(seed)
    n = b.Nc_list[0]
    hot = np.arange(n) % 3 != 0
    data, tosum = b.big_data_ar_list[0], b.big_tosum_ar_list[0]
    vh = speed_for_energy(np.full(int(hot.sum()), 40.0))[:, None] * iso_dirs(rng, int(hot.sum()))
    data[np.nonzero(hot)[0], 3:6] = vh
    v = np.asarray(data[0:n, 3:6])
    tosum[0:n, 3] = 0.5 * M_E * J_EV * (v * v).sum(axis=1)
    rec = {"ne": [], "ni": [], "Te": [], "E": [], "ni_src": []}
    ef = b.EF_kernel

    def ef_rec(*a):
        V, E = ef(*a)
        rec["ne"].append(np.array(b.ne_ar, dtype=np.float64))
        rec["ni"].append(np.array(b.ni_ar, dtype=np.float64))
        rec["Te"].append(np.array(b.Te_ar, dtype=np.float64))
        rec["E"].append(np.array(E, dtype=np.float64))
        rec["ni_src"].append(np.array(b.ni_src, dtype=np.float64))
        return V, E

    b.EF_kernel = ef_rec
    b.run(steps, name, 0)
    files = sorted(os.listdir(tmp))
    blobs = {}
    for f in files:
        with open(os.path.join(tmp, f), "rb") as fh:
            blobs[f[len("ref_"):]] = np.frombuffer(fh.read(), dtype=np.uint8)
    out = {f"rec_{k}": np.stack(v) for k, v in rec.items()}
    out.update({f"file_{k}": v for k, v in blobs.items()})
    np.savez_compressed(os.path.join(HERE, "cycle.npz"), spc=spc, cycles=cycles, N=b.N,
                        file_names=np.array(sorted(blobs)), **out)
    for f in files:
        os.remove(os.path.join(tmp, f))
    os.rmdir(tmp)
    print("cycle: steps", steps, "files", len(blobs))


def main():
    if "--cycle" in sys.argv:  # only the run-loop fixture
        case_cycle(seed=50)
        return
    ns = rs.load_variant("1bin")
    # 1 Torr, dt = tau/400: many collisions and ionizations per step
    case_push(ns, "push_1torr.npz", 3.22e16 * 1.0 * 1e6, TAU / 400.0, Te=8.0, seed=11)
    # 0.1 Torr, dt = tau/1e5 (the reference's testrun.sh settings): rare collisions
    case_push(ns, "push_0p1torr.npz", 3.22e16 * 0.1 * 1e6, TAU / 1e5, Te=3.0, seed=12, efield=300.0)
    for i, var in enumerate(("1bin", "3bin", "5bin")):
        case_bins(var, seed=20 + i)
    for i, var in enumerate(("1bin", "3bin", "5bin")):
        case_resample(var, seed=30 + i)
    case_field(seed=40)
    case_cycle(seed=50)


if __name__ == "__main__":
    main()
