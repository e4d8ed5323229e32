"""GPU parity of the fused push + collide + deposit + compaction kernel.

Against the reference (golden vectors from its own source, replayed random numbers,
the reference's cross-section fits): float64 kernel to 1e-12, float32 kernel to 1e-6
relative (velocities relative to the particle's speed), deposited moments to 1e-5,
counts exact. Against the C oracle with Philox random numbers and the analytic
n*sigma table at larger sizes, particles whose float32/float64 decision is genuinely
ambiguous (decision uniform or new position within 1e-5 of a boundary) are removed
from the input first.
"""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from boltzmann_gb300 import _lib, kernels as K, xsec  # noqa: E402
from oracle import oracle as O  # noqa: E402

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DT = {"f32": torch.float32, "f64": torch.float64}


def golden(name):
    return np.load(os.path.join(G, name))


def gpu_push(g_x, g_v, g_w, E, params, dtype, R=None, gas=None, cap_factor=3, deposit=True):
    n = len(g_x)
    src = K.ParticleSet(max(n, 1), dtype)
    dst = K.ParticleSet(cap_factor * max(n, 1), dtype)
    src.load(g_x, g_v[:, 0], g_v[:, 1], g_v[:, 2], g_w)
    Et = torch.as_tensor(np.asarray(E), dtype=dtype, device="cuda")
    mom = torch.zeros(4, params.n_nodes, dtype=torch.float64, device="cuda") if deposit else None
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    ws = K.Workspace()
    Rt = None if R is None else torch.as_tensor(R, dtype=torch.float64, device="cuda").contiguous()
    gt = None if gas is None else torch.as_tensor(gas, dtype=torch.float64, device="cuda").contiguous()
    K.electron_kernel(params, src, dst, Et, st, ws, moments=mom, replay_R=Rt, replay_gas=gt)
    torch.cuda.synchronize()
    cnt = dst.cnt.cpu().numpy()
    out = dst.to_numpy(int(cnt[2]))
    return cnt, out, (None if mom is None else mom.cpu().numpy()), int(st.item())


def node_allowance(ref_x, vals, L, N, bnf, f32):
    """Per-node moment allowance for float32 positions: a particle whose reference
    position lies within float32 rounding (4 ulp) of a node boundary may be deposited
    on either side, so its contribution is allowed on both neighbouring nodes."""
    allow = np.zeros(N + 1)
    if not f32:
        return allow
    dx = L / N
    s = (ref_x + 0.5 * dx) / dx  # node boundaries at integer s
    near = np.abs(s - np.rint(s)) * dx < 4 * np.spacing(np.float32(1.0)) * np.maximum(np.abs(ref_x), dx)
    k = np.rint(s).astype(int)
    for kk, v in zip(k[near], np.abs(vals[near])):
        for nd in (kk - 1, kk):
            if 0 <= nd <= N:
                allow[nd] += v
    return allow


def check_moments(mom, ref, tol, allow=None):
    a = 0.0 if allow is None else allow
    err = np.abs(mom - ref)
    lim = tol * np.abs(ref) + tol * np.abs(ref).max() + a + 1e-300
    assert np.all(err <= lim), f"moment mismatch at nodes {np.nonzero(err > lim)[0][:10]}: {err[err > lim][:5]}"


def params_for(g, xs_mode, flags=_lib.QUIRK_DEAD_IONFLAG, **kw):
    N = int(g["N"])
    L = float(g["L"])
    return K.make_params(n_faces=N, n_nodes=N + 1, bnf=int(g["bnf"]), advect=1, L=L, dx=L / N, dt=float(g["dt"]),
                         nn=float(g["nn"]), xs_mode=xs_mode, flags=flags, **kw)


QM100 = (1.602 * 1e-19 / (9.10938 * 1e-31)) * 100.0


def velocity_scale(x_in, v_in, w_in, alive_after_push, E, dt, L, N, child_v):
    """Magnitude scale of each output particle's float32 velocity update: survivors
    (input order) |v_in| + |E kick|, children their own speed. A kick can nearly cancel
    the velocity, and float32 rounds the terms, not the small result."""
    dx = L / N
    face = np.clip((x_in / dx).astype(int), 0, N - 1)
    kick = np.abs(dt * QM100 * np.asarray(E)[face])
    s = np.sqrt((v_in ** 2).sum(axis=1)) + kick
    surv = s[(w_in > 0) & alive_after_push]
    return np.concatenate([surv, np.sqrt((child_v ** 2).sum(axis=1))])


def check_state(out, ref_x, ref_v, ref_w, rtol, dt=0.0, vscale=None):
    """x to rtol of max(|x|, step displacement); v to rtol of its magnitude scale
    (default: the reference speed); w to rtol."""
    speed = np.sqrt((ref_v ** 2).sum(axis=1))
    if vscale is not None:
        speed = np.maximum(speed, vscale)
    scale = np.maximum(np.abs(ref_x), 100.0 * dt * speed)
    xerr = np.abs(out["x"] - ref_x)
    bad = xerr > rtol * scale + 1e-30
    assert not bad.any(), f"x: {bad.sum()} particles beyond {rtol}, max rel {(xerr / scale).max()}"
    for k, f in enumerate(("vx", "vy", "vz")):
        err = np.abs(out[f] - ref_v[:, k])
        bad = err > rtol * speed + 1e-30
        assert not bad.any(), f"{f}: {bad.sum()} particles beyond {rtol} of their speed, max {err.max()}"
    np.testing.assert_allclose(out["w"], ref_w, rtol=rtol, atol=0)


@pytest.mark.parametrize("case", ["push_1torr", "push_0p1torr"])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_push_matches_reference_golden(case, prec):
    g = golden(case + ".npz")
    p = params_for(g, _lib.XS_REF_FITS)
    cnt, out, mom, st = gpu_push(g["x"], g["v"], g["w"], g["E"], p, DT[prec], R=g["R"], gas=g["gas"])
    assert st == 0
    nnew = int(g["Nnew"])
    assert int(cnt[2]) == nnew
    assert int(cnt[1]) == int(g["nni"])
    c_data, c_tosum = g["c_data"], g["c_tosum"]
    rtol = 1e-12 if prec == "f64" else 1e-6
    n = len(g["x"])
    kt = g["k_tosum"]
    vs = velocity_scale(g["x"], g["v"], g["w"], kt[:n, 0] > 0, g["E"], float(g["dt"]), float(g["L"]), int(g["N"]),
                        g["k_data"][n:, 3:6])
    check_state(out, c_data[:, 0], c_data[:, 3:6], c_tosum[:, 0], rtol, dt=float(g["dt"]), vscale=vs)
    mrtol = 1e-12 if prec == "f64" else 1e-5
    N, L = int(g["N"]), float(g["L"])
    col = {"ne": c_tosum[:, 0], "ni_src": c_tosum[:, 0] * 1.0, "nrg": c_tosum[:, 0] * c_tosum[:, 3]}
    for j, k in ((0, "ne"), (1, "ni_src"), (3, "nrg")):
        allow = node_allowance(c_data[:, 0], col[k], L, N, int(g["bnf"]), prec == "f32")
        check_moments(mom[j], g[k], mrtol, allow)
    assert np.all(mom[2] == 0.0)


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_deposit_matches_reference_golden(prec):
    g = golden("push_1torr.npz")
    p = params_for(g, _lib.XS_REF_FITS)
    kd, kt = g["k_data"], g["k_tosum"]
    n = len(kd)
    s = K.ParticleSet(n, DT[prec])
    s.load(kd[:, 0], kd[:, 3], kd[:, 4], kd[:, 5], kt[:, 0])
    flag = torch.as_tensor(kt[:, 1].astype(np.uint8), device="cuda")
    mom = torch.zeros(4, p.n_nodes, dtype=torch.float64, device="cuda")
    K.deposit(p, s, mom, ionflag=flag)
    mom = mom.cpu().numpy()
    tol = 1e-12 if prec == "f64" else 1e-5
    for j, k in ((0, "ne"), (1, "ni_src"), (3, "nrg")):
        np.testing.assert_allclose(mom[j], g[k], rtol=tol, atol=tol * np.abs(g[k]).max())


def philox_case(n, N, seed, prec, gas_sigma, coll_model=_lib.COLL_DIRECT, Te=6.0, tab=None):
    rng = np.random.default_rng(seed)
    L = 2.54
    x = rng.uniform(1e-4, L - 1e-4, n).astype(np.float32).astype(np.float64)
    sig = np.sqrt(Te / (9.10938e-31 * 6.241509e18))
    v = rng.normal(0, sig, (n, 3)).astype(np.float32).astype(np.float64)
    w = rng.uniform(1e4, 1e5, n).astype(np.float32).astype(np.float64)
    E = rng.uniform(-2000, 2000, N).astype(np.float32).astype(np.float64)
    tab = tab or xsec.analytic_argon(2000)
    nn = 3.22e22
    nst = tab.nsigma(nn)
    dt = 1.0 / 13.56e6 / 400
    nu_max = tab.nu_max(nn)
    prec_bits = 64 if prec == "f64" else 32
    op = O.make_params(N, L=L, bnf=4, dt=dt, nn=nn, xs_mode=0, coll_model=coll_model, rng_mode=1,
                       precision=prec_bits, seed=seed, step=7, gas_sigma=gas_sigma, xs_table=nst,
                       xs_emin=tab.emin, xs_emax=tab.emax, nu_max=nu_max, e_exc=tab.e_exc)
    data, tosum = O.soa_to_aos(x, v[:, 0], v[:, 1], v[:, 2], w, cap=3 * n)
    _, margin = O.push_margin(op, data.copy(), tosum.copy(), n, E)
    w = np.where(margin < 1e-5, 0.0, w)  # ambiguous between float32 and float64: drop from both
    data, tosum = O.soa_to_aos(x, v[:, 0], v[:, 1], v[:, 2], w, cap=3 * n)
    nni = O.push(op, data, tosum, n, E)
    vs = velocity_scale(x, v, w, tosum[:n, 0] > 0, E, dt, L, N, data[n:n + nni, 3:6])
    mom, nnew = O.post(op, data, tosum, n + nni)
    tab_t = torch.as_tensor(nst, device="cuda")
    gp = K.make_params(n_faces=N, n_nodes=N + 1, bnf=4, advect=1, L=L, dx=L / N, dt=dt, nn=nn,
                       gas_sigma=gas_sigma, e_exc=tab.e_exc, nu_max=nu_max, xs_mode=_lib.XS_TABLE,
                       coll_model=coll_model, xs_table=tab_t, xs_emin=tab.emin, xs_emax=tab.emax, seed=seed, step=7,
                       flags=_lib.QUIRK_DEAD_IONFLAG)
    gp._keep = tab_t
    return x, v, w, E, gp, (data, tosum, nni, nnew, mom, vs)


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("coll_model", [_lib.COLL_DIRECT, _lib.COLL_NULL])
def test_push_philox_table_matches_oracle(prec, coll_model):
    x, v, w, E, gp, (data, tosum, nni, nnew, mom_o, vs) = philox_case(120_000, 256, 5, prec, 6.74e4, coll_model)
    cnt, out, mom, st = gpu_push(x, v, w, E, gp, DT[prec])
    assert st == 0
    assert int(cnt[1]) == nni
    assert int(cnt[2]) == nnew
    rtol = 1e-10 if prec == "f64" else 1e-6
    check_state(out, data[:nnew, 0], data[:nnew, 3:6], tosum[:nnew, 0], rtol, dt=gp.dt, vscale=vs)
    mt = 1e-10 if prec == "f64" else 1e-5
    xw = data[:nnew, 0]
    col = {0: tosum[:nnew, 0], 1: tosum[:nnew, 0], 3: tosum[:nnew, 0] * tosum[:nnew, 3]}
    for j in (0, 1, 3):
        allow = node_allowance(xw, col[j], gp.L, gp.n_faces, 4, prec == "f32")
        check_moments(mom[j], mom_o[j], mt, allow)


def lxcat_text(rng):
    """An LXCat-style cross-section file (ELASTIC / EXCITATION / IONIZATION blocks: a
    header, the species, a mass-ratio or threshold line, a table between dashed lines)
    holding argon-like cross sections tabulated at irregular energies, with comment lines
    in between, as the format carries them."""
    def block(kind, thr_line, e, sig):
        rows = "\n".join(f"{a:.6e}\t{b:.6e}" for a, b in zip(e, sig))
        return (f"{kind}\nAr\n {thr_line}\nSPECIES: e / Ar\nPROCESS: E + Ar -> E + Ar, {kind.title()}\n"
                f"COLUMNS: Energy (eV) | Cross section (m2)\n-----------------------------\n{rows}\n"
                f"-----------------------------\n\n")
    e = np.sort(np.concatenate([[0.0], 10 ** rng.uniform(-2.2, 3.1, 300)]))
    el = np.minimum(1e-19 * np.maximum(e, 1e-3) ** 0.3, 1.5e-19)
    ex_e = np.concatenate([[11.5], np.sort(11.5 + 10 ** rng.uniform(-3, 3, 150))])
    ex = 3e-21 * np.log(ex_e / 11.5) / (ex_e / 11.5)
    io_e = np.concatenate([[15.76], np.sort(15.76 + 10 ** rng.uniform(-3, 3, 150))])
    io = 3e-20 * np.log(io_e / 15.76) / (io_e / 15.76)
    return ("xxxxxxxx comment lines of the database header xxxxxxxx\n\n" + block("ELASTIC", "1.360000e-5", e, el)
            + block("EXCITATION", "1.150000e+1", ex_e, ex) + block("IONIZATION", "1.576000e+1", io_e, io))


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_push_with_an_ingested_lxcat_table_matches_oracle(prec):
    """Cross sections ingested from LXCat-style text (xsec.read_lxcat, in place of the
    reference's hard-coded fits, electron_kernel_numba.py:66-174) drive the GPU push and the
    oracle alike: same particles, counts exact, states to the push tolerances."""
    tab = xsec.read_lxcat(lxcat_text(np.random.default_rng(77)), n=2000)
    assert abs(tab.e_exc - 11.5) < 1e-12 and np.all(tab.sigma >= 0) and tab.sigma[2].max() > 0
    x, v, w, E, gp, (data, tosum, nni, nnew, mom_o, vs) = philox_case(100_000, 256, 13, prec, 6.74e4, tab=tab)
    cnt, out, mom, st = gpu_push(x, v, w, E, gp, DT[prec])
    assert st == 0
    assert int(cnt[1]) == nni and nni > 0
    assert int(cnt[2]) == nnew
    rtol = 1e-10 if prec == "f64" else 1e-6
    check_state(out, data[:nnew, 0], data[:nnew, 3:6], tosum[:nnew, 0], rtol, dt=gp.dt, vscale=vs)


def test_push_is_deterministic():
    x, v, w, E, gp, _ = philox_case(50_000, 128, 9, "f32", 6.74e4)
    a = gpu_push(x, v, w, E, gp, torch.float32)
    b = gpu_push(x, v, w, E, gp, torch.float32)
    assert np.array_equal(a[0], b[0])
    for f in ("x", "vx", "vy", "vz", "w"):
        assert np.array_equal(a[1][f], b[1][f])


def test_push_empty_and_tiny():
    x, v, w, E, gp, _ = philox_case(5, 16, 3, "f32", 0.0)
    for n in (0, 1, 5):
        cnt, out, mom, st = gpu_push(x[:n], v[:n], w[:n], E, gp, torch.float32)
        assert st == 0
        assert int(cnt[2]) <= 2 * n


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_dense_push_through_segments_matches_lookback(prec):
    """bz_push_collide_* with the fast workspace (the segmented kernel over the array read
    as segments, then a gather into the reference order) against the single-pass look-back
    push: the same particles in the same order, the same counts, the moments up to the
    float summation order."""
    x, v, w, E, gp, _ = philox_case(150_000, 256, 9, prec, 6.74e4)
    res = []
    for fast in (False, True):
        n = len(x)
        src = K.ParticleSet(n, DT[prec])
        dst = K.ParticleSet(3 * n, DT[prec])
        src.load(x, v[:, 0], v[:, 1], v[:, 2], w)
        mom = torch.zeros(4, gp.n_nodes, dtype=torch.float64, device="cuda")
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        K.electron_kernel(gp, src, dst, torch.as_tensor(E, dtype=DT[prec], device="cuda"), st, K.Workspace(),
                          moments=mom, fast=fast)
        torch.cuda.synchronize()
        assert int(st.item()) == 0
        cnt = dst.cnt.cpu().numpy()
        res.append((cnt, dst.to_numpy(int(cnt[2])), mom.cpu().numpy()))
    (c1, o1, m1), (c2, o2, m2) = res
    np.testing.assert_array_equal(c1[:3], c2[:3])
    assert c1[1] > 0  # children were appended
    for f in K.ParticleSet.FIELDS:
        np.testing.assert_array_equal(o2[f], o1[f])
    for j in (0, 1, 3):
        np.testing.assert_allclose(m2[j], m1[j], rtol=1e-5, atol=1e-6 * np.abs(m1[j]).max())


def test_push_capacity_flag():
    """Too small an output buffer: the kernel drops particles and raises BZ_DEV_CAPACITY,
    it does not write out of bounds."""
    x, v, w, E, gp, _ = philox_case(4096, 64, 4, "f32", 0.0)
    n = len(x)
    src = K.ParticleSet(n, torch.float32)
    dst = K.ParticleSet(n // 2, torch.float32)
    src.load(x, v[:, 0], v[:, 1], v[:, 2], w)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    K.electron_kernel(gp, src, dst, torch.as_tensor(E, dtype=torch.float32, device="cuda"), st, K.Workspace())
    torch.cuda.synchronize()
    assert int(st.item()) & _lib.DEV_CAPACITY


def test_device_philox_known_answer():
    """The device Philox4x32-10 (plain rounds and the interleaved pair with round keys)
    gives the Random123 known-answer vectors and agrees with the oracle's Philox on random
    counters and keys; so does the 7-round form the push draws from."""
    ctr = [[0, 0, 0, 0], [0xffffffff] * 4, [0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344]]
    key = [[0, 0], [0xffffffff] * 2, [0xa4093822, 0x299f31d0]]
    kat = [[0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8], [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd],
           [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]]
    for variant in (0, 1, 2):
        assert K.philox(ctr, key, variant).tolist() == kat, variant
    rng = np.random.default_rng(12)
    c = rng.integers(0, 2 ** 32, (1000, 4), dtype=np.uint64)
    k = rng.integers(0, 2 ** 32, (1000, 2), dtype=np.uint64)
    got = K.philox(c, k, 1)
    for i in range(0, 1000, 37):
        assert list(got[i]) == list(O.philox([int(v) for v in c[i]], [int(v) for v in k[i]])), i
    # the push's draws: the same generator with 7 rounds (Philox4x32-7), device and oracle
    got = K.philox(c, k, 3)
    for i in range(0, 1000, 37):
        assert list(got[i]) == list(O.philox([int(v) for v in c[i]], [int(v) for v in k[i]], rounds=7)), i
    assert got[0].tolist() != K.philox(c[:1], k[:1], 1)[0].tolist()
