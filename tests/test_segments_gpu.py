"""GPU parity of the segmented particle state used by the solver's hot loop.

One segment reproduces the reference's order exactly (survivors, then children), so it
is checked against the golden vectors like the dense push; many segments are checked
against the oracle run on the slot-indexed array (Philox counters are slot indices);
repack, binning, resampling and deposit are checked against their dense counterparts.
"""
import ctypes
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from boltzmann_gb300 import _lib, kernels as K, xsec  # noqa: E402
from oracle import oracle as O  # noqa: E402

from test_push_gpu import (check_moments, check_state, golden, node_allowance, params_for,  # noqa: E402
                           velocity_scale)

DT = {"f32": torch.float32, "f64": torch.float64}


def seg_push(seg_in, p, E, R=None, gas=None):
    out = K.SegmentSet(seg_in.nseg, seg_in.half, seg_in.dtype)
    mom = torch.zeros(4, p.n_nodes, dtype=torch.float64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    fl = torch.zeros(1, dtype=torch.int32, device="cuda")
    Et = torch.as_tensor(np.asarray(E), dtype=seg_in.dtype, device="cuda")
    Rt = None if R is None else torch.as_tensor(R, dtype=torch.float64, device="cuda").contiguous()
    gt = None if gas is None else torch.as_tensor(gas, dtype=torch.float64, device="cuda").contiguous()
    K.seg_electron_kernel(p, seg_in, out, Et, st, fl, K.Workspace(), moments=mom, replay_R=Rt, replay_gas=gt)
    torch.cuda.synchronize()
    return out, mom.cpu().numpy(), int(st.item()), int(fl.item())


@pytest.mark.parametrize("case", ["push_1torr", "push_0p1torr"])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_one_segment_matches_reference_golden(case, prec):
    g = golden(case + ".npz")
    n = len(g["x"])
    seg = K.SegmentSet(1, ((n + 3) // 4) * 4, DT[prec])
    seg.load(g["x"], g["v"][:, 0], g["v"][:, 1], g["v"][:, 2], g["w"])
    # slots equal particle indices in one segment, so R[i] / gas[i] line up
    out, mom, st, fl = seg_push(seg, params_for(g, _lib.XS_REF_FITS), g["E"], g["R"], g["gas"])
    assert st == 0
    c = out.counts.cpu().numpy()
    assert int(c[0] + c[1]) == int(g["Nnew"]) and int(c[1]) == int(g["nni"])
    o = out.to_numpy("runs")
    cd, ct = g["c_data"], g["c_tosum"]
    rtol = 1e-12 if prec == "f64" else 1e-6
    vs = velocity_scale(g["x"], g["v"], g["w"], g["k_tosum"][:n, 0] > 0, g["E"], float(g["dt"]), float(g["L"]),
                        int(g["N"]), g["k_data"][n:, 3:6])
    check_state(o, cd[:, 0], cd[:, 3:6], ct[:, 0], rtol, dt=float(g["dt"]), vscale=vs)
    N, L = int(g["N"]), float(g["L"])
    col = {"ne": ct[:, 0], "ni_src": ct[:, 0], "nrg": ct[:, 0] * ct[:, 3]}
    for j, k in ((0, "ne"), (1, "ni_src"), (3, "nrg")):
        allow = node_allowance(cd[:, 0], col[k], L, N, 4, prec == "f32")
        check_moments(mom[j], g[k], 1e-12 if prec == "f64" else 1e-5, allow)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_many_segments_match_oracle_philox(prec):
    rng = np.random.default_rng(8)
    n, N, L, nseg, half = 100_000, 256, 2.54, 64, 2048
    x = rng.uniform(1e-4, L - 1e-4, n).astype(np.float32).astype(np.float64)
    v = rng.normal(0, 1.3e6, (n, 3)).astype(np.float32).astype(np.float64)
    w = rng.uniform(1e4, 1e5, n).astype(np.float32).astype(np.float64)
    E = rng.uniform(-1500, 1500, N).astype(np.float32).astype(np.float64)
    seg = K.SegmentSet(nseg, half, DT[prec])
    seg.load(x, v[:, 0], v[:, 1], v[:, 2], w)
    cap = seg.capacity
    # the oracle sees the slot-indexed array: holes are w = 0 particles it drops
    sl = seg.slots("segments")
    xs_ = np.zeros(cap); vxs = np.zeros(cap); vys = np.zeros(cap); vzs = np.zeros(cap); ws_ = np.zeros(cap)
    st_np = seg.to_numpy("segments")
    xs_[sl], vxs[sl], vys[sl], vzs[sl], ws_[sl] = st_np["x"], st_np["vx"], st_np["vy"], st_np["vz"], st_np["w"]
    tab = xsec.analytic_argon(2000)
    nn, dt, gas_sigma = 3.22e22, 1.0 / 13.56e6 / 400, 6.74e4
    op = O.make_params(N, L=L, dt=dt, nn=nn, rng_mode=1, precision=64 if prec == "f64" else 32, seed=4, step=3,
                       gas_sigma=gas_sigma, xs_table=tab.nsigma(nn), xs_emin=tab.emin, xs_emax=tab.emax,
                       e_exc=tab.e_exc)
    data, tosum = O.soa_to_aos(xs_, vxs, vys, vzs, ws_, cap=2 * cap)
    _, margin = O.push_margin(op, data.copy(), tosum.copy(), cap, E)
    amb = (margin < 1e-5) & (ws_ > 0)
    ws_[amb] = 0.0
    seg.w[torch.as_tensor(np.nonzero(amb)[0], device="cuda")] = 0.0
    data, tosum = O.soa_to_aos(xs_, vxs, vys, vzs, ws_, cap=2 * cap)
    nni = O.push(op, data, tosum, cap, E)
    vs = velocity_scale(xs_, np.stack([vxs, vys, vzs], 1), ws_, tosum[:cap, 0] > 0, E, dt, L, N,
                        data[cap:cap + nni, 3:6])
    mom_o, nnew = O.post(op, data, tosum, cap + nni)
    xt = torch.as_tensor(tab.nsigma(nn), device="cuda")
    p = K.make_params(n_faces=N, n_nodes=N + 1, bnf=4, advect=1, L=L, dx=L / N, dt=dt, nn=nn, gas_sigma=gas_sigma,
                      e_exc=tab.e_exc, xs_mode=_lib.XS_TABLE, xs_table=xt, xs_emin=tab.emin, xs_emax=tab.emax,
                      flags=_lib.QUIRK_DEAD_IONFLAG, seed=4, step=3)
    out, mom, st, fl = seg_push(seg, p, E)
    assert st == 0
    o = out.to_numpy("runs")
    assert len(o["x"]) == nnew
    assert int(out.counts.cpu().numpy()[1::2].sum()) == nni
    rtol = 1e-10 if prec == "f64" else 1e-6
    check_state(o, data[:nnew, 0], data[:nnew, 3:6], tosum[:nnew, 0], rtol, dt=dt, vscale=vs)
    col = {0: tosum[:nnew, 0], 1: tosum[:nnew, 0], 3: tosum[:nnew, 0] * tosum[:nnew, 3]}
    for j in (0, 1, 3):
        allow = node_allowance(data[:nnew, 0], col[j], L, N, 4, prec == "f32")
        check_moments(mom[j], mom_o[j], 1e-10 if prec == "f64" else 1e-5, allow)


def test_repack_keeps_order_and_balances():
    rng = np.random.default_rng(2)
    torch.manual_seed(2)
    nseg, half = 50, 256
    a = K.SegmentSet(nseg, half)
    c = rng.integers(0, half // 2 + 1, (nseg, 2)).astype(np.int32)  # the total fits run 0 of every segment
    a.counts.copy_(torch.as_tensor(c.reshape(-1), device="cuda"))
    for f in a.FIELDS:
        getattr(a, f).copy_(torch.rand(a.capacity, device="cuda") + 0.5)
    dead = torch.rand(a.capacity, device="cuda") < 0.1
    a.w[dead] = 0.0
    before = a.to_numpy("segments")
    keep = before["w"] != 0
    b = K.SegmentSet(nseg, half)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    K.seg_repack(a, b, st, K.Workspace())
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    after = b.to_numpy("segments")
    for f in a.FIELDS:
        np.testing.assert_array_equal(after[f], before[f][keep])
    cb = b.counts.cpu().numpy().reshape(-1, 2)
    assert cb[:, 1].sum() == 0
    fill = -(-int(keep.sum()) // nseg)
    assert cb[:, 0].max() == min(fill, half)


def test_conditional_repack_skips_without_request():
    a = K.SegmentSet(4, 64)
    a.counts.copy_(torch.tensor([10, 5, 0, 0, 7, 0, 3, 3], dtype=torch.int32, device="cuda"))
    a.w.fill_(1.0)
    b = K.SegmentSet(4, 64)
    b.counts.fill_(-7)
    flags = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    K.seg_repack(a, b, st, K.Workspace(), only_if=flags, clear=flags)
    torch.cuda.synchronize()
    assert b.counts.cpu().tolist() == [-7] * 8  # nothing ran
    flags.fill_(_lib.SEG_NEEDS_REPACK)
    K.seg_repack(a, b, st, K.Workspace(), only_if=flags, clear=flags)
    torch.cuda.synchronize()
    assert int(flags.item()) == 0 and b.n() == 28


def test_rebalance_in_place_matches_repack():
    """bz_seg_rebalance: repack through the scratch set and back in one launch; the
    result equals a plain repack into a fresh set; skipped without the request."""
    rng = np.random.default_rng(4)
    torch.manual_seed(4)
    nseg, half = 40, 512
    a = K.SegmentSet(nseg, half)
    c = rng.integers(0, half // 2 + 1, (nseg, 2)).astype(np.int32)  # the total fits run 0 of every segment
    a.counts.copy_(torch.as_tensor(c.reshape(-1), device="cuda"))
    for f in a.FIELDS:
        getattr(a, f).copy_(torch.rand(a.capacity, device="cuda") + 0.5)
    a.w[torch.rand(a.capacity, device="cuda") < 0.1] = 0.0
    ref = K.SegmentSet(nseg, half)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    K.seg_repack(a, ref, st, K.Workspace())
    scratch = K.SegmentSet(nseg, half)
    flags = torch.zeros(1, dtype=torch.int32, device="cuda")
    before = a.counts.clone()
    K.seg_rebalance(a, scratch, st, K.Workspace(), only_if=flags, clear=flags)
    torch.cuda.synchronize()
    assert torch.equal(a.counts, before)  # no request: nothing ran
    flags.fill_(_lib.SEG_NEEDS_REPACK)
    K.seg_rebalance(a, scratch, st, K.Workspace(), only_if=flags, clear=flags)
    torch.cuda.synchronize()
    assert int(st.item()) == 0 and int(flags.item()) == 0
    np.testing.assert_array_equal(a.counts.cpu().numpy(), ref.counts.cpu().numpy())
    got, want = a.to_numpy("segments"), ref.to_numpy("segments")
    for f in a.FIELDS:
        np.testing.assert_array_equal(got[f], want[f])


@pytest.mark.parametrize("variant", ["3bin", "5bin"])
def test_seg_bin_and_resample_match_dense(variant):
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", f"resample_{variant}.npz"))
    N, L = int(g["N"]), float(g["L"])
    x, v, w = g["x"], g["v"], g["w"]
    n = len(x)
    T = g["targets"]
    nb = len(T)
    edges = g["edges"]
    p = K.make_params(n_faces=N, n_nodes=N + 1, bnf=4, advect=1, L=L, dx=L / N, dt=1e-12, nn=3.22e22,
                      flags=_lib.QUIRK_SPLIT_WRAP | _lib.QUIRK_TRIGGER_LAST)
    nkeys = (N + 1) * nb
    seg = K.SegmentSet(1, ((4 * n + 3) // 4) * 4)
    seg.load(x, v[:, 0], v[:, 1], v[:, 2], w)
    ed = torch.as_tensor(np.asarray(edges, dtype=np.float64), device="cuda")
    perm = torch.zeros(seg.capacity, dtype=torch.int32, device="cuda")
    offs = torch.zeros(nkeys + 1, dtype=torch.int32, device="cuda")
    cnts = torch.zeros(nkeys, dtype=torch.int32, device="cuda")
    hw = torch.zeros(nkeys, dtype=torch.int32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    fl = torch.zeros(1, dtype=torch.int32, device="cuda")
    ws = K.Workspace()
    K.seg_bin_particles(p, seg, ed, float(g["min_wt"]), perm, offs, cnts, hw, st, ws)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(cnts.cpu().numpy().reshape(N + 1, nb).T, g["counts"])
    app = K.ParticleSet(4 * n)
    out = K.SegmentSet(1, seg.half)
    tg = torch.as_tensor(np.asarray(T, dtype=np.int32), device="cuda")
    mp = torch.as_tensor((10 * T).astype(np.int32), device="cuda")
    ru = torch.as_tensor(g["draw_u"], device="cuda")
    need = torch.zeros(1, dtype=torch.int32, device="cuda")
    K.seg_resample(p, seg, app, out, nb, tg, mp, float(g["min_wt"]), 0.5, 3.0, 0.6, perm, offs, cnts, hw, st, fl, ws,
                   need=need, replay_u=ru)
    torch.cuda.synchronize()
    assert int(st.item()) == 0 and int(need.item()) == int(g["need"])
    o = out.to_numpy("runs")
    assert len(o["x"]) == int(g["out_n"])
    od, ot = g["out_data"], g["out_tosum"]
    np.testing.assert_allclose(o["x"], od[:, 0], rtol=2e-6)
    np.testing.assert_allclose(o["w"], ot[:, 0], rtol=2e-6)


def test_load_refuses_more_than_the_segments_hold():
    seg = K.SegmentSet(2, 8)
    with pytest.raises(RuntimeError):
        seg.load(np.ones(20), np.ones(20), np.ones(20), np.ones(20), np.ones(20))


def test_seg_deposit_matches_dense():
    rng = np.random.default_rng(5)
    n, N = 50_000, 128
    x = rng.uniform(0.01, 2.53, n)
    v = rng.normal(0, 1e6, (n, 3))
    w = rng.uniform(1, 2, n)
    p = K.make_params(n_faces=N, n_nodes=N + 1, bnf=4, advect=1, L=2.54, dx=2.54 / N, dt=1e-12, nn=1e22)
    seg = K.SegmentSet(80, 1024)
    seg.load(x, v[:, 0], v[:, 1], v[:, 2], w)
    dense = K.ParticleSet(n)
    dense.load(x, v[:, 0], v[:, 1], v[:, 2], w)
    m1 = torch.zeros(4, N + 1, dtype=torch.float64, device="cuda")
    m2 = torch.zeros_like(m1)
    K.seg_deposit(p, seg, m1)
    K.deposit(p, dense, m2)
    torch.cuda.synchronize()
    np.testing.assert_allclose(m1.cpu().numpy(), m2.cpu().numpy(), rtol=1e-5, atol=1e-9)


def test_deposit_grid_in_the_workspace_matches_shared_memory():
    """With a workspace of bz_seg_push_workspace_nodes bytes the float32 1D deposit sums into
    per-CTA grids in global memory; with the minimal workspace, into shared memory. The
    particles are identical, the moments equal up to the float32 summation order."""
    rng = np.random.default_rng(23)
    n, N, L, nseg, half = 150_000, 256, 2.54, 96, 2048
    x = rng.uniform(1e-4, L - 1e-4, n)
    v = rng.normal(0, 1.4e6, (n, 3))
    w = rng.uniform(1e4, 1e5, n)
    E = torch.as_tensor(rng.uniform(-1200, 1200, N), dtype=torch.float32, device="cuda")
    seg = K.SegmentSet(nseg, half, torch.float32)
    seg.load(x, v[:, 0], v[:, 1], v[:, 2], w)
    tab = xsec.analytic_argon(2000)
    nn = 3.22e22
    xt = torch.as_tensor(tab.nsigma(nn), device="cuda")
    p = K.make_params(n_faces=N, n_nodes=N + 1, bnf=4, advect=1, L=L, dx=L / N, dt=1.0 / 13.56e6 / 400, nn=nn,
                      gas_sigma=6.74e4, e_exc=tab.e_exc, xs_mode=_lib.XS_TABLE, xs_table=xt, xs_emin=tab.emin,
                      xs_emax=tab.emax, flags=_lib.QUIRK_DEAD_IONFLAG, seed=4, step=3)
    lib = _lib.load()
    small, big = lib.bz_seg_push_workspace(), lib.bz_seg_push_workspace_nodes(N + 1)
    assert small == 256 and big > small + 152 * (N + 1) * 8
    res = []
    for nbytes in (small, big):
        out = K.SegmentSet(nseg, half, torch.float32)
        mom = torch.zeros(4, N + 1, dtype=torch.float64, device="cuda")
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        fl = torch.zeros(1, dtype=torch.int32, device="cuda")
        ws = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
        K.call("bz_seg_push_collide_f32", ctypes.byref(p), seg.struct(), out.struct(), K._ptr(E), None, None,
               K._ptr(mom), None, K._ptr(ws), nbytes, K._ptr(fl), K._ptr(st), K._stream())
        torch.cuda.synchronize()
        assert int(st.item()) == 0
        res.append((out.to_numpy("segments"), out.counts.cpu().numpy(), mom.cpu().numpy()))
    (o1, c1, m1), (o2, c2, m2) = res
    np.testing.assert_array_equal(c1, c2)
    for f in K.SegmentSet.FIELDS:
        np.testing.assert_array_equal(o1[f], o2[f])
    assert m1[0].sum() > 0
    for j in (0, 1, 3):
        np.testing.assert_allclose(m2[j], m1[j], rtol=1e-5, atol=1e-6 * np.abs(m1[j]).max())


def test_every_cta_shape_gives_the_same_particles():
    """The push's CTA shapes (bz_seg_push_select) change only the float summation order
    of the moments: particles and counts are identical."""
    rng = np.random.default_rng(19)
    n, N, L, nseg, half = 120_000, 512, 2.54, 96, 2048
    x = rng.uniform(1e-4, L - 1e-4, n)
    v = rng.normal(0, 1.4e6, (n, 3))
    w = rng.uniform(1e4, 1e5, n)
    E = rng.uniform(-1200, 1200, N)
    seg = K.SegmentSet(nseg, half, torch.float32)
    seg.load(x, v[:, 0], v[:, 1], v[:, 2], w)
    tab = xsec.analytic_argon(2000)
    nn = 3.22e22
    xt = torch.as_tensor(tab.nsigma(nn), device="cuda")
    p = K.make_params(n_faces=N, n_nodes=N + 1, bnf=4, advect=1, L=L, dx=L / N, dt=1.0 / 13.56e6 / 400, nn=nn,
                      gas_sigma=6.74e4, e_exc=tab.e_exc, xs_mode=_lib.XS_TABLE, xs_table=xt, xs_emin=tab.emin,
                      xs_emax=tab.emax, flags=_lib.QUIRK_DEAD_IONFLAG, seed=2, step=7)
    shapes = K.seg_push_shapes()
    assert len(shapes) >= 2 and shapes[0] == (512, 1, 2, True)
    # the push's own counter of pushed particles
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    tmp = K.SegmentSet(nseg, half, torch.float32)
    st0 = torch.zeros(1, dtype=torch.int32, device="cuda")
    fl0 = torch.zeros(1, dtype=torch.int32, device="cuda")
    for _ in range(2):
        K.seg_electron_kernel(p, seg, tmp, torch.as_tensor(E, dtype=torch.float32, device="cuda"), st0, fl0,
                              K.Workspace(), n_pushed=cnt)
    assert int(cnt.item()) == 2 * seg.n() == 2 * n
    ref = None
    try:
        for k in range(len(shapes)):
            K.select_seg_push_shape(k)
            out, mom, st, fl = seg_push(seg, p, E)
            assert st == 0
            o = out.to_numpy("segments")
            c = out.counts.cpu().numpy()
            if ref is None:
                ref = (o, c, mom)
                continue
            np.testing.assert_array_equal(c, ref[1])
            for f in K.SegmentSet.FIELDS:
                np.testing.assert_array_equal(o[f], ref[0][f])
            for j in (0, 1, 3):
                np.testing.assert_allclose(mom[j], ref[2][j], rtol=1e-5, atol=1e-6 * np.abs(ref[2][j]).max())
    finally:
        K.select_seg_push_shape(0)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_ragged_segments_match_oracle_philox(prec):
    """Segments filled unevenly — empty, run 0 full, run 1 full, one particle, both runs
    partly filled — push like the oracle on the slot-indexed array (holes are w = 0)."""
    rng = np.random.default_rng(23)
    N, L, half = 128, 2.54, 256
    pattern = [(0, 0), (half, 0), (0, half), (half - 1, 1), (1, 0), (0, 1), (100, 100), (0, 0), (37, 0),
               (half // 2, half // 2)]
    nseg = len(pattern)
    seg = K.SegmentSet(nseg, half, DT[prec])
    cap = seg.capacity
    cnt = np.array(pattern, dtype=np.int32).reshape(-1)
    seg.counts.copy_(torch.as_tensor(cnt, device="cuda"))
    xs_, vxs, vys, vzs, ws_ = (np.zeros(cap) for _ in range(5))
    for s, (a, b) in enumerate(pattern):
        for run, c in ((0, a), (1, b)):
            lo = s * 2 * half + run * half
            sl = slice(lo, lo + c)
            xs_[sl] = rng.uniform(1e-4, L - 1e-4, c)
            vxs[sl], vys[sl], vzs[sl] = rng.normal(0, 1.3e6, (3, c))
            ws_[sl] = rng.uniform(1e4, 1e5, c)
    f32 = lambda a: a.astype(np.float32).astype(np.float64)
    xs_, vxs, vys, vzs, ws_ = (f32(a) for a in (xs_, vxs, vys, vzs, ws_))
    E = f32(rng.uniform(-1500, 1500, N))
    tab = xsec.analytic_argon(2000)
    nn, dt, gas_sigma = 3.22e22, 1.0 / 13.56e6 / 400, 6.74e4
    op = O.make_params(N, L=L, dt=dt, nn=nn, rng_mode=1, precision=64 if prec == "f64" else 32, seed=6, step=2,
                       gas_sigma=gas_sigma, xs_table=tab.nsigma(nn), xs_emin=tab.emin, xs_emax=tab.emax,
                       e_exc=tab.e_exc)
    data, tosum = O.soa_to_aos(xs_, vxs, vys, vzs, ws_, cap=2 * cap)
    _, margin = O.push_margin(op, data.copy(), tosum.copy(), cap, E)
    ws_[(margin < 1e-5) & (ws_ > 0)] = 0.0  # too close to a decision boundary to compare
    for f, a in zip(seg.FIELDS, (xs_, vxs, vys, vzs, ws_)):
        getattr(seg, f).copy_(torch.as_tensor(a, dtype=DT[prec], device="cuda"))
    data, tosum = O.soa_to_aos(xs_, vxs, vys, vzs, ws_, cap=2 * cap)
    nni = O.push(op, data, tosum, cap, E)
    vs = velocity_scale(xs_, np.stack([vxs, vys, vzs], 1), ws_, tosum[:cap, 0] > 0, E, dt, L, N,
                        data[cap:cap + nni, 3:6])
    mom_o, nnew = O.post(op, data, tosum, cap + nni)
    xt = torch.as_tensor(tab.nsigma(nn), device="cuda")
    p = K.make_params(n_faces=N, n_nodes=N + 1, bnf=4, advect=1, L=L, dx=L / N, dt=dt, nn=nn, gas_sigma=gas_sigma,
                      e_exc=tab.e_exc, xs_mode=_lib.XS_TABLE, xs_table=xt, xs_emin=tab.emin, xs_emax=tab.emax,
                      flags=_lib.QUIRK_DEAD_IONFLAG, seed=6, step=2)
    out, mom, st, fl = seg_push(seg, p, E)
    assert st == 0
    o = out.to_numpy("runs")
    assert len(o["x"]) == nnew
    assert int(out.counts.cpu().numpy()[1::2].sum()) == nni
    oc = out.counts.cpu().numpy().reshape(-1, 2)
    assert np.all(oc[[0, 7], :] == 0)  # empty segments stay empty
    rtol = 1e-10 if prec == "f64" else 1e-6
    check_state(o, data[:nnew, 0], data[:nnew, 3:6], tosum[:nnew, 0], rtol, dt=dt, vscale=vs)
    col = {0: tosum[:nnew, 0], 1: tosum[:nnew, 0], 3: tosum[:nnew, 0] * tosum[:nnew, 3]}
    for j in (0, 1, 3):
        allow = node_allowance(data[:nnew, 0], col[j], L, N, 4, prec == "f32")
        check_moments(mom[j], mom_o[j], 1e-10 if prec == "f64" else 1e-5, allow)


def test_empty_state_through_push_bin_resample_deposit():
    """No particle at all: every stage runs, reports no error and leaves everything empty."""
    N, L, nseg, half, nb = 64, 2.54, 6, 128, 3
    seg = K.SegmentSet(nseg, half)
    tab = xsec.analytic_argon(2000)
    xt = torch.as_tensor(tab.nsigma(3.22e22), device="cuda")
    p = K.make_params(n_faces=N, n_nodes=N + 1, bnf=4, advect=1, L=L, dx=L / N, dt=1e-12, nn=3.22e22,
                      gas_sigma=6.74e4, e_exc=tab.e_exc, xs_mode=_lib.XS_TABLE, xs_table=xt, xs_emin=tab.emin,
                      xs_emax=tab.emax, seed=1, step=1)
    out, mom, st, fl = seg_push(seg, p, np.zeros(N))
    assert st == 0 and out.n() == 0 and not np.any(mom)
    nkeys = (N + 1) * nb
    ed = torch.as_tensor(np.array([4.0, 11.5]), device="cuda")
    perm = torch.full((seg.capacity,), -1, dtype=torch.int32, device="cuda")
    offs = torch.full((nkeys + 1,), -1, dtype=torch.int32, device="cuda")
    cnts = torch.full((nkeys,), -1, dtype=torch.int32, device="cuda")
    hw = torch.full((nkeys,), -1, dtype=torch.int32, device="cuda")
    sts = torch.zeros(1, dtype=torch.int32, device="cuda")
    ws = K.Workspace()
    K.seg_bin_particles(p, out, ed, 0.1, perm, offs, cnts, hw, sts, ws)
    torch.cuda.synchronize()
    assert int(sts.item()) == 0
    assert not cnts.any() and not hw.any() and not offs.any()
    app = K.ParticleSet(16)
    res = K.SegmentSet(nseg, half)
    tg = torch.full((nb,), 100, dtype=torch.int32, device="cuda")
    mp = torch.full((nb,), 1000, dtype=torch.int32, device="cuda")
    need = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    fl2 = torch.zeros(1, dtype=torch.int32, device="cuda")
    K.seg_resample(p, out, app, res, nb, tg, mp, 0.1, 0.5, 3.0, 0.6, perm, offs, cnts, hw, sts, fl2, ws, need=need)
    torch.cuda.synchronize()
    assert int(sts.item()) == 0 and int(need.item()) == 0 and res.n() == 0
    m = torch.zeros(4, N + 1, dtype=torch.float64, device="cuda")
    K.seg_deposit(p, res, m)
    torch.cuda.synchronize()
    assert not m.any()
