"""GPU checks of the in-place placement of a resampling step's appended particles
(bz_seg_place_*) and of the in-place resampling that uses it.

The placement is checked slot by slot against a numpy model of its rule (shares of
min(half - n1, half - live) per segment, first up to ceil(total / nseg) live particles,
then in segment order), its fallback against a plain repack, and the in-place resampling
against the out-of-place one: the same live particles, and on one segment the reference's
order (kept particles, then the appended ones) once the emptied slots are dropped.
"""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from boltzmann_gb300 import _lib, kernels as K, xsec  # noqa: E402

FIELDS = K.SegmentSet.FIELDS


def random_host(rng, nseg, half, fill_max, hole_frac):
    """Host arrays of a segmented state: random run counts (n0 + n1 <= fill_max), random
    columns, a fraction of the slots emptied (w = 0)."""
    c = np.zeros((nseg, 2), dtype=np.int32)
    c[:, 0] = rng.integers(0, fill_max + 1, nseg)
    c[:, 1] = [rng.integers(0, fill_max - a + 1) for a in c[:, 0]]
    cap = nseg * 2 * half
    cols = {f: rng.uniform(0.5, 1.5, cap).astype(np.float32) for f in FIELDS}
    cols["w"][rng.random(cap) < hole_frac] = 0.0
    return c, cols


def to_device(c, cols, nseg, half):
    s = K.SegmentSet(nseg, half)
    s.counts.copy_(torch.as_tensor(c.reshape(-1), device="cuda"))
    for f in FIELDS:
        getattr(s, f).copy_(torch.as_tensor(cols[f], device="cuda"))
    return s


def host_runs(c, cols, half):
    """Per segment, per run, the weights of the occupied slots (holes included)."""
    return [[cols["w"][k * 2 * half + r * half: k * 2 * half + r * half + c[k, r]] for r in range(2)]
            for k in range(c.shape[0])]


def appended(rng, n, cap=None):
    a = K.ParticleSet(max(cap or n, 1))
    a.load(*(rng.uniform(2.0, 3.0, n) for _ in FIELDS))
    return a


def place_model(counts, w_slots, half, n_app):
    """The placement rule on the host: (fallback, per-segment app ranges, first-pass
    total A1, second-pass room R)."""
    nseg = counts.shape[0]
    live = np.array([(w_slots[k][0] != 0).sum() + (w_slots[k][1] != 0).sum() for k in range(nseg)], dtype=np.int64)
    n1 = counts[:, 1].astype(np.int64)
    total = int(live.sum()) + n_app
    fill = max(1, -(-total // nseg))
    cap = np.maximum(0, np.minimum(half - n1, half - live))
    a1 = np.minimum(np.maximum(fill - live, 0), cap)
    room = cap - a1
    p1 = np.concatenate([[0], np.cumsum(a1)])[:-1]
    pe = np.concatenate([[0], np.cumsum(room)])[:-1]
    A1, R = int(a1.sum()), int(room.sum())
    fallback = bool((live > half).any()) or A1 + R < n_app
    ranges = []
    for k in range(nseg):
        l1 = int(max(0, min(a1[k], n_app - p1[k])))
        l2 = int(max(0, min(room[k], n_app - A1 - pe[k]))) if A1 < n_app else 0
        ranges.append(list(range(p1[k], p1[k] + l1)) + list(range(A1 + pe[k], A1 + pe[k] + l2)))
    return fallback, ranges, A1, R


def host_slots(s):
    """Per segment, per run, every column of the occupied slots (holes included)."""
    c = s.counts.cpu().numpy().reshape(-1, 2)
    cols = {f: getattr(s, f).cpu().numpy() for f in FIELDS}
    out = []
    for k in range(s.nseg):
        runs = []
        for r in range(2):
            b = k * 2 * s.half + r * s.half
            runs.append({f: cols[f][b: b + c[k, r]].copy() for f in FIELDS})
        out.append(runs)
    return c, out


def run_place(s, app, n_app, flags_value=_lib.SEG_NEEDS_REPACK):
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    fl = torch.full((1,), flags_value, dtype=torch.int32, device="cuda")
    scratch = K.SegmentSet(s.nseg, s.half)
    K.seg_place(s, app, scratch, st, K.Workspace(), clear=fl)
    torch.cuda.synchronize()
    return int(st.item()), int(fl.item())


@pytest.mark.parametrize("case", ["empty", "first_pass", "second_pass"])
def test_place_follows_its_rule_slot_by_slot(case):
    """first_pass: the even fill takes everything; second_pass: every third segment's
    run 1 is nearly full (of emptied slots), so those take 5 at most and the rest goes out
    in segment order. Run 0 and the old part of run 1 stay untouched, the appended
    particles follow the model's ranges exactly, no segment exceeds half live particles."""
    rng = np.random.default_rng(11)
    nseg, half = 37, 128
    c, cols = random_host(rng, nseg, half, fill_max=100, hole_frac=0.2)
    n_app = {"empty": 0, "first_pass": 700, "second_pass": 1500}[case]
    if case == "second_pass":
        for k in range(0, nseg, 3):
            c[k, 1] = half - 5
            b = k * 2 * half + half
            cols["w"][b: b + half] = 0.0
    fb, ranges, A1, R = place_model(c, host_runs(c, cols, half), half, n_app)
    assert not fb
    assert (A1 < n_app) == (case == "second_pass")
    s = to_device(c, cols, nseg, half)
    app = appended(rng, n_app)
    c0, before = host_slots(s)
    st, fl = run_place(s, app, n_app)
    assert st == 0 and fl == 0
    c1, after = host_slots(s)
    np.testing.assert_array_equal(c1[:, 0], c0[:, 0])
    appc = {f: getattr(app, f).cpu().numpy() for f in FIELDS}
    placed = []
    for k in range(nseg):
        assert c1[k, 1] == c0[k, 1] + len(ranges[k])
        live = (after[k][0]["w"] != 0).sum() + (after[k][1]["w"] != 0).sum()
        assert live <= half  # the next push cannot overflow this segment
        for f in FIELDS:
            np.testing.assert_array_equal(after[k][0][f], before[k][0][f])
            np.testing.assert_array_equal(after[k][1][f][: c0[k, 1]], before[k][1][f])
            np.testing.assert_array_equal(after[k][1][f][c0[k, 1]:], appc[f][ranges[k]])
        placed += ranges[k]
    assert sorted(placed) == list(range(n_app))  # every appended particle exactly once


@pytest.mark.parametrize("why", ["too_little_room", "segment_over_half"])
def test_place_falls_back_to_a_repack(why):
    """When the shares cannot take everything (runs 1 full of emptied slots), or a segment
    already holds more than half live particles, s and app are repacked through scratch and
    back into s: the result equals a plain repack of the same particles into a fresh set."""
    rng = np.random.default_rng(5)
    nseg, half = 20, 64
    if why == "too_little_room":
        # 10 live particles in run 0, 50 emptied slots in run 1: room for 14 per segment,
        # 280 in all, against 500 to place (a repack has room for 1080)
        c = np.zeros((nseg, 2), dtype=np.int32)
        c[:, 0], c[:, 1] = 10, 50
        cols = {f: rng.uniform(0.5, 1.5, nseg * 2 * half).astype(np.float32) for f in FIELDS}
        for k in range(nseg):
            b = k * 2 * half + half
            cols["w"][b: b + 50] = 0.0
        n_app = 500
    else:
        c, cols = random_host(rng, nseg, half, fill_max=40, hole_frac=0.05)
        c[3] = (half, 10)  # 74 slots, the 64 of run 0 all live: more than half
        cols["w"][3 * 2 * half: 3 * 2 * half + half] = 1.0
        n_app = 200
    fb, _, _, _ = place_model(c, host_runs(c, cols, half), half, n_app)
    assert fb
    s = to_device(c, cols, nseg, half)
    app = appended(rng, n_app)
    # the expected result: a plain repack of s and app into a fresh set
    ref = K.SegmentSet(nseg, half)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    K.seg_repack(s, ref, st, K.Workspace(), app=app)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    st_p, fl = run_place(s, app, n_app)
    assert st_p == 0 and fl == 0
    np.testing.assert_array_equal(s.counts.cpu().numpy(), ref.counts.cpu().numpy())
    got, want = s.to_numpy("segments"), ref.to_numpy("segments")
    for f in FIELDS:
        np.testing.assert_array_equal(got[f], want[f])


def test_push_drops_emptied_slots_and_counts_only_live_particles():
    """A state with w = 0 slots (as merges leave them): the push produces nothing for them
    and n_pushed counts the w > 0 particles only."""
    rng = np.random.default_rng(8)
    N, L = 64, 2.54
    tab = xsec.analytic_argon(2000)
    xt = torch.as_tensor(tab.nsigma(3.22e22), device="cuda")
    p = K.make_params(n_faces=N, n_nodes=N + 1, bnf=4, advect=1, L=L, dx=L / N, dt=1e-12, nn=3.22e22,
                      gas_sigma=6.74e4, e_exc=tab.e_exc, xs_mode=_lib.XS_TABLE, xs_table=xt, xs_emin=tab.emin,
                      xs_emax=tab.emax, seed=3, step=1)
    s = K.SegmentSet(24, 256)
    n = 4000
    s.load(rng.uniform(0.1, L - 0.1, n), *(rng.normal(0, 3e5, n) for _ in range(3)), rng.uniform(1, 2, n))
    holes = torch.as_tensor(rng.random(s.capacity) < 0.3, device="cuda")
    s.w[holes] = 0.0
    live = int((s.to_numpy("segments")["w"] != 0).sum())
    ref = K.SegmentSet(24, 256)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    K.seg_repack(s, ref, st, K.Workspace())  # the same live particles, without the holes

    def push(src):
        out = K.SegmentSet(src.nseg, src.half)
        cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
        mom = torch.zeros(4, N + 1, dtype=torch.float64, device="cuda")
        sts = torch.zeros(1, dtype=torch.int32, device="cuda")
        fl = torch.zeros(1, dtype=torch.int32, device="cuda")
        K.seg_electron_kernel(p, src, out, torch.zeros(N, device="cuda"), sts, fl, K.Workspace(), moments=mom,
                              n_pushed=cnt)
        torch.cuda.synchronize()
        return out, int(cnt.item()), int(sts.item()), mom.cpu().numpy()

    o1, c1, s1, m1 = push(s)
    o2, c2, s2, m2 = push(ref)
    assert s1 == 0 and s2 == 0
    assert c1 == live and c2 == live
    # different slots give different Philox draws, so compare totals: every live particle
    # is pushed once, and the deposited weight of the survivors matches within the
    # statistics of absorption at the walls
    assert abs(o1.n() - o2.n()) <= 0.05 * live
    assert m1[0].sum() > 0 and abs(m1[0].sum() - m2[0].sum()) <= 0.05 * m2[0].sum()


def resample_case(seed, nseg, half, n, N=32, L=2.54, nb=3):
    rng = np.random.default_rng(seed)
    p = K.make_params(n_faces=N, n_nodes=N + 1, bnf=4, advect=1, L=L, dx=L / N, dt=1e-12, nn=3.22e22)
    s = K.SegmentSet(nseg, half)
    w = rng.choice([0.3, 1.0, 4.0], n)  # light (split) and heavy (merge) particles
    s.load(rng.uniform(0.05, L - 0.05, n), *(rng.normal(0, 1.5e6, n) for _ in range(3)), w)
    return p, s, nb


def resample(p, s, nb, in_place, targets=60):
    nkeys = p.n_nodes * nb
    ed = torch.as_tensor(np.array([4.0, 11.5]), device="cuda")
    perm = torch.zeros(s.capacity, dtype=torch.int32, device="cuda")
    offs = torch.zeros(nkeys + 1, dtype=torch.int32, device="cuda")
    cnts = torch.zeros(nkeys, dtype=torch.int32, device="cuda")
    hw = torch.zeros(nkeys, dtype=torch.int32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    fl = torch.zeros(1, dtype=torch.int32, device="cuda")
    ws = K.Workspace()
    K.seg_bin_particles(p, s, ed, 0.1, perm, offs, cnts, hw, st, ws)
    app = K.ParticleSet(s.capacity)
    out = K.SegmentSet(s.nseg, s.half)
    tg = torch.full((nb,), targets, dtype=torch.int32, device="cuda")
    mp = torch.full((nb,), 10 * targets, dtype=torch.int32, device="cuda")
    need = torch.zeros(1, dtype=torch.int32, device="cuda")
    K.seg_resample(p, s, app, out, nb, tg, mp, 0.1, 0.5, 3.0, 0.6, perm, offs, cnts, hw, st, fl, ws, need=need,
                   in_place=in_place)
    torch.cuda.synchronize()
    return (s if in_place else out), int(st.item()), int(need.item())


def live_rows(s):
    d = s.to_numpy("segments")
    keep = d["w"] != 0
    return np.stack([d[f][keep] for f in FIELDS], axis=1)


@pytest.mark.parametrize("targets", [20, 200])
def test_in_place_resampling_keeps_the_same_particles(targets):
    """targets 20: mostly merges (many emptied slots); 200: mostly splits (many appended).
    In place, the live particles are exactly those of the out-of-place resampling (as a
    set: the slots differ), and no segment holds more than half live particles."""
    p, a, nb = resample_case(3, 64, 512, 12000)
    p2, b, _ = resample_case(3, 64, 512, 12000)
    ra, sa, na = resample(p, a, nb, in_place=False, targets=targets)
    rb, sb, nb2 = resample(p2, b, nb, in_place=True, targets=targets)
    assert sa == 0 and sb == 0 and na == nb2 == 1
    x, y = live_rows(ra), live_rows(rb)
    assert len(x) == len(y) and len(x) != 12000
    x = x[np.lexsort(x.T[::-1])]
    y = y[np.lexsort(y.T[::-1])]
    np.testing.assert_array_equal(x, y)
    c = rb.counts.cpu().numpy().reshape(-1, 2)
    d = rb.to_numpy("segments")
    starts = np.concatenate([[0], np.cumsum(c.sum(axis=1))])
    per_seg = [(d["w"][starts[k]: starts[k + 1]] != 0).sum() for k in range(rb.nseg)]
    assert max(per_seg) <= rb.half


@pytest.mark.parametrize("variant", ["3bin", "5bin"])
def test_in_place_resampling_keeps_the_reference_order_on_one_segment(variant):
    """On one segment the in-place result, with its emptied slots dropped, is the
    reference's output in order: kept particles, then the appended ones."""
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", f"resample_{variant}.npz"))
    N, L = int(g["N"]), float(g["L"])
    x, v, w = g["x"], g["v"], g["w"]
    n = len(x)
    T = g["targets"]
    nb = len(T)
    p = K.make_params(n_faces=N, n_nodes=N + 1, bnf=4, advect=1, L=L, dx=L / N, dt=1e-12, nn=3.22e22,
                      flags=_lib.QUIRK_SPLIT_WRAP | _lib.QUIRK_TRIGGER_LAST)
    nkeys = (N + 1) * nb
    # room for the appended particles in run 1 of the one segment
    seg = K.SegmentSet(1, ((4 * max(n, int(g["out_n"])) + 3) // 4) * 4 * 2)
    seg.load(x, v[:, 0], v[:, 1], v[:, 2], w)
    ed = torch.as_tensor(np.asarray(g["edges"], dtype=np.float64), device="cuda")
    perm = torch.zeros(seg.capacity, dtype=torch.int32, device="cuda")
    offs = torch.zeros(nkeys + 1, dtype=torch.int32, device="cuda")
    cnts = torch.zeros(nkeys, dtype=torch.int32, device="cuda")
    hw = torch.zeros(nkeys, dtype=torch.int32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    fl = torch.zeros(1, dtype=torch.int32, device="cuda")
    ws = K.Workspace()
    K.seg_bin_particles(p, seg, ed, float(g["min_wt"]), perm, offs, cnts, hw, st, ws)
    app = K.ParticleSet(4 * n)
    scratch = K.SegmentSet(1, seg.half)
    tg = torch.as_tensor(np.asarray(T, dtype=np.int32), device="cuda")
    mp = torch.as_tensor((10 * T).astype(np.int32), device="cuda")
    ru = torch.as_tensor(g["draw_u"], device="cuda")
    need = torch.zeros(1, dtype=torch.int32, device="cuda")
    K.seg_resample(p, seg, app, scratch, nb, tg, mp, float(g["min_wt"]), 0.5, 3.0, 0.6, perm, offs, cnts, hw, st, fl,
                   ws, need=need, replay_u=ru, in_place=True)
    torch.cuda.synchronize()
    assert int(st.item()) == 0 and int(need.item()) == int(g["need"])
    o = seg.to_numpy("runs")
    keep = o["w"] != 0
    assert int(keep.sum()) == int(g["out_n"])
    od, ot = g["out_data"], g["out_tosum"]
    np.testing.assert_allclose(o["x"][keep], od[:, 0], rtol=2e-6)
    np.testing.assert_allclose(o["w"][keep], ot[:, 0], rtol=2e-6)
