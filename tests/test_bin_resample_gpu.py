"""GPU parity of binning (cell x energy-bin stable sort) and ES-WPNC resampling.

Bin counts and bin membership are bit-exact against the reference (golden vectors
from its own source) and against the oracle at larger sizes; each bin's list is in
ascending particle index, the order the reference's serial semantics give. The
resampled state is compared with the reference's after replaying its random numbers.
"""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from boltzmann_gb300 import _lib, kernels as K  # noqa: E402
from oracle import oracle as O  # noqa: E402

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DT = {"f32": torch.float32, "f64": torch.float64}
MQ = _lib.QUIRK_SPLIT_WRAP | _lib.QUIRK_TRIGGER_LAST


def grid_params(N, L=2.54, flags=0):
    return K.make_params(n_faces=N, n_nodes=N + 1, bnf=4, advect=1, L=L, dx=L / N, dt=1e-12, nn=3.22e22,
                         flags=flags)


def gpu_bin(x, v, w, N, edges, dtype, L=2.54, min_wt=0.1):
    n = len(x)
    s = K.ParticleSet(max(n, 1), dtype)
    s.load(x, v[:, 0], v[:, 1], v[:, 2], w)
    p = grid_params(N, L)
    nb = len(edges) + 1
    nkeys = (N + 1) * nb
    ed = torch.as_tensor(np.asarray(edges, dtype=np.float64).reshape(-1) if len(edges) else np.zeros(1),
                         device="cuda")
    perm = torch.zeros(max(n, 1), dtype=torch.int32, device="cuda")
    offsets = torch.zeros(nkeys + 1, dtype=torch.int32, device="cuda")
    counts = torch.zeros(nkeys, dtype=torch.int32, device="cuda")
    hw = torch.zeros(nkeys, dtype=torch.int32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    K.bin_particles(p, s, ed[: nb - 1] if nb > 1 else ed[:0], min_wt, perm, offsets, counts, hw, st, K.Workspace())
    torch.cuda.synchronize()
    return (perm.cpu().numpy(), offsets.cpu().numpy(), counts.cpu().numpy().reshape(N + 1, nb),
            hw.cpu().numpy().reshape(N + 1, nb), int(st.item()))


@pytest.mark.parametrize("variant", ["1bin", "3bin", "5bin"])
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_bins_match_reference_golden(variant, prec):
    g = np.load(os.path.join(G, f"bins_{variant}.npz"))
    N = int(g["N"])
    perm, offsets, counts, hw, st = gpu_bin(g["x"], g["v"], g["w"], N, g["edges"], DT[prec], float(g["L"]))
    gc = g["counts"]  # [nb, N+1]
    np.testing.assert_array_equal(counts.T, gc)
    max_ppc = int(g["max_ppc"])
    nb = gc.shape[0]
    for c in range(N + 1):
        for b in range(nb):
            k = c * nb + b
            lst = perm[offsets[k]: offsets[k] + counts[c, b]]
            assert np.all(np.diff(lst) > 0)
            m = min(int(counts[c, b]), max_ppc)
            np.testing.assert_array_equal(lst[:m], g["tables"][b, :m, c])


@pytest.mark.parametrize("edges", [(), (10.0, 15.76), (2.0, 6.0, 11.5, 15.76)])
def test_bins_match_oracle_large(edges):
    rng = np.random.default_rng(len(edges))
    n, N = 300_000, 1024
    x = rng.uniform(0, 2.54, n).astype(np.float32).astype(np.float64)
    e = rng.exponential(6.0, n)
    v = (np.sqrt(2 * e / (9.10938e-31 * 6.241509e18))[:, None] * rng.normal(size=(n, 3)) / np.sqrt(3))
    v = v.astype(np.float32).astype(np.float64)
    w = rng.uniform(0.01, 2.0, n).astype(np.float32).astype(np.float64)
    w[rng.uniform(size=n) < 0.02] = 0.0
    perm, offsets, counts, hw, st = gpu_bin(x, v, w, N, edges, torch.float32)
    assert st == 0
    p = O.make_params(N)
    oc, ol = O.bin_particles(p, x, v[:, 0], v[:, 1], v[:, 2], w, edges, 64)
    np.testing.assert_array_equal(counts.T, oc)
    assert offsets[-1] == int((w > 0).sum())
    # every key's slice is the ascending list of its members
    nb = len(edges) + 1
    key = np.full(n, -1)
    for b in range(nb):
        for c in range(N + 1):
            k = c * nb + b
            sl = perm[offsets[k]: offsets[k] + counts[c, b]]
            key[sl] = k
            m = min(int(counts[c, b]), 64)
            np.testing.assert_array_equal(sl[:m], ol[b, :m, c])
    assert np.all((key >= 0) == (w > 0))
    np.testing.assert_array_equal(hw.T, [[int(((w > 0.1) & (key == c * nb + b)).sum()) for c in range(N + 1)]
                                         for b in range(nb)])


def run_resample_gpu(x, v, w, N, edges, targets, max_ppc, min_wt, dtype, flags, replay_u=None, L=2.54,
                     split_below=0.5, merge_at=3.0, merge_keep=0.6, cap_factor=4, diag=False):
    n = len(x)
    nb = len(edges) + 1
    nkeys = (N + 1) * nb
    s = K.ParticleSet(cap_factor * n, dtype)
    out = K.ParticleSet(cap_factor * n, dtype)
    s.load(x, v[:, 0], v[:, 1], v[:, 2], w)
    p = grid_params(N, L, flags)
    ed = torch.as_tensor(np.asarray(edges, dtype=np.float64).reshape(-1) if len(edges) else np.zeros(1),
                         device="cuda")
    perm = torch.zeros(s.capacity, dtype=torch.int32, device="cuda")
    offsets = torch.zeros(nkeys + 1, dtype=torch.int32, device="cuda")
    counts = torch.zeros(nkeys, dtype=torch.int32, device="cuda")
    hw = torch.zeros(nkeys, dtype=torch.int32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    need = torch.zeros(1, dtype=torch.int32, device="cuda")
    ws = K.Workspace()
    K.bin_particles(p, s, ed[: nb - 1] if nb > 1 else ed[:0], min_wt, perm, offsets, counts, hw, st, ws)
    tg = torch.as_tensor(np.asarray(targets, dtype=np.int32), device="cuda")
    mp = torch.as_tensor(np.asarray(max_ppc, dtype=np.int32), device="cuda")
    ru = None if replay_u is None else torch.as_tensor(np.asarray(replay_u, dtype=np.float64), device="cuda")
    cd = torch.zeros(nkeys, _lib.CONS_DIAG_STRIDE, dtype=torch.float64, device="cuda") if diag else None
    K.resample(p, s, out, nb, tg, mp, min_wt, split_below, merge_at, merge_keep, perm, offsets, counts, hw, st, ws,
               need=need, replay_u=ru, cons_diag=cd)
    torch.cuda.synchronize()
    return out.to_numpy(), int(need.item()), int(st.item()), (None if cd is None else cd.cpu().numpy()), \
        counts.cpu().numpy()


@pytest.mark.parametrize("variant", ["1bin", "3bin", "5bin"])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_resample_matches_reference_golden(variant, prec):
    g = np.load(os.path.join(G, f"resample_{variant}.npz"))
    N = int(g["N"])
    T = g["targets"]
    max_ppc = (10 * T).astype(np.int64)
    out, need, st, _, _ = run_resample_gpu(g["x"], g["v"], g["w"], N, g["edges"], T, max_ppc, float(g["min_wt"]),
                                           DT[prec], MQ, replay_u=g["draw_u"], L=float(g["L"]))
    assert st == 0
    assert need == int(g["need"])
    na = int(g["out_n"])
    assert len(out["x"]) == na
    od, ot = g["out_data"], g["out_tosum"]
    rtol = 1e-12 if prec == "f64" else 2e-6
    speed = np.sqrt((od[:, 3:6] ** 2).sum(axis=1))
    np.testing.assert_allclose(out["x"], od[:, 0], rtol=rtol)
    np.testing.assert_allclose(out["w"], ot[:, 0], rtol=rtol)
    for k, f in enumerate(("vx", "vy", "vz")):
        assert np.all(np.abs(out[f] - od[:, 3 + k]) <= rtol * speed * 4)


def test_resample_conserves_weight_momentum_energy():
    """Merge with the energy-conserving rescale, float64 state: weight, momentum and
    energy of every merged (cell, bin) are conserved to 1e-12 relative."""
    rng = np.random.default_rng(3)
    N, n = 32, 200_000
    x = rng.uniform(0, 2.54, n)
    v = rng.normal(0, 1e6, (n, 3)) + np.array([3e5, -1e5, 0])
    w = rng.uniform(0.5, 2.0, n)
    edges = (5.0, 20.0)
    T = [1000, 500, 200]
    out, need, st, cd, counts = run_resample_gpu(x, v, w, N, edges, T, [10 * t for t in T], 0.1, torch.float64,
                                                 _lib.FIX_MERGE_ENERGY, diag=True)
    assert st == 0 and need == 1
    merged = cd[:, 0] > 0
    assert merged.sum() > 10
    b, a = cd[merged, :5], cd[merged, 5:]
    np.testing.assert_allclose(a[:, 0], b[:, 0], rtol=1e-12)
    pm = np.abs(b[:, 1:4]).max() + np.sqrt(b[:, 0] * b[:, 4]).max()
    np.testing.assert_allclose(a[:, 1:4], b[:, 1:4], rtol=1e-12, atol=1e-12 * pm * 1e3)
    np.testing.assert_allclose(a[:, 4], b[:, 4], rtol=1e-12)


EFAC = 0.5 * 9.10938e-31 * 6.241509e18  # |v|^2 (m/s)^2 -> eV
U24 = 2.0 ** -24  # unit roundoff of float32


def check_merge_conservation(cd, f32):
    """Per merged key: the survivors as formed in float64 conserve weight, momentum and
    energy of the originals to 1e-12; as stored they keep weight to 2^-24 relative,
    momentum to 2.1 * 2^-24 of sum(w|v|) and energy to 3.1 * 2^-24 relative (float32
    storage: the weight W/K and every velocity component rounded once each, relative error
    u = 2^-24; a momentum term w v picks up at most (1+u)^2 - 1, an energy term w v^2 at
    most (1+u)^3 - 1); with float64 storage the stored sums are the formed ones."""
    merged = cd[:, 0] > 0
    b, a, f = cd[merged, 0:5], cd[merged, 5:10], cd[merged, 10:15]
    W, E = b[:, 0], b[:, 4]
    S = np.sqrt(W * E / EFAC)  # bounds sum(w |v_x|) by Cauchy-Schwarz
    # formed in float64
    np.testing.assert_allclose(f[:, 0], W, rtol=1e-12, atol=0)
    for j in (1, 2, 3):
        assert np.all(np.abs(f[:, j] - b[:, j]) <= 1e-12 * S), j
    np.testing.assert_allclose(f[:, 4], E, rtol=1e-12, atol=0)
    # stored
    if f32:
        assert np.all(np.abs(a[:, 0] - W) <= 1.01 * U24 * W)
        for j in (1, 2, 3):
            assert np.all(np.abs(a[:, j] - b[:, j]) <= 2.1 * U24 * S + 1e-12 * S), j
        assert np.all(np.abs(a[:, 4] - E) <= 3.1 * U24 * E + 1e-12 * E)
    else:
        np.testing.assert_allclose(a[:, 0], W, rtol=1e-12, atol=0)
        for j in (1, 2, 3):
            assert np.all(np.abs(a[:, j] - b[:, j]) <= 1e-12 * S), j
        np.testing.assert_allclose(a[:, 4], E, rtol=1e-12, atol=0)
    return int(merged.sum())


def test_merge_conserves_on_the_benchmark_path():
    """The headline configuration's resampling path: float32 segmented state of a 1024-cell
    1 Torr CCP with a drift, 5 bins (edges 2, 6, 11.5, 15.76 eV), the reference's split
    indexing and trigger with the energy-conserving merge (the benchmark's setting), split
    and merge both firing. cons_diag is read for every merged (cell, bin)."""
    rng = np.random.default_rng(17)
    N, n, L = 1024, 4_000_000, 2.54
    x = rng.uniform(0, L, n)
    e = rng.gamma(1.5, 1.2, n)  # ~1.8 eV mean: the sparse 11.5-15.76 eV bin splits
    hot = rng.uniform(size=n) < 0.05
    e[hot] = rng.uniform(20.0, 40.0, int(hot.sum()))  # the open top bin overflows: the trigger fires
    v = np.sqrt(2 * e / (9.10938e-31 * 6.241509e18))[:, None] * rng.normal(size=(n, 3)) / np.sqrt(3)
    v += np.array([2.0e5, -5.0e4, 0.0])  # a drift, where the reference's rescale loses energy
    w = rng.uniform(0.5, 2.0, n)
    f32 = lambda a: np.asarray(a, dtype=np.float32).astype(np.float64)
    x, v, w = f32(x), f32(v), f32(w)
    nb, nkeys = 5, (N + 1) * 5
    edges = (2.0, 6.0, 11.5, 15.76)
    T = [600, 400, 200, 70, 30]  # merges in the lower bins, splits in the sparse upper ones
    seg = K.SegmentSet(-(-2 * n // 2048), 2048)
    seg.load(x, v[:, 0], v[:, 1], v[:, 2], w)
    p = grid_params(N, L, _lib.QUIRK_SPLIT_WRAP | _lib.QUIRK_TRIGGER_LAST | _lib.FIX_MERGE_ENERGY)
    ed = torch.as_tensor(np.asarray(edges), device="cuda")
    perm = torch.zeros(seg.capacity, dtype=torch.int32, device="cuda")
    offs = torch.zeros(nkeys + 1, dtype=torch.int32, device="cuda")
    cnts = torch.zeros(nkeys, dtype=torch.int32, device="cuda")
    hw = torch.zeros(nkeys, dtype=torch.int32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    fl = torch.zeros(1, dtype=torch.int32, device="cuda")
    need = torch.zeros(1, dtype=torch.int32, device="cuda")
    ws = K.Workspace()
    K.seg_bin_particles(p, seg, ed, 0.1, perm, offs, cnts, hw, st, ws)
    app = K.ParticleSet(2 * n)
    out = K.SegmentSet(seg.nseg, seg.half)
    tg = torch.as_tensor(np.asarray(T, dtype=np.int32), device="cuda")
    mp = torch.as_tensor(np.asarray([10 * t for t in T], dtype=np.int32), device="cuda")
    cd = torch.zeros(nkeys, _lib.CONS_DIAG_STRIDE, dtype=torch.float64, device="cuda")
    K.seg_resample(p, seg, app, out, nb, tg, mp, 0.1, 0.5, 3.0, 0.6, perm, offs, cnts, hw, st, fl, ws, need=need,
                   cons_diag=cd)
    torch.cuda.synchronize()
    assert int(st.item()) == 0 and int(need.item()) == 1
    c = cnts.cpu().numpy().reshape(N + 1, nb)
    split = (c > 0) & (c < 0.5 * np.asarray(T))
    assert split.sum() > 10  # both kinds fire
    assert check_merge_conservation(cd.cpu().numpy(), f32=True) > 1000


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_merge_to_one_survivor_stays_finite(prec):
    """Keys merged to a single survivor (K = int(0.6 * 2) = 1) have no kept thermal part:
    the energy-conserving rescale keeps the factor 1 there, so the survivor carries the
    originals' mean velocity (weight and momentum conserved) and nothing turns non-finite."""
    rng = np.random.default_rng(4)
    N, per = 8, 40
    n = (N + 1) * per
    dx = 2.54 / N
    x = np.repeat(np.arange(N + 1) * dx, per) + rng.uniform(-0.3, 0.3, n) * dx
    x = np.clip(x, 0.0, 2.54 - 1e-6)
    v = rng.normal(0, 5e5, (n, 3)) + np.array([1e5, 0, 0])
    w = rng.uniform(0.5, 2.0, n)
    out, need, st, cd, counts = run_resample_gpu(x, v, w, N, (), [2], [20], 0.1, DT[prec], _lib.FIX_MERGE_ENERGY,
                                                 diag=True)
    assert st == 0 and need == 1
    assert all(np.all(np.isfinite(out[f])) for f in K.ParticleSet.FIELDS)
    merged = cd[:, 0] > 0
    assert merged.sum() == N + 1
    b, a = cd[merged, 0:5], cd[merged, 5:10]
    rt = 1e-12 if prec == "f64" else 3e-7
    np.testing.assert_allclose(a[:, 0], b[:, 0], rtol=rt)
    S = np.sqrt(b[:, 0] * b[:, 4] / EFAC)
    for j in (1, 2, 3):
        assert np.all(np.abs(a[:, j] - b[:, j]) <= rt * S)


def test_resample_counts_match_oracle_philox():
    """Post-resample particle count is exact (it depends only on the bin counts)."""
    rng = np.random.default_rng(11)
    N, n = 64, 100_000
    x = rng.uniform(0, 2.54, n) ** 1.5 / 2.54 ** 0.5
    v = rng.normal(0, 1.2e6, (n, 3))
    w = rng.uniform(0.05, 2.0, n)
    edges = (4.0, 11.5)
    T = [700, 200, 100]
    out, need, st, _, counts = run_resample_gpu(x, v, w, N, edges, T, [10 * t for t in T], 0.1, torch.float32,
                                                _lib.QUIRK_SPLIT_WRAP)
    assert st == 0 and need == 1
    c = counts.reshape(N + 1, 3)
    expect = n
    for cc in range(N + 1):
        for b in range(3):
            m, t = int(c[cc, b]), T[b]
            hw_any = True  # every bin here holds particles with w > 0.1 with overwhelming odds
            if 0 < m < 0.5 * t and hw_any:
                expect += 2 * t - m
            elif m >= 3 * t:
                expect += int(0.6 * t) - min(m, 10 * t)
    assert len(out["x"]) == expect


@pytest.mark.parametrize("case", ["merge", "split", "none", "trigger_last", "per_key"])
def test_binning_with_the_trigger_sorts_only_when_resampling_runs(case):
    """bz_seg_bin_check_*: the trigger it evaluates from the counts equals the one
    bz_seg_resample_* evaluates; counts are complete either way; when the trigger is on the
    permutation and offsets equal the plain binning's, when it is off nothing is sorted."""
    rng = np.random.default_rng(31)
    N, L, n, nb = 48, 2.54, 60_000, 3
    x = rng.uniform(0.01, L - 0.01, n)
    v = rng.normal(0, 1.3e6, (n, 3))
    w = rng.uniform(0.5, 2.0, n)
    flags = _lib.QUIRK_TRIGGER_LAST if case == "trigger_last" else 0
    nkeys = (N + 1) * nb
    per_key = case == "per_key"
    if per_key:
        flags |= _lib.PER_KEY_TARGETS
    # about n / nkeys = 400 per key on average (fewer in the hot bin)
    T = {"merge": 60, "split": 4000, "none": 300, "trigger_last": 60, "per_key": None}[case]
    if per_key:
        targ = np.full(nkeys, 300, dtype=np.int32)
        targ[7 * nb + 1] = 20  # one key far above its target: merge
    else:
        targ = np.full(nb, T, dtype=np.int32)
    split_below, merge_at = (0.5, 3.0) if case != "none" else (1e-9, 1e9)
    p = grid_params(N, L, flags)
    seg = K.SegmentSet(80, 1024)
    seg.load(x, v[:, 0], v[:, 1], v[:, 2], w)
    ed = torch.as_tensor(np.array([4.0, 11.5]), device="cuda")
    tg = torch.as_tensor(targ, device="cuda")

    def bins(check):
        perm = torch.full((seg.capacity,), -7, dtype=torch.int32, device="cuda")
        offs = torch.full((nkeys + 1,), -7, dtype=torch.int32, device="cuda")
        cnts = torch.zeros(nkeys, dtype=torch.int32, device="cuda")
        hw = torch.zeros(nkeys, dtype=torch.int32, device="cuda")
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        need = torch.full((1,), -1, dtype=torch.int32, device="cuda")
        K.seg_bin_particles(p, seg, ed, 0.1, perm, offs, cnts, hw, st, K.Workspace(),
                            check=(tg, split_below, merge_at, need) if check else None)
        torch.cuda.synchronize()
        assert int(st.item()) == 0
        return perm, offs, cnts, hw, int(need.item())

    perm0, offs0, cnt0, hw0, _ = bins(False)
    perm1, offs1, cnt1, hw1, need = bins(True)
    assert torch.equal(cnt0, cnt1) and torch.equal(hw0, hw1)
    # the trigger of the resampling itself on the same counts
    app = K.ParticleSet(2_000_000)  # room for every split's copies (up to 147 keys x 2T)
    out = K.SegmentSet(2048, 1024)
    mp = torch.as_tensor(10 * targ, dtype=torch.int32, device="cuda")
    need_rs = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    fl = torch.zeros(1, dtype=torch.int32, device="cuda")
    K.seg_resample(p, seg, app, out, nb, tg, mp, 0.1, split_below, merge_at, 0.6, perm0, offs0, cnt0, hw0, st, fl,
                   K.Workspace(), need=need_rs)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    assert need == int(need_rs.item())
    assert need == (0 if case == "none" else 1)
    if need:
        assert torch.equal(offs0, offs1)
        live = int(cnt0.sum().item())
        assert torch.equal(perm0[:live], perm1[:live])
    else:
        assert int((perm1 != -7).sum().item()) == 0  # nothing sorted
