"""Device-side failure paths, exercised without faulting, trapping or hanging the GPU.

Every wait on the device is bounded and reports BZ_DEV_LOOKBACK when it runs out; the
tests below make each kind of wait run out on purpose (a predecessor tile that nobody
publishes, an mbarrier that nothing arrives on) with a short limit, and check that the
kernel returned, raised the flag and left the context usable. The data checks raise their
flags from ordinary inputs: a NaN in the field (BZ_DEV_NONFINITE) and live particles
outside every cell (BZ_DEV_BINRANGE). The reference's only device-side check is the ion
fluid's break flag (heavies_kernel_1D.py:44-46), tested in test_field_gpu.py.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from boltzmann_gb300 import _lib, kernels as K, xsec  # noqa: E402
from oracle import oracle as O  # noqa: E402


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.fixture
def short_waits():
    lib = _lib.load()
    yield lib
    assert lib.bz_set_wait_limit(0) == _lib.BZ_OK  # back to the defaults
    assert lib.bz_wait_limit() == 0


def test_wait_limit_is_settable(short_waits):
    lib = short_waits
    assert lib.bz_wait_limit() == 0
    assert lib.bz_set_wait_limit(1234) == _lib.BZ_OK
    assert lib.bz_wait_limit() == 1234


@pytest.mark.parametrize("ntiles", [2, 40, 300])
def test_lookback_wait_runs_out_and_reports(short_waits, ntiles):
    """Tile 0 is never published: every look-back that reaches it gives up after the limit,
    counts it as empty, raises BZ_DEV_LOOKBACK and returns; the prefixes of the other tiles
    are still right (tile t sees the t-1 tiles 1..t-1)."""
    lib = short_waits
    assert lib.bz_set_wait_limit(2000) == _lib.BZ_OK
    ws = torch.zeros(lib.bz_lookback_selftest_workspace(ntiles), dtype=torch.uint8, device="cuda")
    prefix = torch.zeros(ntiles, dtype=torch.int32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = lib.bz_lookback_selftest(ntiles, 1, ctypes.c_void_p(prefix.data_ptr()), ctypes.c_void_p(ws.data_ptr()),
                                  ws.numel(), ctypes.c_void_p(st.data_ptr()), _stream())
    assert rc == _lib.BZ_OK
    torch.cuda.synchronize()
    assert int(st.item()) & _lib.DEV_LOOKBACK
    pf = prefix.cpu().numpy().view(np.uint32)
    assert pf[0] == 0xFFFFFFFF  # nobody took tile 0
    np.testing.assert_array_equal(pf[1:], np.arange(ntiles - 1))
    # the same with every tile published: no flag, prefix t
    st.zero_()
    rc = lib.bz_lookback_selftest(ntiles, 0, ctypes.c_void_p(prefix.data_ptr()), ctypes.c_void_p(ws.data_ptr()),
                                  ws.numel(), ctypes.c_void_p(st.data_ptr()), _stream())
    assert rc == _lib.BZ_OK
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    np.testing.assert_array_equal(prefix.cpu().numpy(), np.arange(ntiles))


def test_tensor_core_wait_runs_out_and_reports(short_waits):
    """An mbarrier that nothing arrives on (no MMA issued): the network kernels' bounded
    wait gives up, raises BZ_DEV_LOOKBACK in the network status, frees its TMEM and returns;
    with the arrival the same wait completes and raises nothing."""
    lib = short_waits
    st = ctypes.c_uint32(0)
    assert lib.bz_mlp_status(ctypes.byref(st)) == _lib.BZ_OK  # clear anything earlier
    assert lib.bz_set_wait_limit(64) == _lib.BZ_OK
    done = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert lib.bz_mlp_wait_selftest(0, ctypes.c_void_p(done.data_ptr()), _stream()) == _lib.BZ_OK
    torch.cuda.synchronize()
    assert int(done.item()) == 2
    assert lib.bz_mlp_status(ctypes.byref(st)) == _lib.BZ_OK
    assert st.value & _lib.DEV_LOOKBACK
    assert lib.bz_mlp_wait_selftest(1, ctypes.c_void_p(done.data_ptr()), _stream()) == _lib.BZ_OK
    torch.cuda.synchronize()
    assert int(done.item()) == 1
    assert lib.bz_mlp_status(ctypes.byref(st)) == _lib.BZ_OK
    assert st.value == 0
    # the context is still usable: a real network forward after the timeout
    from boltzmann_gb300 import surrogate as S
    net = S.SurrogateMLP(seed=3)
    x = torch.zeros(256, 16, device="cuda")
    y = torch.zeros(256, 80, device="cuda")
    K.mlp_forward(net.wb, net.prm, x, y)
    torch.cuda.synchronize()
    assert torch.isfinite(y).all()
    assert lib.bz_mlp_status(ctypes.byref(st)) == _lib.BZ_OK and st.value == 0


def _push_case(n=20_000, N=64, seed=5):
    rng = np.random.default_rng(seed)
    L = 2.54
    x = rng.uniform(1e-3, L - 1e-3, n)
    v = rng.normal(0.0, 8e5, (n, 3))
    w = rng.uniform(1.0, 2.0, n)
    tab = xsec.analytic_argon(2000)
    xs = torch.as_tensor(tab.nsigma(3.22e22), device="cuda")
    p = K.make_params(n_faces=N, n_nodes=N + 1, bnf=4, advect=1, L=L, dx=L / N, dt=1.0 / 13.56e6 / 400, nn=3.22e22,
                      gas_sigma=6.74e4, e_exc=tab.e_exc, xs_mode=_lib.XS_TABLE, xs_table=xs, xs_emin=tab.emin,
                      xs_emax=tab.emax, seed=seed, step=3)
    return (x, v, w), p, xs


def test_nonfinite_field_raises_flag():
    """A NaN in the field reaches the kicked velocity of the particles at that face: both
    pushes raise BZ_DEV_NONFINITE and write only the particles (no fault); with a finite
    field the flag stays clear."""
    (x, v, w), p, xs = _push_case()
    N = p.n_faces
    for bad in (False, True):
        E = torch.full((N,), 200.0, dtype=torch.float32, device="cuda")
        if bad:
            E[N // 2] = float("nan")
        # dense drop-in push
        src, dst = K.ParticleSet(len(x)), K.ParticleSet(3 * len(x))
        src.load(x, v[:, 0], v[:, 1], v[:, 2], w)
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        mom = torch.zeros(4, N + 1, dtype=torch.float64, device="cuda")
        K.electron_kernel(p, src, dst, E, st, K.Workspace(), moments=mom)
        torch.cuda.synchronize()
        assert bool(int(st.item()) & _lib.DEV_NONFINITE) == bad
        assert (int(st.item()) & ~_lib.DEV_NONFINITE) == 0
        # segmented push of the solver
        seg_in, seg_out = K.SegmentSet(16, 2048), K.SegmentSet(16, 2048)
        seg_in.load(x, v[:, 0], v[:, 1], v[:, 2], w)
        st2 = torch.zeros(1, dtype=torch.int32, device="cuda")
        fl = torch.zeros(1, dtype=torch.int32, device="cuda")
        K.seg_electron_kernel(p, seg_in, seg_out, E, st2, fl, K.Workspace(), moments=mom)
        torch.cuda.synchronize()
        assert bool(int(st2.item()) & _lib.DEV_NONFINITE) == bad
        assert (int(st2.item()) & ~_lib.DEV_NONFINITE) == 0
        o = dst.to_numpy()
        nan_rows = ~np.isfinite(o["vx"])
        assert nan_rows.any() == bad


@pytest.mark.parametrize("segmented", [False, True])
def test_particle_outside_every_cell_raises_binrange(segmented):
    """Live particles beyond the walls (x < -dx/2 or x >= L + dx/2) belong to no cell: the
    binning raises BZ_DEV_BINRANGE, leaves them out of every bin and bins the others as the
    oracle does."""
    rng = np.random.default_rng(9)
    n, N, L = 50_000, 128, 2.54
    x = rng.uniform(0, L, n)
    out_idx = rng.choice(n, 40, replace=False)
    x[out_idx[:20]] = L + 0.5  # beyond the last cell
    x[out_idx[20:]] = -0.3     # before the first
    e = rng.exponential(5.0, n)
    v = np.sqrt(2 * e / (9.10938e-31 * 6.241509e18))[:, None] * rng.normal(size=(n, 3)) / np.sqrt(3)
    x, v = x.astype(np.float32).astype(np.float64), v.astype(np.float32).astype(np.float64)
    w = np.ones(n)
    edges = (4.0, 11.5)
    nb = 3
    nkeys = (N + 1) * nb
    p = K.make_params(n_faces=N, n_nodes=N + 1, bnf=4, advect=1, L=L, dx=L / N, dt=1e-12, nn=3.22e22)
    ed = torch.as_tensor(np.asarray(edges), device="cuda")
    perm = torch.zeros(2 * n, dtype=torch.int32, device="cuda")
    offs = torch.zeros(nkeys + 1, dtype=torch.int32, device="cuda")
    cnts = torch.zeros(nkeys, dtype=torch.int32, device="cuda")
    hw = torch.zeros(nkeys, dtype=torch.int32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    ws = K.Workspace()
    if segmented:
        s = K.SegmentSet(32, 2048)
        s.load(x, v[:, 0], v[:, 1], v[:, 2], w)
        K.seg_bin_particles(p, s, ed, 0.1, perm, offs, cnts, hw, st, ws)
    else:
        s = K.ParticleSet(n)
        s.load(x, v[:, 0], v[:, 1], v[:, 2], w)
        K.bin_particles(p, s, ed, 0.1, perm, offs, cnts, hw, st, ws)
    torch.cuda.synchronize()
    assert int(st.item()) == _lib.DEV_BINRANGE
    keep = np.ones(n, bool)
    keep[out_idx] = False
    po = O.make_params(N)
    oc, _ = O.bin_particles(po, x[keep], v[keep, 0], v[keep, 1], v[keep, 2], w[keep], edges, 64)
    np.testing.assert_array_equal(cnts.cpu().numpy().reshape(N + 1, nb).T, oc)
    assert int(offs[-1].item()) == n - len(out_idx)
