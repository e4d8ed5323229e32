"""The allocation-free push (bz_push_collide_f32_noalloc) through the C ABI.

It exists for callers that cannot allocate device memory themselves (a plugin inside a
host solver that owns the GPU allocator, or code that must not call cudaMalloc): it
takes no workspace and keeps its scratch in a fixed array inside the library. Here two
calls in a row are checked against the workspace-taking bz_push_collide_f32 on the same
inputs (particles and counts exactly, moments to 1e-5 as the push tests use), and an
input above the fixed limit is refused before anything is launched. This file is
collected last so that a run that stops at the first failure has run everything else.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from boltzmann_gb300 import _lib, kernels as K, xsec  # noqa: E402


def _args(p, src, dst, E, mom, status):
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return (ctypes.byref(p), src.struct(), src.n_ptr(), src.capacity, dst.struct(), dst.capacity, dst.counts_ptr(),
            ctypes.c_void_p(E.data_ptr()), None, None, ctypes.c_void_p(mom.data_ptr())), \
        ctypes.c_void_p(status.data_ptr()), stream


def _case(n=150_000, N=512, seed=21):
    rng = np.random.default_rng(seed)
    L = 2.54
    x = rng.uniform(1e-3, L - 1e-3, n)
    v = rng.normal(0.0, 1.2e6, (n, 3))
    w = rng.uniform(1e4, 1e5, n)
    E = torch.as_tensor(rng.uniform(-800, 800, N), dtype=torch.float32, device="cuda")
    tab = xsec.analytic_argon(2000)
    nn = 3.22e22
    xs = torch.as_tensor(tab.nsigma(nn), device="cuda")
    p = K.make_params(n_faces=N, n_nodes=N + 1, bnf=4, advect=1, L=L, dx=L / N, dt=1.0 / 13.56e6 / 400, nn=nn,
                      gas_sigma=6.74e4, e_exc=tab.e_exc, xs_mode=_lib.XS_TABLE, xs_table=xs, xs_emin=tab.emin,
                      xs_emax=tab.emax, flags=_lib.QUIRK_DEAD_IONFLAG, seed=seed, step=1)
    return (x, v, w), E, p, xs


def _push(lib, fn, p, src, dst, E, ws=None):
    mom = torch.zeros(4, p.n_nodes, dtype=torch.float64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    a, sp, stream = _args(p, src, dst, E, mom, st)
    if ws is None:
        rc = getattr(lib, fn)(*a, sp, stream)
    else:
        rc = getattr(lib, fn)(*a, ctypes.c_void_p(ws.data_ptr()), ws.numel(), sp, stream)
    assert rc == _lib.BZ_OK, rc
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    return dst.cnt.cpu().numpy().copy(), dst.to_numpy(int(dst.cnt[2].item())), mom.cpu().numpy()


def test_noalloc_push_matches_workspace_push_twice_in_a_row():
    lib = _lib.load()
    (x, v, w), E, p, xs = _case()
    n = len(x)
    cap = 3 * n
    a_in, a_out = K.ParticleSet(cap), K.ParticleSet(cap)  # allocation-free entry point
    b_in, b_out = K.ParticleSet(cap), K.ParticleSet(cap)  # workspace entry point
    a_in.load(x, v[:, 0], v[:, 1], v[:, 2], w)
    b_in.load(x, v[:, 0], v[:, 1], v[:, 2], w)
    ws = torch.zeros(lib.bz_push_workspace(cap), dtype=torch.uint8, device="cuda")
    for step in (1, 2):  # two calls in a row; the second pushes the first call's output
        p.step = step
        ca, sa, ma = _push(lib, "bz_push_collide_f32_noalloc", p, a_in, a_out, E)
        cb, sb, mb = _push(lib, "bz_push_collide_f32", p, b_in, b_out, E, ws)
        np.testing.assert_array_equal(ca[:3], cb[:3])
        for f in K.ParticleSet.FIELDS:
            np.testing.assert_array_equal(sa[f], sb[f])
        for j in (0, 1, 3):
            np.testing.assert_allclose(ma[j], mb[j], rtol=1e-5, atol=1e-5 * np.abs(mb[j]).max())
        assert ca[1] > 0  # ionizations happened: the child path ran
        a_in, a_out = a_out, a_in
        b_in, b_out = b_out, b_in


def test_noalloc_push_refuses_inputs_above_its_limit():
    lib = _lib.load()
    (x, v, w), E, p, xs = _case(n=1000, N=64)
    src, dst = K.ParticleSet(1000), K.ParticleSet(3000)
    src.load(x, v[:, 0], v[:, 1], v[:, 2], w)
    mom = torch.zeros(4, p.n_nodes, dtype=torch.float64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    a, sp, stream = _args(p, src, dst, E, mom, st)
    a = list(a)
    a[3] = 64 * 1024 * 1024 + 1  # in_capacity above BZ_PUSH_NOALLOC_MAX_PARTICLES
    assert lib.bz_push_collide_f32_noalloc(*a, sp, stream) == _lib.BZ_ERR_TOO_LARGE
