"""The allocation-free push (bz_push_collide_f32_noalloc) through the C ABI.

It exists for callers that cannot allocate device memory themselves (a plugin inside a
host solver that owns the GPU allocator, or code that must not call cudaMalloc): it
takes no workspace and keeps its scratch in a fixed array inside the library. Here two
calls in a row are checked against the workspace-taking bz_push_collide_f32 on the same
inputs (particles and counts exactly, moments to 1e-5 as the push tests use), an input
above the fixed limit is refused before anything is launched, and a caller in a second
CUDA context of its own gets that context's copy of the array. This file is collected
last so that a run that stops at the first failure has run everything else.
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


def _driver():
    """The CUDA driver API through ctypes, for a second context on the same GPU."""
    try:
        cu = ctypes.CDLL("libcuda.so.1")
    except OSError:
        pytest.skip("libcuda.so.1 not loadable")
    for name in ("cuInit", "cuDeviceGet", "cuCtxSynchronize", "cuMemAlloc_v2", "cuMemFree_v2", "cuMemcpyHtoD_v2",
                 "cuMemcpyDtoH_v2", "cuCtxPopCurrent_v2", "cuCtxDestroy_v2"):
        getattr(cu, name).restype = ctypes.c_int
    cu.cuMemAlloc_v2.argtypes = [ctypes.POINTER(ctypes.c_uint64), ctypes.c_size_t]
    cu.cuMemFree_v2.argtypes = [ctypes.c_uint64]
    cu.cuMemcpyHtoD_v2.argtypes = [ctypes.c_uint64, ctypes.c_void_p, ctypes.c_size_t]
    cu.cuMemcpyDtoH_v2.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_size_t]
    cu.cuCtxPopCurrent_v2.argtypes = [ctypes.POINTER(ctypes.c_void_p)]
    cu.cuCtxDestroy_v2.argtypes = [ctypes.c_void_p]
    return cu


def _create_context(cu, dev):
    ctx = ctypes.c_void_p()
    if hasattr(cu, "cuCtxCreate_v4"):
        cu.cuCtxCreate_v4.restype = ctypes.c_int
        cu.cuCtxCreate_v4.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_uint, ctypes.c_int]
        rc = cu.cuCtxCreate_v4(ctypes.byref(ctx), None, 0, dev)
    else:
        cu.cuCtxCreate_v2.restype = ctypes.c_int
        cu.cuCtxCreate_v2.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_uint, ctypes.c_int]
        rc = cu.cuCtxCreate_v2(ctypes.byref(ctx), 0, dev)
    assert rc == 0 and ctx.value, rc
    return ctx


def test_noalloc_push_follows_the_current_context():
    """A host that makes its own CUDA context (a solver that embeds this library and drives
    the GPU through the driver API) gets the scratch array of the context it calls from:
    the same push in a second context, on buffers of that context, gives the same particles
    as in the primary context, and the primary context's calls keep working afterwards."""
    lib = _lib.load()
    (x, v, w), E, p, xs = _case(n=60_000, N=512, seed=23)
    n = len(x)
    cap = 3 * n
    a_in, a_out = K.ParticleSet(cap), K.ParticleSet(cap)
    a_in.load(x, v[:, 0], v[:, 1], v[:, 2], w)
    ca, sa, ma = _push(lib, "bz_push_collide_f32_noalloc", p, a_in, a_out, E)
    addr_primary = ctypes.c_void_p()
    assert lib.bz_push_noalloc_scratch_address(ctypes.byref(addr_primary)) == _lib.BZ_OK and addr_primary.value
    # host copies of every input, for the second context
    f32 = lambda t: np.ascontiguousarray(t.detach().cpu().numpy())
    host_in = {f: f32(getattr(a_in, f)) for f in K.ParticleSet.FIELDS}
    host_E = f32(E)
    host_xs = f32(xs)
    torch.cuda.synchronize()
    cu = _driver()
    assert cu.cuInit(0) == 0
    dev = ctypes.c_int()
    assert cu.cuDeviceGet(ctypes.byref(dev), torch.cuda.current_device()) == 0
    ctx = _create_context(cu, dev.value)  # now current on this thread
    bufs = []

    def alloc(nbytes, host=None):
        d = ctypes.c_uint64()
        assert cu.cuMemAlloc_v2(ctypes.byref(d), max(int(nbytes), 16)) == 0
        bufs.append(d.value)
        if host is not None:
            assert cu.cuMemcpyHtoD_v2(d.value, host.ctypes.data, host.nbytes) == 0
        return d.value

    try:
        addr_ctx = ctypes.c_void_p()
        assert lib.bz_push_noalloc_scratch_address(ctypes.byref(addr_ctx)) == _lib.BZ_OK
        # the second context has its own copy of the array: had the first context's address
        # been reused here, nothing would be launched (the assertion stops the test first)
        assert addr_ctx.value and addr_ctx.value != addr_primary.value
        pin = _lib.Particles(*(alloc(host_in[f].nbytes, host_in[f]) for f in K.ParticleSet.FIELDS))
        pout = _lib.Particles(*(alloc(4 * cap) for _ in K.ParticleSet.FIELDS))
        n_in = alloc(4, np.array([n], dtype=np.int32))
        counts = alloc(16, np.zeros(4, dtype=np.int32))
        d_E = alloc(host_E.nbytes, host_E)
        d_xs = alloc(host_xs.nbytes, host_xs)
        mom = alloc(8 * 4 * p.n_nodes, np.zeros(4 * p.n_nodes))
        st = alloc(4, np.zeros(1, dtype=np.uint32))
        p2 = _lib.BzParams.from_buffer_copy(p)
        p2.xs_table = d_xs
        rc = lib.bz_push_collide_f32_noalloc(ctypes.byref(p2), pin, ctypes.c_void_p(n_in), cap, pout, cap,
                                             ctypes.c_void_p(counts), ctypes.c_void_p(d_E), None, None,
                                             ctypes.c_void_p(mom), ctypes.c_void_p(st), None)
        assert rc == _lib.BZ_OK, rc
        assert cu.cuCtxSynchronize() == 0
        hc = np.zeros(4, dtype=np.int32)
        assert cu.cuMemcpyDtoH_v2(hc.ctypes.data, counts, 16) == 0
        hs = np.zeros(1, dtype=np.uint32)
        assert cu.cuMemcpyDtoH_v2(hs.ctypes.data, st, 4) == 0
        assert hs[0] == 0
        np.testing.assert_array_equal(hc[:3], ca[:3])
        nn = int(hc[2])
        for f, dptr in zip(K.ParticleSet.FIELDS, (pout.x, pout.vx, pout.vy, pout.vz, pout.w)):
            h = np.zeros(nn, dtype=np.float32)
            assert cu.cuMemcpyDtoH_v2(h.ctypes.data, dptr, 4 * nn) == 0
            np.testing.assert_array_equal(h.astype(np.float64), sa[f])
        hm = np.zeros(4 * p.n_nodes)
        assert cu.cuMemcpyDtoH_v2(hm.ctypes.data, mom, hm.nbytes) == 0
        hm = hm.reshape(4, p.n_nodes)
        for j in (0, 1, 3):
            np.testing.assert_allclose(hm[j], ma[j], rtol=1e-5, atol=1e-5 * np.abs(ma[j]).max())
    finally:
        for b in bufs:
            cu.cuMemFree_v2(b)
        old = ctypes.c_void_p()
        cu.cuCtxPopCurrent_v2(ctypes.byref(old))
        cu.cuCtxDestroy_v2(ctx)
    # back in the primary context: its own address again, and the same result
    again = ctypes.c_void_p()
    assert lib.bz_push_noalloc_scratch_address(ctypes.byref(again)) == _lib.BZ_OK
    assert again.value == addr_primary.value
    b_out = K.ParticleSet(cap)
    cb, sb, mb = _push(lib, "bz_push_collide_f32_noalloc", p, a_in, b_out, E)
    np.testing.assert_array_equal(cb[:3], ca[:3])
    for f in K.ParticleSet.FIELDS:
        np.testing.assert_array_equal(sb[f], sa[f])
