"""Surrogate network kernels (csrc/bz_mlp.cu) against the float64 CPU oracle
(oracle/mlp.py), which rounds the matrix operands to bfloat16 where the GPU does; and the
learned start-up against the plain start of the same swarms.

Tolerances: outputs and gradients are compared as relative error norms. With identical
BF16 operands the remaining differences are FP32 vs FP64 accumulation (~1e-6) and the
rare BF16 rounding of an activation that lands on the other side of a rounding boundary
(one BF16 ulp, 2^-8 relative, of single elements), so 2e-3 (outputs) and 1e-2 (per-layer
gradients) leave a wide margin while any indexing or layout error gives O(1).
"""
import math

import numpy as np
import pytest
import torch

from boltzmann_gb300 import kernels as K
from boltzmann_gb300 import surrogate as S
from oracle import mlp as O

pytestmark = pytest.mark.gpu


def rand_case(n, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    p = S.init_params(seed, scale)
    p[O.OFFS[0][1]:O.OFFS[0][1] + 128] = rng.normal(0, 0.1, 128)  # non-zero biases
    for l in range(1, O.NL):
        wo, bo = O.OFFS[l]
        p[bo:bo + O.dims(l)[1]] = rng.normal(0, 0.1, O.dims(l)[1])
    x = np.zeros((n, 16))
    x[:, :9] = rng.uniform(-1, 1, (n, 9))
    t = np.zeros((n, 80))
    t[:, :66] = rng.normal(0, 1, (n, 66))
    return p, x, t


def dev(a, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300))


@pytest.mark.parametrize("n", [1, 37, 128, 300, 1000])
def test_forward_matches_oracle(n):
    p, x, _ = rand_case(n, n)
    net = S.SurrogateMLP(params=p)
    y = net.forward(dev(x)).cpu().numpy()
    # the oracle sees the same FP32 parameters
    y_o, _ = O.forward(net.params(), x.astype(np.float32))
    assert rel(y[:, :80], y_o) < 2e-3
    assert np.abs(y - y_o).max() < 2e-2 * np.abs(y_o).max()


def test_forward_gather_and_saved_preactivations():
    n_rows, n = 500, 200
    p, x, _ = rand_case(n_rows, 5)
    net = S.SurrogateMLP(params=p)
    rng = np.random.default_rng(1)
    idx = rng.integers(0, n_rows, n).astype(np.int32)
    y = torch.zeros(n, 80, device="cuda")
    z = torch.zeros(4, n, 128, device="cuda")
    K.mlp_forward(net.wb, net.prm, dev(x), y, idx=dev(idx, torch.int32), z=z)
    y_o, zs = O.forward(net.params(), x[idx].astype(np.float32))
    assert rel(y.cpu().numpy(), y_o) < 2e-3
    for l in range(4):
        assert rel(z[l].cpu().numpy(), zs[l]) < 2e-3


def test_bf16_copies_are_rounded_weights():
    p, _, _ = rand_case(4, 2)
    net = S.SurrogateMLP(params=p)
    prm = net.prm.cpu().numpy()
    wb = net.wb.cpu().numpy().view(np.uint16).astype(np.uint32) << 16
    wt = net.wt.cpu().numpy().view(np.uint16).astype(np.uint32) << 16
    wbf, wtf = wb.view(np.float32), wt.view(np.float32)
    for l in range(O.NL):
        ni, no = O.dims(l)
        wo, _ = O.OFFS[l]
        ref = O.bf16(prm[wo:wo + ni * no]).reshape(no, ni)
        assert np.array_equal(wbf[wo:wo + ni * no].reshape(no, ni), ref)
        assert np.array_equal(wtf[wo:wo + ni * no].reshape(ni, no), ref.T)


@pytest.mark.parametrize("path", ["mma.sync", "tcgen05"])
@pytest.mark.parametrize("n", [64, 200, 2048, 20000])
def test_backward_matches_oracle(n, path):
    """mma.sync backward (atomics) and tcgen05 backward (per-CTA partial gradients; 20000
    rows give 152 CTAs with several tiles each)."""
    p, x, t = rand_case(n, 10 + n)
    net = S.SurrogateMLP(params=p)
    w = S.output_weights()
    xd, td = dev(x), dev(t)
    y = torch.zeros(n, 80, device="cuda")
    z = torch.zeros(4, n, 128, device="cuda")
    K.mlp_forward(net.wb, net.prm, xd, y, z=z)
    grad = torch.zeros(S.NPARAM, device="cuda")
    loss = torch.zeros(1, device="cuda")
    ws = K.Workspace() if path == "tcgen05" else None
    K.mlp_backward(net.wb, net.wt, net.prm, xd, td, dev(w), y, z, grad, loss, ws=ws)
    g = grad.cpu().numpy()
    L_o, g_o = O.backward(net.params(), x.astype(np.float32), t.astype(np.float32), w)
    assert abs(float(loss.item()) - L_o) <= 1e-3 * L_o
    for l in range(O.NL):
        wo, bo = O.OFFS[l]
        ni, no = O.dims(l)
        assert rel(g[wo:bo], g_o[wo:bo]) < 1e-2, l
        assert rel(g[bo:bo + no], g_o[bo:bo + no]) < 1e-2, l


def test_backward_gradient_is_the_exact_gradient_to_bf16_precision():
    """The kernels' gradient against the float64 network's analytic gradient (itself
    checked against finite differences on the CPU): BF16 operands put them ~1% apart."""
    n = 256
    p, x, t = rand_case(n, 77)
    net = S.SurrogateMLP(params=p)
    w = S.output_weights()
    y = torch.zeros(n, 80, device="cuda")
    z = torch.zeros(4, n, 128, device="cuda")
    K.mlp_forward(net.wb, net.prm, dev(x), y, z=z)
    grad = torch.zeros(S.NPARAM, device="cuda")
    loss = torch.zeros(1, device="cuda")
    K.mlp_backward(net.wb, net.wt, net.prm, dev(x), dev(t), dev(w), y, z, grad, loss)
    _, g_x = O.backward(net.params(), x, t, w, exact=True)
    assert rel(grad.cpu().numpy(), g_x) < 5e-2


def test_adam_matches_oracle():
    p, _, _ = rand_case(4, 3)
    net = S.SurrogateMLP(params=p)
    rng = np.random.default_rng(4)
    m = np.zeros(S.NPARAM)
    v = np.zeros(S.NPARAM)
    pp = net.params()
    for step in (1, 2, 3):
        g = rng.normal(0, 1e-2, S.NPARAM).astype(np.float32).astype(np.float64)
        net.grad.copy_(dev(g))
        K.mlp_adam(net.prm, net.grad, net.m, net.v, net.wb, net.wt, step, 1e-3, weight_decay=0.01)
        pp, m, v = O.adam(pp, g, m, v, step, 1e-3, wd=0.01)
    np.testing.assert_allclose(net.params(), pp, rtol=1e-5, atol=1e-7)
    assert float(net.grad.abs().max()) == 0.0  # cleared for the next step
    wb = (net.wb.cpu().numpy().view(np.uint16).astype(np.uint32) << 16).view(np.float32)
    wo, bo = O.OFFS[2]
    assert np.array_equal(wb[wo:bo], O.bf16(net.prm.cpu().numpy()[wo:bo]))


def test_minibatch_indices_in_range_and_uniform():
    idx = torch.zeros(200_000, dtype=torch.int32, device="cuda")
    K.mlp_batch(1000, idx, seed=3, step=9)
    a = idx.cpu().numpy()
    assert a.min() >= 0 and a.max() < 1000
    h = np.bincount(a, minlength=1000)
    assert h.std() < 4 * math.sqrt(200.0)
    b = torch.zeros_like(idx)
    K.mlp_batch(1000, b, seed=3, step=9)
    assert torch.equal(idx, b)


def test_training_fits_a_smooth_map():
    """Adam on a synthetic regression: targets smooth functions of the features."""
    rng = np.random.default_rng(0)
    n = 20_000
    x = np.zeros((n, 16), dtype=np.float32)
    x[:, :9] = rng.uniform(-1, 1, (n, 9))
    t = np.zeros((n, 80), dtype=np.float32)
    for c in range(66):
        a = rng.normal(0, 1, 9)
        t[:, c] = np.tanh(x[:, :9] @ a / 2) + 0.3 * np.sin(2 * x[:, c % 9])
    net = S.SurrogateMLP(seed=1)
    xd, td = dev(x), dev(t)
    before = net.evaluate(xd, td)
    hist = net.train(xd, td, steps=1500, batch=1024, lr=2e-3, log_every=500)
    after = net.evaluate(xd, td)
    assert hist[-1] < hist[0]
    assert after < 0.05 * before


@pytest.fixture
def tcgen05_path():
    from boltzmann_gb300 import _lib
    lib = _lib.load()
    old = lib.bz_mlp_selected()
    yield lib
    lib.bz_mlp_select(old)


def mlp_status(lib):
    import ctypes
    v = ctypes.c_uint32(0)
    assert lib.bz_mlp_status(ctypes.byref(v)) == 0
    return v.value


@pytest.mark.parametrize("n", [1, 100, 128, 300, 2000])
def test_tcgen05_forward_matches_mma_sync_and_oracle(n, tcgen05_path):
    """The tcgen05 forward (TMEM accumulator, canonical shared-memory operands) computes
    the same network as the mma.sync one: identical BF16 operands, FP32 accumulation in
    another order (single activations may round to the neighbouring BF16 value)."""
    lib = tcgen05_path
    p, x, _ = rand_case(n, 50 + n)
    net = S.SurrogateMLP(params=p)
    xd = dev(x)
    lib.bz_mlp_select(0)
    y0 = torch.zeros(n, 80, device="cuda")
    z0 = torch.zeros(4, n, 128, device="cuda")
    K.mlp_forward(net.wb, net.prm, xd, y0, z=z0)
    lib.bz_mlp_select(1)
    y1 = torch.zeros(n, 80, device="cuda")
    z1 = torch.zeros(4, n, 128, device="cuda")
    K.mlp_forward(net.wb, net.prm, xd, y1, z=z1)
    y2 = net.forward(xd)  # inference path (no saved pre-activations)
    torch.cuda.synchronize()
    assert mlp_status(lib) == 0
    a, b = y0.cpu().numpy(), y1.cpu().numpy()
    assert rel(b, a) < 1e-3
    assert np.median(np.abs(b - a)) <= 1e-5 * np.abs(a).max()
    assert torch.equal(y1, y2)
    for l in range(4):
        assert rel(z1[l].cpu().numpy(), z0[l].cpu().numpy()) < 1e-3
    y_o, _ = O.forward(net.params(), x.astype(np.float32))
    assert rel(b, y_o) < 2e-3


def test_tcgen05_training_step_matches(tcgen05_path):
    """One training step with the tcgen05 forward gives the gradient of the oracle."""
    lib = tcgen05_path
    lib.bz_mlp_select(2)
    n = 512
    p, x, t = rand_case(n, 91)
    net = S.SurrogateMLP(params=p)
    w = S.output_weights()
    y = torch.zeros(n, 80, device="cuda")
    z = torch.zeros(4, n, 128, device="cuda")
    K.mlp_forward(net.wb, net.prm, dev(x), y, z=z)
    grad = torch.zeros(S.NPARAM, device="cuda")
    loss = torch.zeros(1, device="cuda")
    K.mlp_backward(net.wb, net.wt, net.prm, dev(x), dev(t), dev(w), y, z, grad, loss, ws=K.Workspace())
    torch.cuda.synchronize()
    assert mlp_status(lib) == 0
    L_o, g_o = O.backward(net.params(), x.astype(np.float32), t.astype(np.float32), w)
    assert abs(float(loss.item()) - L_o) <= 1e-3 * L_o
    assert rel(grad.cpu().numpy(), g_o) < 1e-2
    # deterministic: the partial gradients are summed in a fixed order
    g2 = torch.zeros_like(grad)
    K.mlp_backward(net.wb, net.wt, net.prm, dev(x), dev(t), dev(w), y, z, g2, torch.zeros(1, device="cuda"),
                   ws=K.Workspace())
    assert torch.equal(grad, g2)


def test_training_step_paths_agree(tcgen05_path):
    """bz_mlp_train_step with each kernel choice: the same minibatches, parameters within
    BF16 rounding of each other after a few Adam steps, and the loss going down."""
    lib = tcgen05_path
    rng = np.random.default_rng(3)
    n = 5000
    x = np.zeros((n, 16), dtype=np.float32)
    x[:, :9] = rng.uniform(-1, 1, (n, 9))
    t = np.zeros((n, 80), dtype=np.float32)
    t[:, :66] = np.tanh(x[:, :1] * 2)
    res = []
    for path in (0, 1, 2):
        lib.bz_mlp_select(path)
        net = S.SurrogateMLP(seed=4)
        hist = net.train(dev(x), dev(t), steps=40, batch=1024, lr=1e-3, log_every=20)
        torch.cuda.synchronize()
        assert mlp_status(lib) == 0
        assert hist[-1] < hist[0]
        res.append(net.params())
    for p in res[1:]:
        assert rel(p - S.init_params(4), res[0] - S.init_params(4)) < 0.05
