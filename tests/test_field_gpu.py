"""GPU parity of the device-resident grid step: Poisson solve (EF_kernel_1D.py) and
ion drift-diffusion (heavies_kernel_1D.py) against the reference's own outputs."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from boltzmann_gb300 import _lib, kernels as K  # noqa: E402

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_poisson_and_fluid_match_reference():
    g = np.load(os.path.join(G, "field.npz"))
    N = int(g["N"])
    dx = float(g["dx"])
    dev = "cuda"
    d = torch.zeros(N - 1, dtype=torch.float64, device=dev)
    l = torch.zeros(N - 1, dtype=torch.float64, device=dev)
    plan = torch.zeros(4 * (N - 1), dtype=torch.float64, device=dev)
    K.poisson_factor(N, dx, d, l, plan)
    ne = torch.as_tensor(g["ne"], device=dev)
    ni = torch.as_tensor(g["ni"], device=dev)
    V = torch.zeros(N - 1, dtype=torch.float64, device=dev)
    E = torch.zeros(N, dtype=torch.float64, device=dev)
    E32 = torch.zeros(N, dtype=torch.float32, device=dev)
    K.EF_kernel(N, dx, float(g["eps0"]), float(g["V0"]), float(g["freq"]), float(g["t"]), ne, ni, plan, V, E, E32)
    torch.cuda.synchronize()
    np.testing.assert_allclose(V.cpu().numpy(), g["V"], rtol=1e-11, atol=1e-9)
    np.testing.assert_allclose(E.cpu().numpy(), g["E"], rtol=1e-11, atol=1e-7)
    np.testing.assert_allclose(E32.cpu().numpy(), g["E"], rtol=1e-6, atol=1e-4)
    Ji = torch.zeros(N, dtype=torch.float64, device=dev)
    brk = torch.zeros(1, dtype=torch.int32, device=dev)
    Eg = torch.as_tensor(g["E"], device=dev)
    K.heavies_kernel_fluid(N, dx, float(g["dt"]), float(g["mu_i"]), float(g["D_i"]), Eg, ni, Ji, brk)
    torch.cuda.synchronize()
    np.testing.assert_allclose(ni.cpu().numpy(), g["ni_out"], rtol=1e-13)
    np.testing.assert_allclose(Ji.cpu().numpy(), g["Ji"], rtol=1e-12, atol=1e-3)
    assert int(brk.item()) == int(g["brk"])


def test_grid_update_and_clock():
    n = 33
    mom = torch.rand(4, n, dtype=torch.float64, device="cuda")
    mom[0, 3] = 0.0
    mom[3, 3] = 0.0
    ni = torch.ones(n, dtype=torch.float64, device="cuda")
    Te = torch.zeros(n, dtype=torch.float64, device="cuda")
    g2 = torch.zeros(n, dtype=torch.float64, device="cuda")
    K.grid_update(n, mom, ni, Te, g2)
    t = torch.zeros(1, dtype=torch.float64, device="cuda")
    step = torch.zeros(1, dtype=torch.int64, device="cuda")
    for _ in range(3):
        K.advance_clock(t, step, 0.5)
    torch.cuda.synchronize()
    m = mom.cpu().numpy()
    np.testing.assert_allclose(ni.cpu().numpy(), 1.0 + m[1])
    te = (2.0 / 3.0) * m[3] / m[0]
    te[3] = 0.0  # 0/0 -> nan -> 0 (np.nan_to_num, boltzmann.py:646)
    np.testing.assert_allclose(Te.cpu().numpy(), te)
    assert float(t.item()) == 1.5 and int(step.item()) == 3


def test_fused_field_step_equals_the_four_kernels():
    """bz_field_step = grid update, clock, ion fluid, Poisson, bit for bit."""
    g = np.load(os.path.join(G, "field.npz"))
    N, dx, dev = int(g["N"]), float(g["dx"]), "cuda"
    rng = np.random.default_rng(3)
    nn = N + 1
    d = torch.zeros(N - 1, dtype=torch.float64, device=dev)
    l = torch.zeros(N - 1, dtype=torch.float64, device=dev)
    plan = torch.zeros(4 * (N - 1), dtype=torch.float64, device=dev)
    K.poisson_factor(N, dx, d, l, plan)
    mom = torch.as_tensor(np.abs(rng.normal(1e9, 1e8, (4, nn))), device=dev)
    ni0 = torch.as_tensor(g["ni"], device=dev)
    E0 = torch.as_tensor(rng.normal(0, 50, N), device=dev)
    out = []
    for fused in (False, True):
        ni, E = ni0.clone(), E0.clone()
        Te = torch.zeros(nn, dtype=torch.float64, device=dev)
        t = torch.full((1,), 1e-8, dtype=torch.float64, device=dev)
        step = torch.zeros(1, dtype=torch.int64, device=dev)
        V = torch.zeros(N - 1, dtype=torch.float64, device=dev)
        E32 = torch.zeros(N, dtype=torch.float32, device=dev)
        Ji = torch.zeros(N, dtype=torch.float64, device=dev)
        args = (float(g["dt"]), float(g["mu_i"]), float(g["D_i"]))
        if fused:
            K.field_step(N, dx, *args, float(g["eps0"]), float(g["V0"]), float(g["freq"]), mom, ni, Te, None, t,
                         step, plan, V, E, E32, Ji)
        else:
            K.grid_update(nn, mom, ni, Te, None)
            K.advance_clock(t, step, args[0])
            K.heavies_kernel_fluid(N, dx, *args, E, ni, Ji)
            K.EF_kernel(N, dx, float(g["eps0"]), float(g["V0"]), float(g["freq"]), 0.0, mom[0], ni, plan, V, E, E32,
                        t_dev=t)
        torch.cuda.synchronize()
        out.append([a.cpu().numpy() for a in (ni, Te, t, step, V, E, E32, Ji)])
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("N", [None, 130, 1024, 4096])
def test_cooperative_field_step_equals_the_one_cta_kernel(N, mode):
    """bz_field_step_coop (the float64 work over ceil((N-1)/64) CTAs; mode 1 a cooperative
    launch with grid-wide barriers, mode 2 one thread-block cluster with its hardware
    barrier) against bz_field_step: the densities, the clock and the ion fluxes bit for bit,
    the Poisson solution to the association of its float64 sums. The cluster form takes at
    most 16 CTAs (1025 nodes) and refuses more."""
    g = np.load(os.path.join(G, "field.npz"))
    N = int(g["N"]) if N is None else N
    dx, dev = 2.54 / N if N != int(g["N"]) else float(g["dx"]), "cuda"
    rng = np.random.default_rng(N)
    nn = N + 1
    d = torch.zeros(N - 1, dtype=torch.float64, device=dev)
    l = torch.zeros(N - 1, dtype=torch.float64, device=dev)
    plan = torch.zeros(4 * (N - 1), dtype=torch.float64, device=dev)
    K.poisson_factor(N, dx, d, l, plan)
    mom = torch.as_tensor(np.abs(rng.normal(1e9, 1e8, (4, nn))), device=dev)
    ni0 = torch.as_tensor(np.abs(rng.normal(1e9, 2e8, nn)), device=dev)
    E0 = torch.as_tensor(rng.normal(0, 50, N), device=dev)
    out = []
    for coop in (False, True):
        ni, E = ni0.clone(), E0.clone()
        Te = torch.zeros(nn, dtype=torch.float64, device=dev)
        g2 = torch.zeros(nn, dtype=torch.float64, device=dev)
        t = torch.full((1,), 1.23e-8, dtype=torch.float64, device=dev)
        step = torch.zeros(1, dtype=torch.int64, device=dev)
        V = torch.zeros(N - 1, dtype=torch.float64, device=dev)
        E32 = torch.zeros(N, dtype=torch.float32, device=dev)
        Ji = torch.zeros(N, dtype=torch.float64, device=dev)
        brk = torch.zeros(1, dtype=torch.int32, device=dev)
        args = (N, dx, float(g["dt"]), float(g["mu_i"]), float(g["D_i"]), float(g["eps0"]), float(g["V0"]),
                float(g["freq"]), mom, ni, Te, g2, t, step, plan, V, E, E32, Ji, brk)
        if coop:
            K.field_step_select(mode)
            try:
                if mode == 2 and N > 1025:
                    with pytest.raises(_lib.BzError):
                        K.field_step_coop(*args)
                    return
                K.field_step_coop(*args)
            finally:
                K.field_step_select(0)
        else:
            K.field_step(*args)
        torch.cuda.synchronize()
        out.append({k: a.cpu().numpy() for k, a in zip(("ni", "Te", "g2", "t", "step", "V", "E", "E32", "Ji", "brk"),
                                                       (ni, Te, g2, t, step, V, E, E32, Ji, brk))})
    a, b = out
    for k in ("ni", "Te", "g2", "t", "step", "Ji", "brk"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    for k in ("V", "E"):
        np.testing.assert_allclose(b[k], a[k], rtol=1e-11, atol=1e-11 * np.abs(a[k]).max(), err_msg=k)
