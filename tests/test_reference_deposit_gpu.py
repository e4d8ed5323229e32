"""libbz's deposit against the reference's own GPU deposit kernels (reda + redcheck of
kernels/reduction/cuda_reduction/kernels-new.cu, compiled from the reference sources into
oracle/_ref by oracle.ref_deposit.build and launched unchanged through the driver API) on
the same particles: node sums of w and of w*energy to 1e-6 (the deposit target is 1e-5):
libbz sums each CTA's particles in float32 shared memory before adding them to the float64
grid, and forms the energy from the float32 state in float32; the reference adds every
particle to the float64 grid. bnf is a power of two: redcheck's shared-memory tree
(kernels-new.cu:26-35) halves blockDim = bnf, so for other bnf it drops fine bins (with
bnf = 3 the third of every node), and it writes each node's sum in place over fine bins
that a lower block may not have read yet (kernels-new.cu:40-47)."""
import math
import os

import numpy as np
import pytest
import torch

from boltzmann_gb300 import kernels as K
from oracle import ref_deposit as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dep():
    if not os.path.exists(R.CUBIN):
        pytest.skip(f"{R.CUBIN} not built (the reference sources were not present at build time)")
    return R.ReferenceDeposit()


@pytest.mark.parametrize("n,N,bnf", [(100_000, 128, 4), (257, 16, 1), (50_000, 1024, 4), (20_000, 100, 2)])
def test_deposit_matches_the_reference_kernels(dep, n, N, bnf):
    L = 2.54
    rng = np.random.default_rng(n + N)
    x = rng.uniform(0, L, n).astype(np.float32).astype(np.float64)
    x[: min(n, N + 1)] = np.linspace(0, L, N + 1)[: min(n, N + 1)].astype(np.float32)  # node positions too
    v = (rng.normal(0, math.sqrt(1.5 * 1.17255e11), (n, 3))).astype(np.float32).astype(np.float64)
    w = rng.uniform(1e3, 1e4, n).astype(np.float32).astype(np.float64)
    t = lambda a: torch.as_tensor(a, device="cuda")
    ref = R.reference_moments(dep, t(x), t(v[:, 0]), t(v[:, 1]), t(v[:, 2]), t(w), N, L, bnf).cpu().numpy()
    seg = K.SegmentSet(max(1, -(-n // 1024)), 1024, torch.float32)
    seg.load(x, v[:, 0], v[:, 1], v[:, 2], w)
    p = K.make_params(n_faces=N, n_nodes=N + 1, bnf=bnf, advect=1, L=L, dx=L / N, dt=1e-12, nn=3.22e22)
    mom = torch.zeros(4, N + 1, dtype=torch.float64, device="cuda")
    K.seg_deposit(p, seg, mom)
    ours = mom.cpu().numpy()
    np.testing.assert_allclose(ours[0], ref[0], rtol=1e-6, atol=1e-6 * ref[0].max())
    np.testing.assert_allclose(ours[3], ref[3], rtol=1e-6, atol=1e-6 * ref[3].max())
    assert np.all(ours[1] == 0) and np.all(ref[1] == 0)


def test_node_assignment_is_exact(dep):
    """Unit weights: every node count must equal the reference's, including particles that
    sit exactly on a node boundary (x = 0.837158203125 with 1024 cells and bnf 4 gives
    (x + dx/2)/(L + dx) * 4100 = 1352 exactly, node 338)."""
    n, N, L, bnf = 2_000_000, 1024, 2.54, 4
    rng = np.random.default_rng(5)
    x = rng.uniform(0, L, n).astype(np.float32).astype(np.float64)
    edge = np.array([0.837158203125, 2.325439453125, 1.395263671875, 2.015380859375, 1.705322265625])
    x[: 5 * 1000] = np.repeat(edge, 1000)
    z = np.zeros(n)
    w = np.ones(n)
    t = lambda a: torch.as_tensor(a, device="cuda")
    ref = R.reference_moments(dep, t(x), t(z), t(z), t(z), t(w), N, L, bnf).cpu().numpy()
    seg = K.SegmentSet(-(-n // 2048), 2048, torch.float32)
    seg.load(x, z, z, z, w)
    p = K.make_params(n_faces=N, n_nodes=N + 1, bnf=bnf, advect=1, L=L, dx=L / N, dt=1e-12, nn=3.22e22)
    mom = torch.zeros(4, N + 1, dtype=torch.float64, device="cuda")
    K.seg_deposit(p, seg, mom)
    assert np.array_equal(mom[0].cpu().numpy(), ref[0])
    assert ref[0][338] >= 1000  # the boundary particles are in the upper node
