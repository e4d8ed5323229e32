"""libbz's deposit against the reference's own GPU deposit kernels (reda + redcheck of
kernels/reduction/cuda_reduction/kernels-new.cu, compiled from the reference sources into
oracle/_ref by oracle.ref_deposit.build and launched unchanged through the driver API) on
the same particles: node sums of w to 1e-12 (float64 sums in another order), of w*energy
to 1e-6 (libbz forms the energy from the float32 state in float32)."""
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


@pytest.mark.parametrize("n,N,bnf", [(100_000, 128, 4), (257, 16, 1), (50_000, 1024, 4), (20_000, 100, 3)])
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
    np.testing.assert_allclose(ours[0], ref[0], rtol=1e-12, atol=1e-12 * ref[0].max())
    np.testing.assert_allclose(ours[3], ref[3], rtol=1e-6, atol=1e-6 * ref[3].max())
    assert np.all(ours[1] == 0) and np.all(ref[1] == 0)
