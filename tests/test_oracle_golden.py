"""Pin the C oracle (oracle/bz_oracle.c) to the reference's own outputs.

The fixtures under tests/golden were produced by running the reference's Python source
(jfabell/boltzmann, 1bin/3bin/5bin) on the CPU (tests/golden/make_golden.py). Every
random number the reference drew is stored in the fixture and replayed here.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(G, name))


@pytest.mark.parametrize("case", ["push_1torr", "push_0p1torr"])
def test_push_and_post_match_reference(case):
    g = load(case + ".npz")
    N, n = int(g["N"]), len(g["x"])
    p = O.make_params(N, L=float(g["L"]), bnf=int(g["bnf"]), dt=float(g["dt"]), nn=float(g["nn"]), xs_mode=1)
    data, tosum = O.soa_to_aos(g["x"], g["v"][:, 0], g["v"][:, 1], g["v"][:, 2], g["w"], cap=3 * n)
    nni = O.push(p, data, tosum, n, g["E"], g["R"], g["gas"])
    assert nni == int(g["nni"])
    m = n + nni
    kd, kt = g["k_data"], g["k_tosum"]
    # libm differences only: float64 round-off
    np.testing.assert_allclose(data[:m], kd, rtol=1e-13, atol=1e-9)
    np.testing.assert_allclose(tosum[:m], kt, rtol=1e-13, atol=1e-12)
    mom, nnew = O.post(p, data, tosum, m)
    assert nnew == int(g["Nnew"])
    for j, k in enumerate(["ne", "ni_src", "ns_src", "nrg"]):
        np.testing.assert_allclose(mom[j], g[k], rtol=1e-13, atol=1e-9)
    np.testing.assert_allclose(data[:nnew], g["c_data"], rtol=1e-13, atol=1e-9)
    np.testing.assert_allclose(tosum[:nnew], g["c_tosum"], rtol=1e-13, atol=1e-12)


@pytest.mark.parametrize("variant", ["1bin", "3bin", "5bin"])
def test_bins_match_reference(variant):
    g = load(f"bins_{variant}.npz")
    N = int(g["N"])
    p = O.make_params(N, L=float(g["L"]))
    v = g["v"]
    max_ppc = int(g["max_ppc"])
    counts, lists = O.bin_particles(p, g["x"], v[:, 0], v[:, 1], v[:, 2], g["w"], g["edges"], max_ppc)
    np.testing.assert_array_equal(counts, g["counts"])
    for b in range(counts.shape[0]):
        for c in range(N + 1):
            k = min(int(counts[b, c]), max_ppc)
            np.testing.assert_array_equal(lists[b, :k, c], g["tables"][b, :k, c])


@pytest.mark.parametrize("variant", ["1bin", "3bin", "5bin"])
def test_resample_matches_reference(variant):
    g = load(f"resample_{variant}.npz")
    N = int(g["N"])
    p = O.make_params(N, L=float(g["L"]))
    v, x, w = g["v"], g["x"], g["w"]
    n = len(x)
    T = g["targets"]
    nb = len(T)
    max_ppc = (10 * T).astype(np.int64)  # boltzmann.py:542 and its 3/5-bin copies
    counts, lists = O.bin_particles(p, x, v[:, 0], v[:, 1], v[:, 2], w, g["edges"], int(max_ppc.max()))
    np.testing.assert_array_equal(counts, g["counts"])
    data, tosum = O.soa_to_aos(x, v[:, 0], v[:, 1], v[:, 2], w, cap=4 * n)
    tosum[:n, 3] = (tosum[:n, 3] * w) / w
    na, used = O.resample(p, data, tosum, n, nb, T, float(g["min_wt"]), max_ppc, counts, lists, g["draw_u"], flags=1)
    assert used == len(g["draw_u"])
    assert na == int(g["out_n"])
    np.testing.assert_allclose(data[:na], g["out_data"], rtol=1e-12, atol=1e-9)
    np.testing.assert_allclose(tosum[:na], g["out_tosum"], rtol=1e-12, atol=1e-9)


def test_field_and_fluid_match_reference():
    g = load("field.npz")
    N = int(g["N"])
    V, E = O.poisson(N, float(g["dx"]), float(g["eps0"]), float(g["V0"]), float(g["freq"]), float(g["t"]),
                     g["ne"], g["ni"])
    np.testing.assert_allclose(V, g["V"], rtol=1e-11, atol=1e-9)
    np.testing.assert_allclose(E, g["E"], rtol=1e-11, atol=1e-7)
    ni, Ji, brk = O.fluid(N, float(g["dx"]), float(g["dt"]), float(g["mu_i"]), float(g["D_i"]), g["E"], g["ni"])
    np.testing.assert_allclose(ni, g["ni_out"], rtol=1e-13)
    np.testing.assert_allclose(Ji, g["Ji"], rtol=1e-13, atol=1e-3)
    assert brk == int(g["brk"])


def test_philox_known_answer():
    """Philox4x32-10 known-answer vectors published with Random123 (kat_vectors)."""
    assert list(O.philox([0, 0, 0, 0], [0, 0])) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert list(O.philox([0xffffffff] * 4, [0xffffffff] * 2)) == [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert list(O.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0])) == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_philox_seven_rounds_sanity():
    """The push draws from Philox4x32-7 (the round count Salmon et al. report as passing
    BigCrush). The round-parametrised generator gives Philox4x32-10 at 10 rounds, and its
    7-round words are uniform and uncorrelated at the level a quick check sees: chi-square
    of the top byte over 2^18 words, lag-1 correlation of consecutive counters."""
    from scipy.stats import chi2
    ctr0 = [0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344]
    key = [0xa4093822, 0x299f31d0]
    assert list(O.philox(ctr0, key, rounds=10)) == list(O.philox(ctr0, key))
    words = np.array([O.philox([i, 17, 0, 1], key, rounds=7) for i in range(1 << 16)], dtype=np.uint64).ravel()
    hist = np.bincount((words >> 24).astype(np.int64), minlength=256)
    stat = float(((hist - words.size / 256) ** 2 / (words.size / 256)).sum())
    assert chi2.sf(stat, 255) > 1e-4, stat
    u = (words.astype(np.float64) + 0.5) / 2.0 ** 32
    r = np.corrcoef(u[:-4:4], u[4::4])[0, 1]  # word 0 of counter i against word 0 of counter i+1
    assert abs(r) < 5.0 / np.sqrt(u.size / 4), r


def test_low_bits_uniform_is_uniform_and_independent():
    """The float32 push takes the ionization child's azimuth from the 23 bits of the collision
    draw's first three words that its other uniforms leave unused (low 9, 9 and 5 bits). On
    2^16 seven-round draws it is uniform (chi-square over 64 bins) and uncorrelated with the
    four high-bit uniforms of the same draw (which decide and orient the collision)."""
    from scipy.stats import chi2
    key = [0xa4093822, 0x299f31d0]
    w = np.array([O.philox([i, 23, 0, 1], key, rounds=7) for i in range(1 << 16)], dtype=np.uint64)
    r5 = ((w[:, 0] << 23) | ((w[:, 1] & 511) << 14) | ((w[:, 2] & 511) << 5)) & 0xFFFFFFFF
    u5 = ((r5 >> 9).astype(np.float64) + 0.5) * 2.0 ** -23
    hist = np.bincount((u5 * 64).astype(np.int64), minlength=64)
    stat = float(((hist - u5.size / 64) ** 2 / (u5.size / 64)).sum())
    assert chi2.sf(stat, 63) > 1e-4, stat
    assert abs(u5.mean() - 0.5) < 5 * np.sqrt(1 / 12 / u5.size)
    for k in range(4):
        uk = ((w[:, k] >> 9).astype(np.float64) + 0.5) * 2.0 ** -23
        assert abs(np.corrcoef(u5, uk)[0, 1]) < 5.0 / np.sqrt(u5.size), k
