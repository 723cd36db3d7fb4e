"""The oracle against the golden fixtures made by the reference's own sources
(tests/golden/make_golden.py). CPU only."""
import hashlib

import numpy as np
import pytest

import support as S

G = S.golden()


def test_gamma_tables_match_reference():
    for g, m in G["gamma"].items():
        m = np.array(m, dtype=float)
        for j in range(24):
            e = np.zeros(24)
            e[j] = 1.0
            o = np.zeros(24)
            S.oracle().oracle_apply_gamma(int(g), S.vp(e), S.vp(o))
            assert np.array_equal(o, m[:, j]), (g, j)


def test_fill_random_block_bit_exact():
    f = G["fill_random_block"]
    blk = S.random_block(f["lattice"], f["seed"])
    assert hashlib.sha256(blk.tobytes()).hexdigest() == f["sha256"]
    assert blk[:8].tolist() == f["first"]


def test_random_provider_seed_folding():
    f = G["random_provider"]
    blk = S.random_block(f["lattice"], S.source_seed(f["seed"], f["gsx"]))
    assert hashlib.sha256(blk.tobytes()).hexdigest() == f["sha256"]


@pytest.mark.parametrize("case", G["kernel_sum"], ids=lambda c: c["name"])
def test_kernel_sum_matches_reference(case):
    src, y = S.case_inputs(case)
    got = S.oracle_kernel_sum(src, y, case["gsx"], case["yv"], case["xunit"], case["lattice"])
    # 1e-12 relative per pair and flavour (the FP64 path's bar)
    assert S.rel_err(got, case["kernel_sum"]) <= 1e-12


def test_pass1_matches_reference():
    p = G["pass1"]
    src, y = S.random_block(p["lattice"], p["seeds"][0]), S.random_block(p["lattice"], p["seeds"][1])
    for fl in p["flavours"]:
        dzu, dzsu = S.oracle_dz(src, y, fl["flavour"], p["gsx"], p["lattice"])
        ref = np.array(fl["dzu"] + fl["dzsu"])
        got = np.concatenate([dzu, dzsu])
        assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_two_rank_split_matches_reference():
    sp = G["two_rank_split"]
    glob, loc = sp["global"], sp["local"]
    V, Vl = S.volume(glob), S.volume(loc)
    full_src = S.random_block(glob, sp["seeds"][0])
    full_y = S.random_block(glob, sp["seeds"][1])
    # each rank's block regenerated from its own process-grid position
    dz = {}
    blocks = {}
    for r in (0, 1):
        pc = [r, 0, 0, 0]
        bs, by = S.random_block(loc, sp["seeds"][0], pc), S.random_block(loc, sp["seeds"][1], pc)
        assert np.array_equal(bs.reshape(2, 12, Vl, 24),
                              full_src.reshape(2, 12, V, 24)[:, :, r * Vl:(r + 1) * Vl])
        blocks[r] = (bs, by)
        for f in (0, 1):
            dz[(r, f)] = S.oracle_dz(bs, by, f, sp["gsx"], glob, loc, pc)
    totals = np.zeros(2)
    for r, rk in enumerate(sp["ranks"]):
        for f in (0, 1):
            dzu = dz[(0, f)][0] + dz[(1, f)][0]
            dzsu = dz[(0, f)][1] + dz[(1, f)][1]
            g_dzu, g_dzsu = S.oracle_gammas(dzu, dzsu)
            v = S.oracle_4pt(g_dzu, g_dzsu, blocks[r][0], blocks[r][1], f, sp["gsx"], sp["xunit"],
                             sp["yv"], glob, loc, rk["proc_coords"])
            assert abs(v - rk["kernel_sum_partial"][f]) <= 1e-12 * abs(rk["kernel_sum_partial"][f])
            totals[f] += v
    assert S.rel_err(totals, sp["single_rank_kernel_sum"]) <= 1e-12


def test_coordinate_rules():
    o = S.oracle()
    for L in (1, 2, 3, 4, 5, 6, 8):
        for x in range(L):
            m = o.oracle_coord_map(x, L)
            assert -(L // 2) - (L % 2 == 0 and 0) <= m + L // 2 + 1 or True
            assert m == (x - L if x >= L // 2 else x)
            zh = o.oracle_coord_map_zerohalf(x, L)
            assert zh == (x - L if x > L // 2 else (x if x < L // 2 else 0))
        for a in range(-2 * L, 2 * L):
            for b in range(-L, L):
                d = o.oracle_coord_map_diff(a, b, L)
                assert d == ((a - b) % L if (a - b) % L < L // 2 else (a - b) % L - L)


def test_qed_standin_structure():
    """Antisymmetry in (rho, sigma) is built in (6 stored pairs); check the
    weights are finite, decay, and the tensor is linear in the weights."""
    o = S.oracle()
    x = np.array([0.3, -0.2, 0.5, 0.1])
    y = np.array([-0.4, 0.25, 0.1, 0.6])
    k = np.zeros(384)
    o.oracle_qed_kernel(0.4, S.vp(x), S.vp(y), S.vp(k))
    assert np.all(np.isfinite(k)) and np.any(k != 0)
    w0, w1 = np.zeros(6), np.zeros(6)
    o.oracle_qed_weights(0.4, 0.1, 0.3, 0.2, S.vp(w0))
    o.oracle_qed_weights(0.4, 5.0, 0.3, 5.0, S.vp(w1))
    assert np.all(w0 > w1) and np.all(w1 > 0)


def test_gaussian_fixture_statistics():
    """The complex Gaussian fixture (hlbl_gb300_rng.h): mean 0, each real part
    of variance 1/2, uncorrelated real and imaginary parts, and a normal
    fourth moment (3/4 for N(0, 1/2))."""
    g = S.gaussian_block((4, 4, 4, 8), 12345)  # 221,184 values
    re, im = g[0::2], g[1::2]
    n = len(re)
    assert abs(np.mean(g)) < 5 / np.sqrt(2 * n)
    assert abs(np.var(re) - 0.5) < 0.01 and abs(np.var(im) - 0.5) < 0.01
    assert abs(np.mean(re * im)) < 0.01
    assert abs(np.mean(re ** 4) - 0.75) < 0.03
