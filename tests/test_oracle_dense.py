"""The oracle with the dense test weight (a QED tensor with no closed form,
include/hlbl_gb300_qed.h) against the reference's own sources run with the
same weight served through KQED's QED_Mkernel_L2
(tests/golden/reference_dense_qed.json, made by make_golden_dense.py). CPU
only."""
import json
import os

import numpy as np
import pytest

import support as S

with open(os.path.join(os.path.dirname(__file__), "golden", "reference_dense_qed.json")) as fh:
    GD = json.load(fh)


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def test_fixture_seed_is_the_tests_seed():
    assert GD["dense_seed"] == S.DENSE_SEED


def test_dense_tensor_has_no_kronecker_structure():
    """Every entry of kerv is nonzero and the (rho, sigma) blocks are unrelated,
    unlike the stand-in, whose entries vanish off its Kronecker pattern."""
    x, y = np.array([0.3, -0.2, 0.5, 0.1]), np.array([-0.4, 0.25, 0.05, 0.6])
    kv = np.zeros(384)
    with S.dense_qed():
        S.oracle().oracle_qed_kernel(0.4, S.vp(x), S.vp(y), S.vp(kv))
    std = np.zeros(384)
    S.oracle().oracle_qed_kernel(0.4, S.vp(x), S.vp(y), S.vp(std))
    assert np.count_nonzero(kv) == 384
    assert np.count_nonzero(std) < 384
    k = kv.reshape(6, 64)
    assert np.linalg.matrix_rank(k) == 6


@pytest.mark.parametrize("case", GD["kernel_sum"], ids=lambda c: c["name"])
def test_kernel_sum_matches_reference_dense(case):
    src, y = S.case_inputs(case)
    with S.dense_qed():
        got = S.oracle_kernel_sum(src, y, case["gsx"], case["yv"], case["xunit"], case["lattice"])
    assert S.rel_err(got, case["kernel_sum"]) <= 1e-12


def test_pass2_matches_reference_dense():
    p = GD["pass2"]
    src, y = S.random_block(p["lattice"], p["seeds"][0]), S.random_block(p["lattice"], p["seeds"][1])
    with S.dense_qed():
        for f in (0, 1):
            dzu, dzsu = S.oracle_dz(src, y, f, p["gsx"], p["lattice"])
            g_dzu, g_dzsu = S.oracle_gammas(dzu, dzsu)
            got = S.oracle_4pt(g_dzu, g_dzsu, src, y, f, p["gsx"], p["xunit"], p["yv"], p["lattice"])
            assert S.rel_err(got, p["kernel_sum_per_flavour"][f]) <= 1e-12


@pytest.mark.parametrize("case", GD["pieces_2p2"], ids=lambda c: c["name"])
def test_pieces_2p2_match_reference_dense(case):
    lat = case["lattice"]
    fwd = S.random_block(lat, case["seed"])
    with S.dense_qed():
        p1, p234 = S.oracle_pieces_2p2(fwd, case["gsw"], case["targets"], case["xunit"], lat)
    assert rel(p1, np.asarray(case["p1"]).reshape(p1.shape)) < 1e-13
    ref = np.asarray(case["p234"]).reshape(p234.shape)
    for t in range(p234.shape[0]):
        for g in range(5):
            assert rel(p234[t, g], ref[t, g]) < 1e-12, (t, g)


def test_dense_switch_is_scoped():
    case = S.golden()["kernel_sum"][0]
    src, y = S.case_inputs(case)
    with S.dense_qed():
        pass
    got = S.oracle_kernel_sum(src, y, case["gsx"], case["yv"], case["xunit"], case["lattice"])
    assert S.rel_err(got, case["kernel_sum"]) <= 1e-12
