"""The 2+2 oracle (oracle/hlbl_oracle.c: oracle_pi, oracle_p1_2p2, oracle_p234,
oracle_pieces_2p2) against the reference's own 2+2 code run as a host
emulation (tests/golden/reference_2p2.json, made by make_golden_2p2.py), and
the index structure of P1 and P234 that the reference's test checks
(sanity_check/test_contract_random.cpp:69-137)."""
import json
import os

import numpy as np
import pytest

from support import oracle_pieces_2p2, random_block

GOLDEN_2P2 = os.path.join(os.path.dirname(__file__), "golden", "reference_2p2.json")


def golden_2p2():
    with open(GOLDEN_2P2) as fh:
        return json.load(fh)


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


CASES = golden_2p2()["pieces_2p2"]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_pieces_match_reference(case):
    lat = case["lattice"]
    fwd = random_block(lat, case["seed"])
    p1, p234 = oracle_pieces_2p2(fwd, case["gsw"], case["targets"], case["xunit"], lat)
    ref_p1 = np.asarray(case["p1"]).reshape(p1.shape)
    ref_p234 = np.asarray(case["p234"]).reshape(p234.shape)
    assert rel(p1, ref_p1) < 1e-13
    # every (target, geometry) row against its own scale
    for t in range(p234.shape[0]):
        for g in range(5):
            assert rel(p234[t, g], ref_p234[t, g]) < 1e-12, (t, g)


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_index_structure(case):
    """P1 is zero beyond each extent; P2_0, P2_1, P3, P4_0 fill rho < sigma
    only, P4_1 everything but rho == sigma (contract.hpp:27-33)."""
    lat = case["lattice"]
    fwd = random_block(lat, case["seed"])
    p1, p234 = oracle_pieces_2p2(fwd, case["gsw"], case["targets"], case["xunit"], lat)
    for r in range(4):
        assert np.all(p1[r, :, :, lat[r]:] == 0)
        assert np.all(np.abs(p1[r, :, :, :lat[r]]).sum(axis=-1) > 0)
    blk = p234.reshape(-1, 5, 4, 4, 4)
    for rho in range(4):
        for sigma in range(4):
            upper = rho < sigma
            for g in range(4):
                nz = np.any(blk[:, g, rho, sigma] != 0)
                assert nz == upper, (g, rho, sigma)
            assert np.any(blk[:, 4, rho, sigma] != 0) == (rho != sigma)
    # P1 summed over zeta is the sum of Pi over the lattice, the same for every rho
    tot = p1.sum(axis=-1)
    for r in range(1, 4):
        assert rel(tot[r], tot[0]) < 1e-12


def test_rank_split_partials_and_sum():
    """compute_2p2_gpu's per-rank partials on a 2-rank split (flavour 1),
    and that they sum to the single-rank result of the whole lattice."""
    sp = golden_2p2()["compute_2p2_split"]
    glob, loc = sp["global"], sp["local"]
    n_y = len(sp["targets"])
    full = random_block(glob, sp["seed"])
    V, Vl = int(np.prod(glob)), int(np.prod(loc))
    s1 = np.zeros((4, 4, 4, max(glob)))
    s234 = np.zeros((n_y, 5, 64))
    for r, rk in enumerate(sp["ranks"]):
        sl = np.ascontiguousarray(full.reshape(2, 12, V, 24)[:, :, r * Vl:(r + 1) * Vl, :]).ravel()
        p1, p234 = oracle_pieces_2p2(sl, sp["gsw"], sp["targets"], sp["xunit"], glob, local=loc,
                                     pc=rk["proc_coords"], iflavor=sp["iflavor"])
        ref1 = np.asarray(rk["p1"]).reshape(p1.shape)
        ref234 = np.asarray(rk["p234_raw"]).reshape(5, n_y, 64).transpose(1, 0, 2)
        assert rel(p1, ref1) < 1e-13
        for t in range(n_y):
            for g in range(5):
                assert rel(p234[t, g], ref234[t, g]) < 1e-12, (r, t, g)
        s1 += p1
        s234 += p234
    w1, w234 = oracle_pieces_2p2(full, sp["gsw"], sp["targets"], sp["xunit"], glob,
                                 iflavor=sp["iflavor"])
    assert rel(s1, w1) < 1e-13
    assert rel(s234, w234) < 1e-12


def test_flavour_symmetry_of_pi_trace():
    """Swapping the flavours of the block swaps iflavor: the pieces of
    flavour 1 equal those of flavour 0 on the swapped block."""
    lat = [4, 2, 2, 4]
    fwd = random_block(lat, 17)
    sw = np.ascontiguousarray(fwd.reshape(2, -1)[::-1]).ravel()
    a1, a234 = oracle_pieces_2p2(fwd, [1, 0, 1, 2], [[0, 1, 1, 3]], 0.8, lat, iflavor=1)
    b1, b234 = oracle_pieces_2p2(sw, [1, 0, 1, 2], [[0, 1, 1, 3]], 0.8, lat, iflavor=0)
    assert rel(a1, b1) < 1e-14 and rel(a234, b234) < 1e-14


def test_empty_target_list():
    lat = [2, 2, 2, 2]
    p1, p234 = oracle_pieces_2p2(random_block(lat, 1), [0, 0, 0, 0], np.zeros((0, 4)), 1.0, lat)
    assert p234.shape == (0, 5, 64) and np.all(np.isfinite(p1))


@pytest.mark.parametrize("case", golden_2p2()["plan_2p2"], ids=lambda c: c["name"])
def test_plan_2p2_matches_reference(case):
    """Which solves get the 2+2 over several chains (schedule.cpp:284-347):
    the reference's plan and warning lines."""
    from hlbl_gb300 import schedule

    chains = [schedule.build_schedule(tuple(h), case["stride"], case["n_steps"], tuple(o))
              for h, o in zip(case["h"], case["origins"])]
    plan = schedule.plan_2p2(chains, [tuple(s) for s in case["sources"]], case["lattice"])
    mine_at = sorted([c] + list(pos) + [idx] for c, d in enumerate(plan.at) for pos, idx in d.items())
    assert mine_at == sorted(case["at"])
    assert [list(p) + [c, w] for p, c, w in plan.not_sources] == case["not_sources"]
    assert plan.unsolved == case["unsolved"]
    assert schedule.report_2p2(plan, [tuple(s) for s in case["sources"]]) == case["report"]
