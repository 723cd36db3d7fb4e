"""The 2+2 pieces on the GPU (pieces_2p2.cu) through the C ABI, against the
reference's own outputs (tests/golden/reference_2p2.json) and the oracle.
Needs a GPU.

Tolerances, per (target, geometry) row of P234 relative to that row's largest
element, and for P1 relative to its largest element: FP64 path 1e-12
(P1 1e-13); FP32 path 1e-5 (P1 1e-6)."""
import json
import os

import numpy as np
import pytest

import support as S

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
TOL64, TOL64_P1 = 1e-12, 1e-13
TOL32, TOL32_P1 = 1e-5, 1e-6

with open(os.path.join(os.path.dirname(__file__), "golden", "reference_2p2.json")) as _fh:
    G2 = json.load(_fh)


def dev(a: np.ndarray):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def hg():
    import hlbl_gb300

    return hlbl_gb300


def rel(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def assert_rows(got, want, tol):
    """Every (target, geometry) row of P234 against its own scale."""
    got = np.asarray(got).reshape(-1, 5, 64)
    want = np.asarray(want).reshape(-1, 5, 64)
    for t in range(want.shape[0]):
        for g in range(5):
            e = rel(got[t, g], want[t, g])
            assert e <= tol, (t, g, e)
            # the zero pattern is exact
            assert np.all(got[t, g][want[t, g] == 0] == 0), (t, g)


@pytest.mark.parametrize("case", G2["pieces_2p2"], ids=lambda c: c["name"])
def test_pieces_fp64_match_reference(hg, case):
    lat = case["lattice"]
    fwd = S.random_block(lat, case["seed"])
    with hg.Contractor(lat) as c:
        r = c.pieces_2p2(dev(fwd), case["gsw"], case["targets"], case["xunit"], hg.FP64)
    assert rel(r.p1, case["p1"]) <= TOL64_P1
    assert_rows(r.p234, case["p234"], TOL64)


@pytest.mark.parametrize("case", G2["pieces_2p2"], ids=lambda c: c["name"])
def test_pieces_fp32_within_1e5(hg, case):
    lat = case["lattice"]
    fwd = S.random_block(lat, case["seed"])
    with hg.Contractor(lat) as c:
        r = c.pieces_2p2(dev(fwd), case["gsw"], case["targets"], case["xunit"], hg.FP32)
    assert rel(r.p1, case["p1"]) <= TOL32_P1
    assert_rows(r.p234, case["p234"], TOL32)


def test_compute_2p2_rank_split_raw_layout(hg):
    """compute_2p2_gpu's layout [5][n_y][64], flavour 1, each rank of a 2-rank
    split on its own context (its local block and proc_coords), against the
    reference's per-rank partials."""
    sp = G2["compute_2p2_split"]
    glob, loc = sp["global"], sp["local"]
    full = S.random_block(glob, sp["seed"])
    V, Vl = int(np.prod(glob)), int(np.prod(loc))
    for r, rk in enumerate(sp["ranks"]):
        sl = full.reshape(2, 12, V, 24)[:, :, r * Vl:(r + 1) * Vl, :]
        with hg.Contractor(glob, loc, rk["proc_coords"]) as c:
            p1, p234 = c.compute_2p2(dev(sl), sp["iflavor"], sp["gsw"], sp["targets"], sp["xunit"],
                                     hg.FP64)
        assert rel(p1, rk["p1"]) <= TOL64_P1
        n_y = len(sp["targets"])
        got = p234.reshape(5, n_y, 64).transpose(1, 0, 2)
        want = np.asarray(rk["p234_raw"]).reshape(5, n_y, 64).transpose(1, 0, 2)
        assert_rows(got, want, TOL64)


@pytest.mark.parametrize("prec,tol,tol1", [(0, TOL64, TOL64_P1), (1, TOL32, TOL32_P1)])
def test_many_targets_chunks_vs_oracle(hg, prec, tol, tol1):
    """40 targets (more than one launch's 32) on an 8x6x4x10 lattice, every
    target a distinct site incl. the source and L/2 offsets."""
    lat = [8, 6, 4, 10]
    fwd = S.gaussian_block(lat, 31)
    rng = np.random.default_rng(5)
    gsw = [3, 5, 0, 9]
    targets = [gsw, [(gsw[0] + 4) % 8, (gsw[1] + 3) % 6, (gsw[2] + 2) % 4, (gsw[3] + 5) % 10]]
    while len(targets) < 40:
        t = [int(rng.integers(0, L)) for L in lat]
        if t not in targets:
            targets.append(t)
    xu = 0.11
    o1, o234 = S.oracle_pieces_2p2(fwd, gsw, targets, xu, lat)
    with hg.Contractor(lat) as c:
        r = c.pieces_2p2(dev(fwd), gsw, targets, xu, prec)
    assert rel(r.p1, o1) <= tol1
    assert_rows(r.p234, o234, tol)


def test_async_graph_and_empty_targets(hg):
    lat = [4, 4, 6, 4]
    fwd = dev(S.random_block(lat, 9))
    gsw, targets, xu = [1, 2, 3, 0], [[0, 0, 0, 0], [2, 3, 1, 1], [3, 3, 5, 3]], 0.4
    with hg.Contractor(lat) as c:
        ref = c.pieces_2p2(fwd, gsw, targets, xu, hg.FP32)
        d1 = torch.zeros(64 * c.lmax, dtype=torch.float64, device="cuda")
        d234 = torch.zeros(len(targets) * 320, dtype=torch.float64, device="cuda")
        c.pieces_2p2_async(fwd, gsw, targets, xu, d1, d234, hg.FP32)
        c.check()
        assert np.array_equal(d1.cpu().numpy(), ref.p1)
        assert np.array_equal(d234.cpu().numpy(), ref.p234)
        # recorded into a CUDA graph, replayed
        g1, g234 = torch.zeros_like(d1), torch.zeros_like(d234)
        c.reserve_2p2()
        c.graph_begin()
        c.pieces_2p2_async(fwd, gsw, targets, xu, g1, g234, hg.FP32)
        graph = c.graph_end()
        torch.cuda.synchronize()
        assert torch.count_nonzero(g234).item() == 0
        graph.launch()
        torch.cuda.synchronize()
        assert torch.equal(g1, d1) and torch.equal(g234, d234)
        graph.close()
        # no targets: P1 only
        e = c.pieces_2p2(fwd, gsw, [], xu, hg.FP64)
        assert e.p234.size == 0
        o1, _ = S.oracle_pieces_2p2(S.random_block(lat, 9), gsw, [[0, 0, 0, 0]], xu, lat)
        assert rel(e.p1, o1) <= TOL64_P1


def test_pieces_from_fp32_tile_copy(hg):
    """Pi read from the block's FP32 tile copy: bit-identical to the FP32 path
    on the FP64 block (the copy holds the same rounded values), and within
    the FP32 bar of the reference."""
    case = G2["pieces_2p2"][1]  # odd extents, a padded last tile
    lat = case["lattice"]
    fwd = dev(S.random_block(lat, case["seed"]))
    with hg.Contractor(lat) as c:
        x32 = torch.empty(c.f32_block_length, dtype=torch.float32, device="cuda")
        c.f32_tile_copy(fwd, x32)
        d1 = torch.zeros(64 * c.lmax, dtype=torch.float64, device="cuda")
        d234 = torch.zeros(len(case["targets"]) * 320, dtype=torch.float64, device="cuda")
        c.pieces_2p2_f32(x32, case["gsw"], case["targets"], case["xunit"], d1, d234)
        c.check()
        ref = c.pieces_2p2(fwd, case["gsw"], case["targets"], case["xunit"], hg.FP32)
    assert np.array_equal(d1.cpu().numpy(), ref.p1)
    assert np.array_equal(d234.cpu().numpy(), ref.p234)
    assert rel(ref.p1, case["p1"]) <= TOL32_P1
    assert_rows(ref.p234, case["p234"], TOL32)


def test_bad_arguments_fail_loudly(hg):
    lat = [4, 4, 4, 4]
    fwd = dev(S.random_block(lat, 1))
    with hg.Contractor(lat) as c:
        with pytest.raises(hg.HlblError):
            c.pieces_2p2(fwd, [0, 0, 0, 4], [[0, 0, 0, 0]], 1.0)   # gsw outside [0, L)
        with pytest.raises(hg.HlblError):
            c.pieces_2p2(fwd, [0, 0, 0, 0], [[0, -1, 0, 0]], 1.0)  # target outside [0, L)
        with pytest.raises(hg.HlblError):
            c.compute_2p2(fwd, 2, [0, 0, 0, 0], [[0, 0, 0, 0]], 1.0)  # iflavor
        raw = fwd.view(torch.uint8)[8:8 + fwd.numel() * 8 - 16].view(torch.float64)
        with pytest.raises(hg.HlblError):
            c.pieces_2p2(raw, [0, 0, 0, 0], [[0, 0, 0, 0]], 1.0)   # misaligned block
