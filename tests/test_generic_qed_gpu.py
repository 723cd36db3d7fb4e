"""The generic QED paths on the GPU (hlbl_ctx_set_qed_kernel): a QED kernel
with no closed form -- the dense test weight, whose 384 entries share no
index structure -- through the coefficient stage and the FP64, CUDA-core
FP32 and tensor-core pass 2, the interface-B launchers and the 2+2 pieces,
against the reference's own code run with the same weight
(tests/golden/reference_dense_qed.json) and the oracle. The stand-in through
the generic paths must equal its closed-form paths.

Bars: FP64 1e-12 relative per pair and flavour; FP32 products 1e-4 per pair
(both flavours as one vector, support.pair_rel_err); 2+2 rows FP64 1e-12,
FP32 1e-5 against their own scale."""
import json
import os

import numpy as np
import pytest

import support as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
TOL64, TOL32 = 1e-12, 1e-4

with open(os.path.join(os.path.dirname(__file__), "golden", "reference_dense_qed.json")) as fh:
    GD = json.load(fh)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("kind", ["QED_DENSE", "QED_DENSE_KERV"])
@pytest.mark.parametrize("case", GD["kernel_sum"], ids=lambda c: c["name"])
def test_dense_weight_fp64_matches_reference(case, kind):
    import hlbl_gb300 as hg

    src, y = S.case_inputs(case)
    with hg.Contractor(case["lattice"]) as c:
        c.set_qed_kernel(getattr(hg, kind), S.DENSE_SEED)
        got = c.kernel_sum(dev(src), dev(y), case["gsx"], case["yv"], case["xunit"], hg.FP64)
    assert S.rel_err(got, case["kernel_sum"]) <= TOL64, (got, case["kernel_sum"])


@pytest.mark.parametrize("tc", [True, False], ids=["tensor_cores", "cuda_cores"])
@pytest.mark.parametrize("case", GD["kernel_sum"], ids=lambda c: c["name"])
def test_dense_weight_fp32_matches_reference(case, tc):
    import hlbl_gb300 as hg

    src, y = S.case_inputs(case)
    with hg.Contractor(case["lattice"]) as c:
        c.set_qed_kernel(hg.QED_DENSE, S.DENSE_SEED)
        c.set_tensor_cores(tc)
        got = c.kernel_sum(dev(src), dev(y), case["gsx"], case["yv"], case["xunit"], hg.FP32)
    assert S.pair_rel_err(got, case["kernel_sum"]) <= TOL32, (got, case["kernel_sum"])


def test_dense_weight_interface_b_pass2_matches_reference():
    """cu_4pt_contraction's replacement with the dense weight, from the
    oracle's pass-1 sums (the reference's pass 1 is pinned elsewhere)."""
    import hlbl_gb300 as hg

    p = GD["pass2"]
    lat = p["lattice"]
    src, y = S.random_block(lat, p["seeds"][0]), S.random_block(lat, p["seeds"][1])
    with hg.Contractor(lat) as c:
        c.set_qed_kernel(hg.QED_DENSE, S.DENSE_SEED)
        d_src, d_y = dev(src), dev(y)
        for f in (0, 1):
            dzu, dzsu = S.oracle_dz(src, y, f, p["gsx"], lat)
            g_dzu, g_dzsu = S.oracle_gammas(dzu, dzsu)
            ks = torch.zeros(1, dtype=torch.float64, device="cuda")
            c.cu_4pt_contraction(ks, dev(g_dzu), dev(g_dzsu), d_src, d_y, f, (0, 0, 0, 0), p["gsx"],
                                 p["xunit"], p["yv"], lat, lat)
            torch.cuda.synchronize()
            assert S.rel_err(ks.item(), p["kernel_sum_per_flavour"][f]) <= TOL64


@pytest.mark.parametrize("lat", [(8, 8, 8, 8), (7, 5, 6, 3)])
def test_dense_weight_batched_tensor_cores_match_oracle(lat):
    """Many 32-site tiles (and a ragged last one) through the FP32-copy path
    (tile copies, batched pass 1, tensor-core pass 2 with the generic
    epilogue), four partners in one call, against the oracle."""
    import hlbl_gb300 as hg

    xu = hg.xunit(105.658, 0.1)
    y = S.gaussian_block(lat, 17)
    srcs = [S.gaussian_block(lat, 200 + i) for i in range(4)]
    gsxs = [(i % lat[0], (i + 1) % lat[1], (2 * i) % lat[2], (3 + i) % lat[3]) for i in range(4)]
    yvs = [(1, 0, -1, 1), (0, 1, 1, -1), (2, -1, 0, 0), (-1, -1, 1, 1)]
    with S.dense_qed():
        want = [S.oracle_kernel_sum(s, y, g, v, xu, lat) for s, g, v in zip(srcs, gsxs, yvs)]
    with hg.Contractor(lat) as c:
        c.set_qed_kernel(hg.QED_DENSE, S.DENSE_SEED)
        n32 = c.f32_block_length
        d_y, d_y32 = dev(y), torch.empty(n32, dtype=torch.float32, device="cuda")
        c.f32_tile_copy(d_y, d_y32)
        d_x32s = []
        for s in srcs:
            t = torch.empty(n32, dtype=torch.float32, device="cuda")
            c.f32_tile_copy(dev(s), t)
            d_x32s.append(t)
        out = torch.zeros(8, dtype=torch.float64, device="cuda")
        c.kernel_sums_batched_f32(d_y32, d_x32s, gsxs, yvs, xu, out)
        c.check()
        got = out.cpu().numpy().reshape(4, 2)
        # the FP64 path of the same pairs
        f64 = [c.kernel_sum(dev(s), d_y, g, v, xu, hg.FP64) for s, g, v in zip(srcs, gsxs, yvs)]
    for i in range(4):
        assert S.pair_rel_err(got[i], want[i]) <= TOL32, (i, got[i], want[i])
        assert S.rel_err(f64[i], want[i]) <= TOL64, (i, f64[i], want[i])


def test_standin_generic_equals_closed_form():
    """The stand-in through the generic coefficient path against its closed
    form: FP64 within 1e-12 of the reference's golden sums, FP32 (tensor
    cores) within FP32 rounding of the closed-form FP32 path."""
    import hlbl_gb300 as hg

    for case in S.golden()["kernel_sum"]:
        src, y = S.case_inputs(case)
        args = (case["gsx"], case["yv"], case["xunit"])
        with hg.Contractor(case["lattice"]) as c:
            d_src, d_y = dev(src), dev(y)
            closed32 = c.kernel_sum(d_src, d_y, *args, hg.FP32)
            c.set_qed_kernel(hg.QED_STANDIN_GENERIC)
            g64 = c.kernel_sum(d_src, d_y, *args, hg.FP64)
            g32 = c.kernel_sum(d_src, d_y, *args, hg.FP32)
        assert S.rel_err(g64, case["kernel_sum"]) <= TOL64, case["name"]
        assert S.pair_rel_err(g32, closed32) <= 1e-5, case["name"]
        assert S.pair_rel_err(g32, case["kernel_sum"]) <= TOL32, case["name"]


@pytest.mark.parametrize("kind", ["QED_DENSE", "QED_DENSE_KERV"])
@pytest.mark.parametrize("case", GD["pieces_2p2"], ids=lambda c: c["name"])
def test_dense_weight_pieces_2p2_match_reference(case, kind):
    import hlbl_gb300 as hg

    lat = case["lattice"]
    fwd = S.random_block(lat, case["seed"])
    ref_p1 = np.asarray(case["p1"])
    with hg.Contractor(lat) as c:
        c.set_qed_kernel(getattr(hg, kind), S.DENSE_SEED)
        d = dev(fwd)
        p64 = c.pieces_2p2(d, case["gsw"], case["targets"], case["xunit"], hg.FP64)
        p32 = c.pieces_2p2(d, case["gsw"], case["targets"], case["xunit"], hg.FP32)
    ref = np.asarray(case["p234"]).reshape(-1, 5, 64)
    g64, g32 = np.asarray(p64.p234).reshape(-1, 5, 64), np.asarray(p32.p234).reshape(-1, 5, 64)
    assert rel(np.ravel(p64.p1), ref_p1) <= 1e-13
    for t in range(ref.shape[0]):
        for g in range(5):
            r = ref[t, g]
            assert rel(g64[t, g], r) <= TOL64, (t, g)
            assert rel(g32[t, g], r) <= 1e-5, (t, g)
            # the zero pattern is exact
            assert np.all(g64[t, g][r == 0] == 0) and np.all(g32[t, g][r == 0] == 0), (t, g)


def test_standin_generic_pieces_2p2_equal_closed_form():
    import hlbl_gb300 as hg

    with open(os.path.join(os.path.dirname(__file__), "golden", "reference_2p2.json")) as fh:
        cases = json.load(fh)["pieces_2p2"]
    for case in cases[:2]:
        lat = case["lattice"]
        fwd = S.random_block(lat, case["seed"])
        with hg.Contractor(lat) as c:
            d = dev(fwd)
            c.set_qed_kernel(hg.QED_STANDIN_GENERIC)
            g64 = c.pieces_2p2(d, case["gsw"], case["targets"], case["xunit"], hg.FP64)
        ref = np.asarray(case["p234"]).reshape(-1, 5, 64)
        got = np.asarray(g64.p234).reshape(-1, 5, 64)
        for t in range(ref.shape[0]):
            for g in range(5):
                assert rel(got[t, g], ref[t, g]) <= TOL64, (case["name"], t, g)


def test_generic_kind_is_capturable_after_reserve():
    """A window recorded into a CUDA graph with the dense weight replays to
    the sums of the direct calls (the coefficient buffer is reserved before
    capture, so nothing is allocated inside it)."""
    import hlbl_gb300 as hg

    lat, xu = (6, 4, 4, 4), 0.3
    y = S.gaussian_block(lat, 5)
    srcs = [S.gaussian_block(lat, 50 + i) for i in range(3)]
    gsxs = [(0, 0, 0, 0), (1, 2, 3, 0), (5, 3, 1, 2)]
    yvs = [(1, 1, 1, 1), (-1, 1, -1, 1), (2, 0, 1, -1)]
    with hg.Contractor(lat) as c:
        c.set_qed_kernel(hg.QED_DENSE, S.DENSE_SEED)
        d_y, d_srcs = dev(y), [dev(s) for s in srcs]
        direct = torch.zeros(6, dtype=torch.float64, device="cuda")
        c.kernel_sums_batched(d_y, d_srcs, gsxs, yvs, xu, direct, hg.FP64)
        c.check()
        c.reserve(3)
        replay = torch.zeros(6, dtype=torch.float64, device="cuda")
        c.graph_begin()
        c.kernel_sums_batched(d_y, d_srcs, gsxs, yvs, xu, replay, hg.FP64)
        g = c.graph_end()
        g.launch()
        torch.cuda.synchronize()
        c.check()
        g.close()
    assert np.array_equal(direct.cpu().numpy(), replay.cpu().numpy())


def test_surrogate_and_generic_kind_exclude_each_other():
    import hlbl_gb300 as hg

    with hg.Contractor((4, 4, 4, 4)) as c:
        c.set_qed_kernel(hg.QED_DENSE, 1)
        with pytest.raises(hg.HlblError):
            c.set_qed_kernel(7)
        c.set_qed_kernel(hg.QED_STANDIN)


def test_dense_weight_two_rank_site_split():
    """The reference's domain decomposition with the dense weight: two ranks
    along t, the pass-1 sums of both added before pass 2 (the all-reduce),
    each rank's pass 2 on its own sites with the generic coefficients; the
    ranks' total equals the oracle's one-rank sums of the whole lattice."""
    import hlbl_gb300 as hg

    glob, loc = (8, 4, 4, 6), (4, 4, 4, 6)
    gsx, yv, xu = (5, 1, 3, 2), (-2, 1, 0, 3), hg.xunit(105.658, 0.1)
    seeds = (611, 612)
    whole = [S.random_block(glob, s) for s in seeds]
    with S.dense_qed():
        want = S.oracle_kernel_sum(whole[0], whole[1], gsx, yv, xu, glob)
    V, Vl = S.volume(glob), S.volume(loc)
    # t is the slowest site index: rank r holds sites [r Vl, (r + 1) Vl)
    blocks = {r: [dev(b.reshape(2, 12, V, 24)[:, :, r * Vl:(r + 1) * Vl, :]) for b in whole] for r in (0, 1)}
    with hg.Contractor(glob, loc, (0, 0, 0, 0)) as c:
        c.set_qed_kernel(hg.QED_DENSE, S.DENSE_SEED)
        total = np.zeros(2)
        for f in (0, 1):
            d_dzu = torch.zeros(1728, dtype=torch.float64, device="cuda")
            d_dzsu = torch.zeros(1152, dtype=torch.float64, device="cuda")
            for r in (0, 1):
                c.cu_dzu_dzsu(d_dzu, d_dzsu, blocks[r][0], blocks[r][1], f, (r, 0, 0, 0), gsx, glob, loc)
            d_gu = torch.zeros(6912, dtype=torch.float64, device="cuda")
            d_gs = torch.zeros(4608, dtype=torch.float64, device="cuda")
            c.insert_gammas(d_dzu, d_dzsu, d_gu, d_gs)
            for r in (0, 1):
                d_ks = torch.zeros(1, dtype=torch.float64, device="cuda")
                c.cu_4pt_contraction(d_ks, d_gu, d_gs, blocks[r][0], blocks[r][1], f, (r, 0, 0, 0),
                                     gsx, xu, yv, glob, loc)
                torch.cuda.synchronize()
                total[f] += d_ks.item()
    assert S.rel_err(total, want) <= TOL64, (total, want)
