"""Parity of the CUDA path with the oracle (and the reference's own outputs in
tests/golden), through the C ABI. Needs a GPU.

Tolerances: FP64 path 1e-12 relative per pair and flavour; FP32 path 1e-4
relative per pair, the pair's two flavour sums taken as one vector
(support.pair_rel_err), so a flavour that nearly cancels is measured
against the pair's scale."""
import numpy as np
import pytest

import support as S

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
G = S.golden()
TOL64 = 1e-12
TOL32 = 1e-4


def dev(a: np.ndarray):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def hg():
    import hlbl_gb300

    return hlbl_gb300


@pytest.mark.parametrize("case", G["kernel_sum"], ids=lambda c: c["name"])
def test_kernel_sum_fp64_matches_reference_and_oracle(hg, case):
    src, y = S.case_inputs(case)
    ref = np.array(case["kernel_sum"])
    orc = S.oracle_kernel_sum(src, y, case["gsx"], case["yv"], case["xunit"], case["lattice"])
    with hg.Contractor(case["lattice"]) as c:
        got = c.kernel_sum(dev(src), dev(y), case["gsx"], case["yv"], case["xunit"], hg.FP64)
    assert S.rel_err(got, ref) <= TOL64
    assert S.rel_err(got, orc) <= TOL64


@pytest.mark.parametrize("case", G["kernel_sum"], ids=lambda c: c["name"])
def test_kernel_sum_fp32_within_1e4(hg, case):
    src, y = S.case_inputs(case)
    ref = np.array(case["kernel_sum"])
    with hg.Contractor(case["lattice"]) as c:
        got = c.kernel_sum(dev(src), dev(y), case["gsx"], case["yv"], case["xunit"], hg.FP32)
    assert S.pair_rel_err(got, ref) <= TOL32


def _pairs_config1():
    from hlbl_gb300 import schedule

    st = schedule.build_schedule((1, 1, 1, 1), 1, 1)
    return schedule.all_pairs(st)


def test_config1_all_80_pairs_fp64(hg):
    """8^3 x 16, Gaussian blocks, stride 1, h = (1,1,1,1), K = 1: 80 pairs x 2
    flavours, every one against the oracle at 1e-12. Blocks are made on the
    host and copied in (host cache)."""
    from hlbl_gb300 import schedule

    lat = (16, 8, 8, 8)
    xu = hg.xunit(105.658, 0.1)
    pairs = _pairs_config1()
    assert len(pairs) == 80
    blocks = {}

    def block(p):
        site = schedule.mod_pos(p, lat)
        if site not in blocks:
            blocks[site] = S.gaussian_block(lat, S.source_seed(1234, site))
        return blocks[site]

    worst = 0.0
    with hg.Contractor(lat) as c:
        for older, newer, _ in pairs:
            gx = schedule.mod_pos(older, lat)
            yv = schedule.site_map_diff(newer, older, lat)
            src, y = block(older), block(newer)
            got = c.kernel_sum(dev(src), dev(y), gx, yv, xu, hg.FP64)
            orc = S.oracle_kernel_sum(src, y, gx, yv, xu, lat)
            worst = max(worst, S.rel_err(got, orc))
    assert worst <= TOL64, worst


def test_interface_b_launchers(hg):
    """cu_dzu_dzsu / gamma insertion / cu_4pt_contraction, one flavour at a
    time, each against the oracle."""
    lat, gsx, yv, xu = (4, 4, 4, 6), (1, 3, 0, 5), (1, -1, 2, -3), 0.6
    src, y = S.random_block(lat, 31), S.random_block(lat, 32)
    d_src, d_y = dev(src), dev(y)
    z = (0, 0, 0, 0)
    with hg.Contractor(lat) as c:
        for f in (0, 1):
            dzu_o, dzsu_o = S.oracle_dz(src, y, f, gsx, lat)
            g_o = S.oracle_gammas(dzu_o, dzsu_o)
            ks_o = S.oracle_4pt(g_o[0], g_o[1], src, y, f, gsx, xu, yv, lat)
            d_dzu = torch.zeros(1728, dtype=torch.float64, device="cuda")
            d_dzsu = torch.zeros(1152, dtype=torch.float64, device="cuda")
            c.cu_dzu_dzsu(d_dzu, d_dzsu, d_src, d_y, f, z, gsx, lat, lat)
            d_gu = torch.zeros(6912, dtype=torch.float64, device="cuda")
            d_gs = torch.zeros(4608, dtype=torch.float64, device="cuda")
            c.insert_gammas(d_dzu, d_dzsu, d_gu, d_gs)
            d_ks = torch.zeros(1, dtype=torch.float64, device="cuda")
            c.cu_4pt_contraction(d_ks, d_gu, d_gs, d_src, d_y, f, z, gsx, xu, yv, lat, lat)
            torch.cuda.synchronize()
            got = np.concatenate([d_dzu.cpu().numpy(), d_dzsu.cpu().numpy()])
            ref = np.concatenate([dzu_o, dzsu_o])
            assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
            gg = np.concatenate([d_gu.cpu().numpy(), d_gs.cpu().numpy()])
            gr = np.concatenate(g_o)
            assert np.max(np.abs(gg - gr)) <= 1e-12 * np.max(np.abs(gr))
            assert abs(d_ks.item() - ks_o) <= TOL64 * abs(ks_o)


def test_two_rank_site_split(hg):
    """The reference's domain decomposition: two ranks along t, each with its
    own sub-block and process-grid coordinates, the pass-1 sums added between
    the passes (the all-reduce) -- the partials and the total match the
    reference's own split."""
    sp = G["two_rank_split"]
    glob, loc = sp["global"], sp["local"]
    blocks = {r: (dev(S.random_block(loc, sp["seeds"][0], [r, 0, 0, 0])),
                  dev(S.random_block(loc, sp["seeds"][1], [r, 0, 0, 0]))) for r in (0, 1)}
    with hg.Contractor(glob, loc, (0, 0, 0, 0)) as c:
        total = np.zeros(2)
        for f in (0, 1):
            d_dzu = torch.zeros(1728, dtype=torch.float64, device="cuda")
            d_dzsu = torch.zeros(1152, dtype=torch.float64, device="cuda")
            for r in (0, 1):
                c.cu_dzu_dzsu(d_dzu, d_dzsu, blocks[r][0], blocks[r][1], f, (r, 0, 0, 0),
                              sp["gsx"], glob, loc)
            d_gu = torch.zeros(6912, dtype=torch.float64, device="cuda")
            d_gs = torch.zeros(4608, dtype=torch.float64, device="cuda")
            c.insert_gammas(d_dzu, d_dzsu, d_gu, d_gs)
            for r in (0, 1):
                d_ks = torch.zeros(1, dtype=torch.float64, device="cuda")
                c.cu_4pt_contraction(d_ks, d_gu, d_gs, blocks[r][0], blocks[r][1], f, (r, 0, 0, 0),
                                     sp["gsx"], sp["xunit"], sp["yv"], glob, loc)
                torch.cuda.synchronize()
                want = sp["ranks"][r]["kernel_sum_partial"][f]
                assert abs(d_ks.item() - want) <= TOL64 * abs(want)
                total[f] += d_ks.item()
    assert S.rel_err(total, sp["single_rank_kernel_sum"]) <= TOL64


def test_device_fixture_generators(hg):
    lat = (4, 4, 2, 6)
    with hg.Contractor(lat) as c:
        d = torch.empty(c.block_length, dtype=torch.float64, device="cuda")
        c.fill_random_block(d, 77)
        torch.cuda.synchronize()
        assert np.array_equal(d.cpu().numpy(), S.random_block(lat, 77))
        c.fill_gaussian_block(d, 78)
        torch.cuda.synchronize()
        g = d.cpu().numpy()
        h = S.gaussian_block(lat, 78)
        # bit-identical: the fixture's log and sincos are built from exactly
        # rounded operations that neither compiler fuses (hlbl_gb300_rng.h)
        assert np.array_equal(g, h)
        assert abs(np.mean(g)) < 0.1 and abs(np.mean(g * g) - 0.5) < 0.1


def test_deterministic_and_exact_properties(hg):
    """Fixed-order reductions: repeated runs are bit-identical. The sum is
    bilinear in (src, y), so doubling src quadruples it exactly; swapping
    the flavours of both blocks swaps the two results."""
    lat, gsx, yv, xu = (6, 4, 4, 4), (2, 1, 0, 3), (1, 1, -1, 1), 0.3
    src, y = S.gaussian_block(lat, 5), S.gaussian_block(lat, 6)
    V = S.volume(lat)
    with hg.Contractor(lat) as c:
        for prec in (hg.FP64, hg.FP32):
            a = c.kernel_sum(dev(src), dev(y), gsx, yv, xu, prec)
            b = c.kernel_sum(dev(src), dev(y), gsx, yv, xu, prec)
            assert a == b
            d = c.kernel_sum(dev(2.0 * src), dev(y), gsx, yv, xu, prec)
            assert d == (4.0 * a[0], 4.0 * a[1])
            sw = lambda blk: np.ascontiguousarray(blk.reshape(2, 12 * V * 24)[::-1])
            e = c.kernel_sum(dev(sw(src)), dev(sw(y)), gsx, yv, xu, prec)
            assert e == (a[1], a[0])


def test_tail_tiles_and_tiny_lattices(hg):
    """Volumes that are not a multiple of any tile size, and 1^4 / 2^4."""
    for lat in ((1, 1, 1, 1), (2, 2, 2, 2), (3, 5, 1, 7), (7, 3, 3, 3)):
        src, y = S.random_block(lat, 8), S.random_block(lat, 9)
        gsx, yv, xu = (0, 0, 0, 0), (1, 1, 1, 1), 0.8
        orc = S.oracle_kernel_sum(src, y, gsx, yv, xu, lat)
        with hg.Contractor(lat) as c:
            got = c.kernel_sum(dev(src), dev(y), gsx, yv, xu, hg.FP64)
        assert S.rel_err(got, orc) <= TOL64, lat


def test_errors_are_reported(hg):
    lat = (2, 2, 2, 2)
    with hg.Contractor(lat) as c:
        d = torch.zeros(c.block_length + 2, dtype=torch.float64, device="cuda")
        with pytest.raises(hg.HlblError) as ei:
            c.kernel_sum(d.data_ptr() + 8, d, (0, 0, 0, 0), (1, 1, 1, 1), 1.0)
        assert ei.value.code == 1 and "aligned" in str(ei.value)
        with pytest.raises(hg.HlblError) as ei:
            c.kernel_sum(d, d, (0, 0, 2, 0), (1, 1, 1, 1), 1.0)
        assert ei.value.code == 1 and "gsx" in str(ei.value)
        with pytest.raises(hg.HlblError):
            c.kernel_sum(d, d, (0, 0, 0, 0), (1, 1, 1, 1), 1.0, precision=7)
    with pytest.raises(hg.HlblError):
        hg.Contractor((4, 4, 4, 4), (4, 4, 4, 3), (0, 0, 0, 1))  # 2*3 > 4
    assert hg.Contractor(lat).reserve_kernel_memory() >= 0


def test_reserve_kernel_memory_reserves_once():
    """Contractor::reserve_kernel_memory (contract.cpp:158-197) warm-launches
    the kernels so that whatever the first launches take is taken before
    free memory is measured. The library's kernels keep no per-thread stack
    (the reference's 4-point kernel reserves ~27 KB per thread slot, 3.7 GB
    on this GPU), so: the first call takes well under the reference's
    figure, a second call takes nothing more, and contractions of every
    precision afterwards leave free device memory where it was."""
    import hlbl_gb300 as hg

    lat = (2, 2, 2, 2)
    mib = 1 << 20
    with hg.Contractor(lat) as c:
        first = c.reserve_kernel_memory()
        second = c.reserve_kernel_memory()
        assert first < 512 * mib, first
        assert second <= 2 * mib, second  # the allocation granularity at most
        d = dev(S.random_block(lat, 3))
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        for prec in (hg.FP64, hg.FP32):
            c.kernel_sum(d, d, (0, 0, 0, 0), (1, 1, 1, 1), 1.0, prec)
        torch.cuda.synchronize()
        assert abs(torch.cuda.mem_get_info()[0] - free0) <= 2 * mib
