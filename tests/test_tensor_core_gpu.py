"""The tensor-core pass 2 (tcgen05, 3xTF32 products) against the oracle and
against the CUDA-core FP32 pass 2, through the C ABI: tail tiles (volumes
that are not a multiple of the 32-site tile), tiny lattices, batches, and
repeatability. Needs a GPU.

Tolerance: 1e-4 relative per pair, the pair's two flavour sums as one
vector (support.pair_rel_err), as for every FP32-product path."""
import numpy as np
import pytest

import support as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
TOL32 = 1e-4


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("lat", [(1, 1, 1, 1), (2, 2, 2, 2), (3, 5, 1, 7), (7, 3, 3, 3), (8, 4, 4, 4),
                                 (16, 8, 8, 8)])
def test_tensor_core_pass2_matches_oracle(lat):
    import hlbl_gb300 as hg

    src, y = S.gaussian_block(lat, 41), S.gaussian_block(lat, 42)
    gsx = tuple(min(1, L - 1) for L in lat)
    yv, xu = (1, -1, 1, 0), hg.xunit(105.658, 0.1)
    orc = S.oracle_kernel_sum(src, y, gsx, yv, xu, lat)
    with hg.Contractor(lat) as c:
        d_src, d_y = dev(src), dev(y)
        c.set_tensor_cores(True)
        tc = c.kernel_sum(d_src, d_y, gsx, yv, xu, hg.FP32)
        tc2 = c.kernel_sum(d_src, d_y, gsx, yv, xu, hg.FP32)
        c.set_tensor_cores(False)
        cc = c.kernel_sum(d_src, d_y, gsx, yv, xu, hg.FP32)
    assert tc == tc2  # fixed-order reductions
    assert S.pair_rel_err(tc, orc) <= TOL32, (tc, orc)
    assert S.pair_rel_err(cc, orc) <= TOL32, (cc, orc)


def test_tensor_core_batched_equals_per_pair():
    """Five partners of one new block in one launch against one launch per
    pair: the CTA partition of the sites differs, and with it the rounding of
    pass 1's FP32 tile sums (flushed to FP64 every 32 sites of a CTA), so
    the two agree to FP32 accuracy (1e-5 at the pair's scale); each is
    within 1e-4 of the oracle."""
    import hlbl_gb300 as hg

    lat = (6, 4, 4, 4)
    xu = hg.xunit(105.658, 0.1)
    y = S.gaussian_block(lat, 7)
    srcs = [S.gaussian_block(lat, 100 + i) for i in range(5)]
    gsxs = [(i % 6, (i + 1) % 4, (2 * i) % 4, 3 - i % 4) for i in range(5)]
    yvs = [(1, 0, -1, 1), (0, 1, 1, -1), (2, -1, 0, 0), (-1, -1, 1, 1), (1, 2, 0, -2)]
    with hg.Contractor(lat) as c:
        c.set_tensor_cores(True)
        d_y = dev(y)
        d_srcs = [dev(s) for s in srcs]
        out = torch.zeros((5, 2), dtype=torch.float64, device="cuda")
        c.kernel_sums_batched(d_y, d_srcs, gsxs, yvs, xu, out, hg.FP32)
        c.check()
        got = out.cpu().numpy()
        for i in range(5):
            one = c.kernel_sum(d_srcs[i], d_y, gsxs[i], yvs[i], xu, hg.FP32)
            assert S.pair_rel_err(got[i], one) <= 1e-5
            orc = S.oracle_kernel_sum(srcs[i], y, gsxs[i], yvs[i], xu, lat)
            assert S.pair_rel_err(got[i], orc) <= TOL32


def test_fp32_quadrature_weight_matches_fp64_weight():
    """The mixed path's exact QED weight in FP32 (FP64 within r64 of the
    origin) against the FP64 weight everywhere: the same kernel sums to FP32
    accuracy (every quadrature term is positive). With r64 larger than the
    lattice, every row takes the FP64 branch and the sums are identical."""
    import hlbl_gb300 as hg

    lat = (8, 6, 6, 6)
    xu = hg.xunit(105.658, 0.1)
    src, y = S.gaussian_block(lat, 51), S.gaussian_block(lat, 52)
    gsx, yv = (2, 1, 0, 5), (2, -2, 1, 0)
    orc = S.oracle_kernel_sum(src, y, gsx, yv, xu, lat)
    with hg.Contractor(lat) as c:
        d_src, d_y = dev(src), dev(y)
        c.set_qed_fp32(False)
        w64 = c.kernel_sum(d_src, d_y, gsx, yv, xu, hg.FP32)
        c.set_qed_fp32(True, 0.1)
        w32 = c.kernel_sum(d_src, d_y, gsx, yv, xu, hg.FP32)
        c.set_qed_fp32(True, 1e3)
        w32_all64 = c.kernel_sum(d_src, d_y, gsx, yv, xu, hg.FP32)
    assert w32_all64 == w64
    assert S.pair_rel_err(w32, w64) <= 1e-6
    assert S.pair_rel_err(w32, orc) <= TOL32


def test_f32_tile_copy_rounds_like_ieee_and_lays_out_tiles():
    """The FP64 -> FP32 conversion of pass 1 (integer pipe, round to nearest
    even) against numpy's IEEE conversion, bit for bit, on Gaussian values
    and planted edge cases (ties, zeros, subnormals, overflow, infinities);
    and the tile layout [f][ia][tile][half][6][16][4] with a ragged last tile."""
    import hlbl_gb300 as hg

    lat = (3, 5, 1, 7)  # V = 105: four tiles of 32, the last one ragged
    V = S.volume(lat)
    blk = S.gaussian_block(lat, 61)
    edge = np.array([0.0, -0.0, 1.0 + 2.0 ** -24, 1.0 + 3 * 2.0 ** -24, -(1.0 + 2.0 ** -24), 1e-40, -3e-39,
                     1e-50, 3.5e38, -3.5e38, 3.4028235677973366e38, np.inf, -np.inf, 1.17549435e-38,
                     2.0 ** -126 * (1 - 2.0 ** -25), 65504.0 + 2.0 ** -13])
    blk[:edge.size] = edge
    blk[1000:1000 + edge.size] = edge * 3.0
    nt = (V + 31) // 32
    with hg.Contractor(lat) as c:
        assert c.f32_block_length == 2 * 12 * nt * 768 + 32  # the tiles, then the trailer
        out = torch.full((c.f32_block_length,), float("nan"), dtype=torch.float32, device="cuda")
        c.f32_tile_copy(dev(blk), out)
        c.check()
    full = out.cpu().numpy()
    got = full[:2 * 12 * nt * 768].reshape(2 * 12, nt, 2, 6, 16, 4)
    want = blk.astype(np.float32).reshape(2 * 12, V, 6, 4)
    for site in range(V):
        a = got[:, site // 32, (site % 32) // 16, :, site % 16, :]
        assert np.array_equal(a.view(np.uint32), want[:, site].view(np.uint32)), site
    # the trailer: the largest magnitude per flavour (here infinities were planted)
    trailer = full[2 * 12 * nt * 768:]
    for f in range(2):
        assert trailer[f] == np.max(np.abs(want[12 * f:12 * f + 12])), (f, trailer[f])


@pytest.mark.parametrize("fp16", [False, True])
@pytest.mark.parametrize("lat", [(6, 4, 4, 4), (3, 5, 1, 7)])
def test_f32_copy_path_matches_oracle_and_fp64_input_path(lat, fp16):
    """hlbl_kernel_sums_batched_f32 on FP32 tile copies made once per block
    (hlbl_f32_tile_copy), with TF32 or FP16 operands in pass 2: within 1e-4
    of the oracle and within FP32 accuracy (1e-5 at the pair's scale; pass 1's
    tiling differs) of the same batch on the FP64 blocks; the autotuner's
    choice stays within the same bars."""
    import hlbl_gb300 as hg

    xu = hg.xunit(105.658, 0.1)
    y = S.gaussian_block(lat, 71)
    srcs = [S.gaussian_block(lat, 80 + i) for i in range(3)]
    gsxs = [tuple((i + r) % L for r, L in enumerate(lat)) for i in range(3)]
    yvs = [(1, 0, -1, 1), (0, 1, 1, -1), (2, -1, 0, 0)]
    with hg.Contractor(lat) as c:
        c.set_tc_fp16(fp16)
        d_y, d_srcs = dev(y), [dev(s) for s in srcs]
        n32 = c.f32_block_length
        y32 = torch.empty(n32, dtype=torch.float32, device="cuda")
        x32 = [torch.empty(n32, dtype=torch.float32, device="cuda") for _ in srcs]
        c.f32_tile_copy(d_y, y32)
        for d, o in zip(d_srcs, x32):
            c.f32_tile_copy(d, o)
        out = torch.zeros((3, 2), dtype=torch.float64, device="cuda")
        c.kernel_sums_batched_f32(y32, x32, gsxs, yvs, xu, out)
        ref = torch.zeros_like(out)
        c.kernel_sums_batched(d_y, d_srcs, gsxs, yvs, xu, ref, hg.FP32)
        # every pass-1 variant and pair grouping gives the same sums (the
        # per-thread order of the FP32 sums is the same; CTA counts differ)
        per_var = []
        for v in range(4):
            for g in (1, 3):
                c.set_p1f32_variant(v, g)
                o = torch.zeros_like(out)
                c.kernel_sums_batched_f32(y32, x32, gsxs, yvs, xu, o)
                per_var.append(o.cpu().numpy())
        tuned = torch.zeros_like(out)
        best = c.autotune_f32(y32, x32, gsxs, yvs, xu, tuned)
        c.kernel_sums_batched_f32(y32, x32, gsxs, yvs, xu, tuned)
        c.check()
        got, r64, tun = out.cpu().numpy(), ref.cpu().numpy(), tuned.cpu().numpy()
    assert best["batch_group"] in (1, 2, 4, 8, 16)
    for o in per_var:
        for i in range(3):
            assert S.pair_rel_err(o[i], got[i]) <= 1e-6
    for i in range(3):
        orc = S.oracle_kernel_sum(srcs[i], y, gsxs[i], yvs[i], xu, lat)
        assert S.pair_rel_err(got[i], orc) <= TOL32
        assert S.pair_rel_err(tun[i], orc) <= TOL32
        assert S.pair_rel_err(got[i], r64[i]) <= 1e-5


@pytest.mark.parametrize("fp16", [False, True])
@pytest.mark.parametrize("lat", [(8, 8, 8, 24), (4, 6, 5, 21), (5, 3, 7, 40)])
def test_f32_copy_pass1_over_many_tiles(lat, fp16):
    """Every pass-1 variant of the FP32-copy path on lattices with several
    16-site tiles per CTA and runs along z that cross tiles (LZ = 24, 21, 40;
    odd extents, whose zero-half point is not L/2 of an even L), pass 2 with
    TF32 or FP16 operands: each pair against the oracle (1e-4) and against
    the FP64 path at FP32 accuracy (1e-5 at the pair's scale), repeatable bit
    for bit."""
    import hlbl_gb300 as hg

    xu = hg.xunit(105.658, 0.1)
    y = S.gaussian_block(lat, 171)
    srcs = [S.gaussian_block(lat, 180 + i) for i in range(2)]
    gsxs = [(1, 2, 3, 5), tuple(L - 1 for L in lat)]
    yvs = [(1, -1, 2, -3), (0, 2, -1, 7)]
    with hg.Contractor(lat) as c:
        c.set_tc_fp16(fp16)
        d_y, d_srcs = dev(y), [dev(s) for s in srcs]
        n32 = c.f32_block_length
        y32 = torch.empty(n32, dtype=torch.float32, device="cuda")
        x32 = [torch.empty(n32, dtype=torch.float32, device="cuda") for _ in srcs]
        c.f32_tile_copy(d_y, y32)
        for d, o in zip(d_srcs, x32):
            c.f32_tile_copy(d, o)
        res = {}
        for v in range(4):
            c.set_p1f32_variant(v, 1)
            o = torch.zeros((2, 2), dtype=torch.float64, device="cuda")
            c.kernel_sums_batched_f32(y32, x32, gsxs, yvs, xu, o)
            o2 = torch.zeros_like(o)
            c.kernel_sums_batched_f32(y32, x32, gsxs, yvs, xu, o2)
            assert torch.equal(o, o2)  # fixed order: repeatable bit for bit
            res[v] = o.cpu().numpy()
        r64 = torch.zeros((2, 2), dtype=torch.float64, device="cuda")
        c.kernel_sums_batched(d_y, d_srcs, gsxs, yvs, xu, r64, hg.FP64)
        c.check()
        r64 = r64.cpu().numpy()
    for i in range(2):
        orc = S.oracle_kernel_sum(srcs[i], y, gsxs[i], yvs[i], xu, lat)
        assert S.pair_rel_err(r64[i], orc) <= 1e-12
        for v in range(4):
            assert S.pair_rel_err(res[v][i], orc) <= TOL32
            assert S.pair_rel_err(res[v][i], r64[i]) <= 1e-5, (v, res[v][i], r64[i])


def test_fp16_operands_over_scales():
    """FP16 operands on blocks of very different magnitudes (1e-12, 1, 1e9 and
    a block whose flavours differ by 1e6): the power-of-two scales keep every
    pair within FP32 accuracy of the TF32 operands (1e-5 at the pair's scale)
    and within 1e-4 of the oracle."""
    import hlbl_gb300 as hg

    lat = (6, 4, 4, 8)
    xu = hg.xunit(105.658, 0.1)
    base_y = S.gaussian_block(lat, 301)
    base_x = S.gaussian_block(lat, 302)
    half = base_y.size // 2
    cases = [(1e-12, 1.0), (1.0, 1e9), (1e-3, 1e3)]
    with hg.Contractor(lat) as c:
        n32 = c.f32_block_length
        for sy, sx in cases:
            y = base_y * sy
            x = base_x * sx
            x[half:] *= 1e-6  # flavour 1 of the partner far smaller than flavour 0
            y32 = torch.empty(n32, dtype=torch.float32, device="cuda")
            x32 = torch.empty(n32, dtype=torch.float32, device="cuda")
            c.f32_tile_copy(dev(y), y32)
            c.f32_tile_copy(dev(x), x32)
            res = {}
            for fp16 in (False, True):
                c.set_tc_fp16(fp16)
                o = torch.zeros((1, 2), dtype=torch.float64, device="cuda")
                c.kernel_sums_batched_f32(y32, [x32], [(1, 2, 3, 4)], [(2, -1, 1, 3)], xu, o)
                c.check()
                res[fp16] = o.cpu().numpy()[0]
            orc = S.oracle_kernel_sum(x, y, (1, 2, 3, 4), (2, -1, 1, 3), xu, lat)
            assert S.pair_rel_err(res[True], orc) <= TOL32, (sy, sx, res[True], orc)
            assert S.pair_rel_err(res[True], res[False]) <= 1e-5, (sy, sx, res)
