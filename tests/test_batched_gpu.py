"""The batched path (hlbl_kernel_sums_batched): all pairs a new source closes
in launches that share its block, against the oracle and the per-pair API."""
import numpy as np
import pytest

import support as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _source_batch(lat, stride=1, h=(1, 1, 1, 1), steps=1, which=3):
    """The new source `which` of window 1 and its partners, with blocks."""
    from hlbl_gb300 import schedule

    st = schedule.build_schedule(h, stride, steps)
    srcs = [s for s in st[1].sources if s.partners]
    src = srcs[which]
    y_site = schedule.mod_pos(src.position, lat)
    pairs = [(schedule.mod_pos(q, lat), schedule.site_map_diff(src.position, q, lat)) for q in src.partners]
    return y_site, pairs


@pytest.mark.parametrize("group", [0, 1, 3])
def test_batched_fp64_matches_oracle_and_single(group):
    import hlbl_gb300 as hg

    lat, xu = (8, 6, 6, 6), 0.3
    y_site, pairs = _source_batch(lat)
    assert len(pairs) >= 4
    y_h = S.random_block(lat, S.source_seed(9, y_site))
    xs = [S.random_block(lat, S.source_seed(9, g)) for g, _ in pairs]
    d_y = torch.from_numpy(y_h).cuda()
    d_x = [torch.from_numpy(a).cuda() for a in xs]
    out = torch.zeros((len(pairs), 2), dtype=torch.float64, device="cuda")
    with hg.Contractor(lat) as c:
        c.set_batch_group(group)
        c.kernel_sums_batched(d_y, d_x, [g for g, _ in pairs], [v for _, v in pairs], xu, out, hg.FP64)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        for i, (g, v) in enumerate(pairs):
            single = c.kernel_sum(d_x[i], d_y, g, v, xu, hg.FP64)
            orc = S.oracle_kernel_sum(xs[i], y_h, g, v, xu, lat)
            assert S.rel_err(got[i], orc) <= 1e-12
            assert S.rel_err(got[i], single) <= 1e-12


def test_batched_fp32_and_more_than_sixteen_pairs():
    """n > 16 runs in chunks; FP32 within 1e-4 of the oracle (per pair, the
    two flavours as one vector); n = 0 is a no-op."""
    import hlbl_gb300 as hg

    lat, xu = (6, 4, 4, 4), 0.5
    rng = np.random.default_rng(0)
    y_h = S.random_block(lat, 1)
    xs = [S.random_block(lat, 100 + i) for i in range(3)]
    n = 19
    gsx = [tuple(int(v) for v in rng.integers(0, lat)) for _ in range(n)]
    yv = [tuple(int(v) for v in rng.integers(-3, 4, 4)) for _ in range(n)]
    d_y = torch.from_numpy(y_h).cuda()
    d_x = [torch.from_numpy(a).cuda() for a in xs]
    srcs = [d_x[i % 3] for i in range(n)]
    out = torch.zeros((n, 2), dtype=torch.float64, device="cuda")
    with hg.Contractor(lat) as c:
        c.kernel_sums_batched(d_y, srcs, gsx, yv, xu, out, hg.FP32)
        c.kernel_sums_batched(d_y, [], [], [], xu, out, hg.FP32)
        torch.cuda.synchronize()
    got = out.cpu().numpy()
    for i in range(n):
        orc = S.oracle_kernel_sum(xs[i % 3], y_h, gsx[i], yv[i], xu, lat)
        assert S.pair_rel_err(got[i], orc) <= 1e-4, i


def test_window_graph_staging_and_autotune():
    """A window recorded as one CUDA graph and replayed gives the same sums as
    the direct calls; a block staged from pinned host memory on the side
    stream is waited for; the autotuner's choice stays within 1e-4."""
    import hlbl_gb300 as hg
    from hlbl_gb300 import schedule

    lat, xu = (8, 4, 4, 6), 0.4
    st = schedule.build_schedule((1, 1, 1, 1), 1, 1)
    sources = [s for s in st[1].sources if s.partners][:3]
    blocks = {}

    def blk(p):
        site = schedule.mod_pos(p, lat)
        if site not in blocks:
            blocks[site] = torch.from_numpy(S.random_block(lat, S.source_seed(5, site))).cuda()
        return blocks[site]

    calls = []
    for s in sources:
        qs = s.partners
        calls.append((blk(s.position), [blk(q) for q in qs], [schedule.mod_pos(q, lat) for q in qs],
                      [schedule.site_map_diff(s.position, q, lat) for q in qs]))
    n_tot = sum(len(c[1]) for c in calls)
    direct = torch.zeros((n_tot, 2), dtype=torch.float64, device="cuda")
    graphed = torch.zeros_like(direct)
    with hg.Contractor(lat) as c:
        k = 0
        for y, xs, g, v in calls:
            c.kernel_sums_batched(y, xs, g, v, xu, direct[k:k + len(xs)], hg.FP32)
            k += len(xs)
        c.graph_begin()
        k = 0
        for y, xs, g, v in calls:
            c.kernel_sums_batched(y, xs, g, v, xu, graphed[k:k + len(xs)], hg.FP32)
            k += len(xs)
        graph = c.graph_end()
        torch.cuda.synchronize()
        assert torch.count_nonzero(graphed).item() == 0  # recorded, not run
        graph.launch()
        torch.cuda.synchronize()
        assert torch.equal(graphed, direct)
        graph.close()

        # staging: copy the first source's block from pinned memory into a
        # fresh device buffer on the side stream, then contract from it
        y0, xs0, g0, v0 = calls[0]
        pinned = y0.cpu().pin_memory()
        fresh = torch.zeros_like(y0)
        staged = torch.zeros((len(xs0), 2), dtype=torch.float64, device="cuda")
        c.stage_async(fresh, pinned, pinned.numel() * 8)
        c.kernel_sums_batched(fresh, xs0, g0, v0, xu, staged, hg.FP32)
        torch.cuda.synchronize()
        assert torch.equal(staged, direct[:len(xs0)])

        tuned = torch.zeros_like(staged)
        best = c.autotune(y0, xs0, g0, v0, xu, tuned)
        assert best["batch_group"] in (1, 2, 4, 8, 16) and best["ms"] > 0
        c.kernel_sums_batched(y0, xs0, g0, v0, xu, tuned, hg.FP32)
        torch.cuda.synchronize()
        t = tuned.cpu().numpy()
        d = direct[:len(xs0)].cpu().numpy()
        for i in range(len(t)):
            assert S.pair_rel_err(t[i], d[i]) <= 1e-4
