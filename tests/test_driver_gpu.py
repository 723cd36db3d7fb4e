"""The driver loop on random fields, as the reference's test_driver_random
(sanity_check/test_driver_random.cpp:133-234): pair count and cache peak
from the schedule simulation, device vs host cache giving the same sums, a
few pairs recomputed directly, 2+2 at first solves against direct calls --
plus the batched loop, with and without a CUDA graph per window, against the
per-pair loop."""
import numpy as np
import pytest

import support as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_driver_device_host_batched_graphs():
    import hlbl_gb300 as hg
    from hlbl_gb300 import schedule
    from hlbl_gb300.cache import PropagatorCache, TorchBuffers
    from hlbl_gb300.driver import run_chain

    lat = (6, 6, 6, 6)
    xu = hg.xunit(105.6583745, 0.07957)
    steps = schedule.build_schedule((1, 1, 1, 1), 1, 2)
    n_prop, n_pairs, peak = schedule.simulate(steps)
    with hg.Contractor(lat) as c:
        def provider(site, dest):
            c.fill_random_block(dest, hg.Contractor.source_seed(7, site))

        solved = [tuple(schedule.mod_pos(s.position, lat)) for st_ in steps for s in st_.sources]
        want_2p2 = {solved[1]: [(0, 0, 0, 0), (3, 3, 3, 3)], solved[7]: [(1, 2, 3, 4)]}
        runs, r22 = {}, {}
        for name, res, batched, graphs in (("device", "device", False, False),
                                           ("host", "host", False, False),
                                           ("batched", "device", True, False),
                                           ("graphs", "device", True, True)):
            cache = PropagatorCache(res, c.block_length, TorchBuffers(c))
            r22[name] = []
            out = run_chain(steps, lat, xu, provider, c, cache, precision=hg.FP64, batched=batched,
                            graphs=graphs,
                            out_factory=lambda n: torch.zeros((n, 2), dtype=torch.float64, device="cuda"),
                            sources_2p2=want_2p2, results_2p2=r22[name])
            runs[name] = out
        # 2+2 at the first solves (driver.cpp:58-96) equal direct calls on the
        # same fields, in every mode (host mode: from the scratch block)
        for name, rows in r22.items():
            assert [r.w for r in rows] == [solved[1], solved[7]], name
            assert runs[name][1].pieces_2p2 == 2 and runs[name][1].targets_2p2 == 3
            for r in rows:
                d = torch.empty(c.block_length, dtype=torch.float64, device="cuda")
                provider(r.w, d)
                direct = c.pieces_2p2(d, r.w, r.y, xu, hg.FP64)
                assert np.array_equal(direct.p1, r.p1) and np.array_equal(direct.p234, r.p234)
        dev, st = runs["device"]
        assert st.pairs == n_pairs == len(dev) and st.positions_solved == n_prop
        assert st.cache_peak == peak
        host = runs["host"][0]
        for a, b in zip(dev, host):
            assert (a.x, a.y, a.yv) == (b.x, b.y, b.yv)
            assert a.kernel_sum == b.kernel_sum  # the same kernels on the same data
        key = lambda r: (r.x, r.y)  # noqa: E731
        ref = {key(r): r.kernel_sum for r in dev}
        # The batched launches split the sites over other CTAs, so the FP64
        # rounding differs. Measured at the pair's scale (both flavours as
        # one vector): a flavour that cancels to ~1e-3 of the pair carries
        # rounding of the pair's size (the oracle's own compensated and plain
        # orders differ by 7e-13 relative on such a flavour here).
        for name in ("batched", "graphs"):
            rows = runs[name][0]
            assert len(rows) == n_pairs
            for r in rows:
                assert S.pair_rel_err(r.kernel_sum, ref[key(r)]) <= 1e-12, name
        for r in dev:
            src = S.random_block(lat, S.source_seed(7, r.x))
            yb = S.random_block(lat, S.source_seed(7, r.y))
            orc = S.oracle_kernel_sum(src, yb, r.x, r.yv, xu, lat)
            assert S.pair_rel_err(r.kernel_sum, orc) <= 1e-12
        # a few pairs recomputed directly from freshly generated fields
        for r in (dev[0], dev[len(dev) // 2], dev[-1]):
            d_x = torch.empty(c.block_length, dtype=torch.float64, device="cuda")
            d_y = torch.empty_like(d_x)
            provider(r.x, d_x)
            provider(r.y, d_y)
            assert c.kernel_sum(d_x, d_y, r.x, r.yv, xu, hg.FP64) == r.kernel_sum


def test_run_chains_equals_independent_chains(tmp_path):
    """Two chains over one cache (driver.cpp:169-208) give the pairs and sums
    of each chain run alone (test_driver_random.cpp's two-chain check), the
    2+2 of a source solved by both chains is computed once, and the result
    file holds the in-memory results bit for bit (test_driver_random.cpp:351-352)."""
    import hlbl_gb300 as hg
    from hlbl_gb300 import schedule
    from hlbl_gb300.cache import PropagatorCache, TorchBuffers
    from hlbl_gb300.driver import run_chain, run_chains
    from hlbl_gb300.output import Chain, ResultWriter, RunInfo, TimingLog, read_results

    lat = (6, 6, 6, 6)
    xu = hg.xunit(105.6583745, 0.07957)
    chains = [schedule.build_schedule((1, 1, 1, 1), 1, 1), schedule.build_schedule((-1, 1, -1, 1), 1, 1)]
    with hg.Contractor(lat) as c:
        def provider(site, dest):
            c.fill_random_block(dest, hg.Contractor.source_seed(11, site))

        out22 = []
        cache = PropagatorCache("device", c.block_length, TorchBuffers(c))
        info = RunInfo(lattice=lat, chains=[Chain((0, 0, 0, 0), (1, 1, 1, 1), 1, 1),
                                            Chain((0, 0, 0, 0), (-1, 1, -1, 1), 1, 1)],
                       xunit=xu, with_2p2=True)
        writer = ResultWriter(str(tmp_path / "run.npz"), info)
        timing = TimingLog(str(tmp_path / "timing.csv"))
        res, st, _ = run_chains(chains, lat, xu, provider, c, cache, precision=hg.FP32,
                                sources_2p2=[((0, 0, 0, 0), [(1, 1, 1, 1)])], results_2p2=out22,
                                writer=writer, timing=timing)
        timing.close()
        alone = []
        for i, ch in enumerate(chains):
            r, _ = run_chain(ch, lat, xu, provider, c, PropagatorCache("device", c.block_length,
                                                                      TorchBuffers(c)),
                             chain=i, precision=hg.FP32)
            alone.extend(r)
        assert [(r.x, r.y, r.yv, r.chain) for r in res] == [(r.x, r.y, r.yv, r.chain) for r in alone]
        assert [r.kernel_sum for r in res] == [r.kernel_sum for r in alone]
        assert len(out22) == 1 and out22[0].chain == 0 and st.pieces_2p2 == 1
        f = read_results(str(tmp_path / "run.npz"))
        assert np.array_equal(f["kernel_sum/kernel_sum"], np.array([r.kernel_sum for r in res]))
        assert [tuple(v) for v in f["kernel_sum/x"]] == [r.x for r in res]
        assert [tuple(v) for v in f["kernel_sum/yv"]] == [tuple(r.yv) for r in res]
        assert list(f["kernel_sum/chain"]) == [r.chain for r in res]
        assert np.array_equal(f["2p2/P1"][0], np.asarray(out22[0].p1).reshape(4, 4, 4, max(lat)))
        assert np.array_equal(f["2p2/P234"].reshape(-1, 5, 64), np.asarray(out22[0].p234).reshape(-1, 5, 64))
        rows = open(tmp_path / "timing.csv").read().splitlines()[1:]
        assert sum(r.startswith("kernel_sum,") for r in rows) == st.pairs


def test_driver_fp32_copies_chain_total():
    """The batched loop on the device32 cache (FP32 tile copies made as each
    block is stored, kernel_sums_batched_f32, a CUDA graph per window) over a
    whole chain (stride 2, two steps) of a 16^4 lattice with Gaussian fields:
    every pair within 1e-4 of the FP64 per-pair loop at the pair's scale, and
    each flavour's chain total within 1e-6 of the chain's scale, the sum of
    its pairs' magnitudes. (Gaussian fields give kernel sums of random sign,
    so a chain total cancels to a few pairs' size -- 145 pairs here sum to
    about half of the largest one -- and its error relative to the cancelled
    total measures the cancellation, not the arithmetic: 4.0e-6 here, while
    the 24^3x48 benchmark's total, 2.7e-7, does not cancel as much.)"""
    import hlbl_gb300 as hg
    from hlbl_gb300 import schedule
    from hlbl_gb300.cache import PropagatorCache, TorchBuffers
    from hlbl_gb300.driver import run_chain

    lat = (16, 16, 16, 16)
    xu = hg.xunit(105.658, 0.1)
    steps = schedule.build_schedule((1, -1, 1, -1), 2, 2)
    with hg.Contractor(lat) as c:
        def provider(site, dest):
            c.fill_gaussian_block(dest, hg.Contractor.source_seed(11, site))

        f64, _ = run_chain(steps, lat, xu, provider, c, PropagatorCache("device", c.block_length, TorchBuffers(c)),
                           precision=hg.FP64)
        f32, st = run_chain(steps, lat, xu, provider, c,
                            PropagatorCache("device32", c.block_length, TorchBuffers(c)), batched=True,
                            graphs=True,
                            out_factory=lambda n: torch.zeros((n, 2), dtype=torch.float64, device="cuda"))
    ref = {(r.x, r.y): r.kernel_sum for r in f64}
    assert len(f32) == len(f64) == st.pairs
    worst = max(S.pair_rel_err(r.kernel_sum, ref[(r.x, r.y)]) for r in f32)
    tot32 = np.sum([r.kernel_sum for r in f32], axis=0)
    tot64 = np.sum([r.kernel_sum for r in f64], axis=0)
    scale = np.sum([np.abs(r.kernel_sum) for r in f64], axis=0)
    assert worst <= 1e-4
    assert np.all(np.abs(tot32 - tot64) <= 1e-6 * scale), (tot32, tot64, scale)
