"""The driver loop on random fields, as the reference's test_driver_random
(sanity_check/test_driver_random.cpp:133-234): pair count and cache peak
from the schedule simulation, device vs host cache giving the same sums, a
few pairs recomputed directly -- plus the batched loop, with and without a
CUDA graph per window, against the per-pair loop."""
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

        runs = {}
        for name, res, batched, graphs in (("device", "device", False, False),
                                           ("host", "host", False, False),
                                           ("batched", "device", True, False),
                                           ("graphs", "device", True, True)):
            cache = PropagatorCache(res, c.block_length, TorchBuffers(c))
            out = run_chain(steps, lat, xu, provider, c, cache, precision=hg.FP64, batched=batched,
                            graphs=graphs,
                            out_factory=lambda n: torch.zeros((n, 2), dtype=torch.float64, device="cuda"))
            runs[name] = out
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
