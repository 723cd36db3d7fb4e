"""PropagatorCache and the driver loop's bookkeeping on CPU (fake buffers,
no contraction), against the reference's schedule simulation."""
import numpy as np
import pytest

import support as S
from hlbl_gb300 import schedule
from hlbl_gb300.cache import PropagatorCache
from hlbl_gb300.driver import run_chain


class NumpyBuffers:
    def __init__(self):
        self.staged = 0

    def device(self, n):
        return np.zeros(n)

    def pinned(self, n):
        return np.zeros(n)

    def stage(self, dst, src):
        dst[:] = src
        self.staged += 1

    def store(self, dst, src):
        dst[:] = src

    def device32(self):
        return np.zeros(4, dtype=np.float32)

    def convert(self, dst32, src):
        dst32[:] = src[:4]


class Recorder:
    """Stands in for the Contractor: returns a value the test can predict."""

    def kernel_sum(self, d_x, d_y, gx, yv, xunit, precision):
        return float(d_x[0] + 10 * d_y[0]), float(sum(gx) + sum(yv))

    def pieces_2p2(self, d_fwd, gsw, targets, xunit, precision):
        from hlbl_gb300.contract import Pieces2p2

        # the block it was given, the source and the number of targets
        return Pieces2p2(np.array([d_fwd[0], sum(gsw)]), np.full(len(targets), float(len(targets))))


def provider(site, dest):
    dest[:] = hash(site) % 1000


@pytest.mark.parametrize("residency", ["device", "host"])
def test_driver_loop_matches_schedule_simulation(residency):
    lat = (6, 6, 6, 6)
    steps = schedule.build_schedule((1, 1, 1, 1), 1, 2)
    n_prop, n_pairs, peak = schedule.simulate(steps)
    buf = NumpyBuffers()
    cache = PropagatorCache(residency, 4, buf)
    res, st = run_chain(steps, lat, 0.1, provider, Recorder(), cache)
    assert st.pairs == n_pairs == len(res) and st.positions_solved == n_prop
    assert st.cache_peak == peak == 16
    for r in res:
        assert r.kernel_sum[0] == (hash(r.x) % 1000) + 10 * (hash(r.y) % 1000)
        assert all(abs(v) == 1 for v in r.yv)
    if residency == "host":
        # slot 0 stays staged across a source's partners (propagator_cache.cpp:63-66)
        assert buf.staged < 2 * n_pairs


class BatchRecorder:
    """Stands in for the Contractor's batched calls (FP64 blocks or FP32
    copies), writing a value the test can predict into the output rows."""

    def __init__(self):
        self.calls = {"f64": 0, "f32": 0}

    def _fill(self, d_y, xs, gxs, yvs, out):
        for i, (x, g, v) in enumerate(zip(xs, gxs, yvs)):
            out[i] = (float(x[0] + 10 * d_y[0]), float(sum(g) + sum(v)))

    def kernel_sums_batched(self, d_y, xs, gxs, yvs, xunit, out, precision):
        self.calls["f64"] += 1
        self._fill(d_y, xs, gxs, yvs, out)

    def kernel_sums_batched_f32(self, d_y32, xs, gxs, yvs, xunit, out):
        assert d_y32.dtype == np.float32 and all(x.dtype == np.float32 for x in xs)
        self.calls["f32"] += 1
        self._fill(d_y32, xs, gxs, yvs, out)

    def check(self):
        pass


class Rows(np.ndarray):
    def cpu(self):
        return self


@pytest.mark.parametrize("residency", ["device", "device32"])
def test_batched_loop_on_fp64_blocks_and_fp32_copies(residency):
    """The batched loop over the device cache (FP64 blocks) and the device32
    cache (FP32 copies converted as each block is stored): the same pairs and
    values as the per-pair loop, one batched call per source with partners,
    and the copies' buffers reused after eviction."""
    lat = (6, 6, 6, 6)
    steps = schedule.build_schedule((1, 1, 1, 1), 1, 2)
    n_prop, n_pairs, _ = schedule.simulate(steps)
    ref, _ = run_chain(steps, lat, 0.1, provider, Recorder(), PropagatorCache("device", 4, NumpyBuffers()))
    rec = BatchRecorder()
    cache = PropagatorCache(residency, 4, NumpyBuffers())
    res, st = run_chain(steps, lat, 0.1, provider, rec, cache, batched=True,
                        out_factory=lambda n: np.zeros((n, 2)).view(Rows))
    assert st.pairs == n_pairs == len(res) and st.positions_solved == n_prop
    assert sorted((r.x, r.y) for r in res) == sorted((r.x, r.y) for r in ref)
    want = {(r.x, r.y): r.kernel_sum[0] for r in ref}
    assert all(r.kernel_sum[0] == want[(r.x, r.y)] for r in res)
    n_src = sum(1 for stp in steps for src in stp.sources if src.partners)
    assert rec.calls == ({"f64": 0, "f32": n_src} if residency == "device32" else {"f64": n_src, "f32": 0})
    if residency == "device32":
        # one copy buffer per entry alive at the peak (the batched loop solves a
        # whole window first), reused after eviction
        assert cache.scratch is not None and len(cache.pool) + cache.size() == st.cache_peak
    with pytest.raises(ValueError):
        run_chain(steps, lat, 0.1, provider, Recorder(), PropagatorCache("device32", 4, NumpyBuffers()))


def test_driver_2p2_at_first_solves():
    """The 2+2 pieces of the listed sources are computed once, at their first
    solve, from the block just solved (driver.cpp:58-96)."""
    lat = (6, 6, 6, 6)
    steps = schedule.build_schedule((1, 1, 1, 1), 1, 2)
    solved = [tuple(schedule.mod_pos(s.position, lat)) for st in steps for s in st.sources]
    want = {solved[0]: [(1, 2, 3, 4)], solved[5]: [(0, 0, 0, 0), (5, 5, 5, 5), (1, 1, 1, 1)]}
    buf = NumpyBuffers()
    cache = PropagatorCache("device", 4, buf)
    out = []
    res, st = run_chain(steps, lat, 0.1, provider, Recorder(), cache, sources_2p2=want,
                        results_2p2=out)
    assert st.pieces_2p2 == 2 and st.targets_2p2 == 4
    assert [r.w for r in out] == [solved[0], solved[5]]
    for r in out:
        assert r.p1[0] == hash(r.w) % 1000 and r.p1[1] == sum(r.w)  # the solved block
        assert r.y == want[r.w] and len(r.p234) == len(r.y)
        assert r.yv == [tuple(schedule.site_map_diff(t, r.w, lat)) for t in r.y]
    with pytest.raises(ValueError):
        run_chain(steps, lat, 0.1, provider, Recorder(), PropagatorCache("device", 4, buf),
                  sources_2p2=want)


def test_run_chains_16_chains_and_2p2_plan():
    """All 16 h as 16 chains over one cache (driver.cpp:169-208): every
    chain's pairs, and the 2+2 of each source once, at its first solve over
    all chains (the plan)."""
    from hlbl_gb300.driver import run_chains

    lat = (6, 6, 6, 6)
    chains = [schedule.build_schedule(h, 1, 1) for h in schedule.sign_vectors()]
    per_chain = [schedule.simulate(c) for c in chains]
    srcs = [((1, 1, 1, 1), [(0, 0, 0, 0)]), ((5, 5, 5, 5), [(1, 2, 3, 4), (2, 2, 2, 2)]),
            ((3, 3, 3, 3), [(0, 1, 0, 1)])]
    out = []
    cache = PropagatorCache("device", 4, NumpyBuffers())
    res, st, warn = run_chains(chains, lat, 0.1, provider, Recorder(), cache, sources_2p2=srcs,
                               results_2p2=out)
    assert st.pairs == len(res) == sum(p for _, p, _ in per_chain)
    assert st.positions_solved == sum(n for n, _, _ in per_chain)
    plan = schedule.plan_2p2(chains, [s for s, _ in srcs], lat)
    want = sorted(tuple(schedule.mod_pos(pos, lat)) for d in plan.at for pos in d)
    assert sorted(r.w for r in out) == want and st.pieces_2p2 == len(want)
    assert len(set(r.w for r in out)) == len(out)  # once per source
    assert any("not solved by any chain" in w for w in warn)  # (3,3,3,3) is not solved
    with pytest.raises(RuntimeError):
        run_chains([], lat, 0.1, provider, Recorder(), cache)


def test_cache_errors_as_the_reference():
    cache = PropagatorCache("host", 4, NumpyBuffers(), {(0, 0, 0, 0): 1})
    cache.begin_insert((0, 0, 0, 0))
    cache.end_insert((0, 0, 0, 0))
    with pytest.raises(RuntimeError, match="inserted twice"):
        cache.begin_insert((0, 0, 0, 0))
    with pytest.raises(RuntimeError, match="not cached"):
        cache.device_ptr((1, 0, 0, 0), 0)
    with pytest.raises(RuntimeError, match="bad slot"):
        cache.device_ptr((0, 0, 0, 0), 2)
    with pytest.raises(RuntimeError, match="still cached"):
        cache.reset({})


def test_schedule_matches_reference():
    G = S.golden()
    for sc in G["schedule"]:
        steps = schedule.build_schedule(tuple(sc["h"]), sc["stride"], sc["steps"])
        mine = [list(o) + list(n) + [w] for o, n, w in schedule.all_pairs(steps)]
        assert mine == sc["pairs"]
    for s in G["schedule_stats"]:
        steps = schedule.build_schedule(tuple(s["h"]), s["stride"], s["steps"])
        assert schedule.simulate(steps) == (s["propagators"], s["pairs"], s["peak"])
    # the counts of the benchmark configurations (16 + 15K, 15 + 65K)
    for K, props, pairs in ((1, 31, 80), (4, 76, 275), (8, 136, 535)):
        n = schedule.simulate(schedule.build_schedule((1, -1, 1, -1), 2, K))
        assert n[0] == props and n[1] == pairs
