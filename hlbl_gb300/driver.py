"""The schedule loop of the reference's driver (src/driver.cpp:23-165): solve
each new source, contract it with its partners, free propagators after
their last pair. Two pair loops:

  per_pair  Contractor.kernel_sum once per pair, as driver.cpp:104-134 does;
  batched   one kernel_sums_batched per new source (all pairs it closes share
            its block), optionally recorded as one CUDA graph per window;
            with the device32 cache (FP32 tile copies of the blocks, made as
            each block is stored) one kernel_sums_batched_f32 per new source.

With `sources_2p2` ({global site: [targets]}), the first solve of each of
those sites computes its 2+2 pieces from the freshly solved block, before the
block is stored (driver.cpp:58-96: Contractor.pieces_2p2 in the solve step).

`provider(site, dest)` fills a block for a global site (the reference's
PropagatorProvider::compute); `contract` is a Contractor (or, in CPU tests,
any object with the same two methods).
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field
from typing import Callable, List, Tuple

from . import schedule as sch
from .cache import PropagatorCache


@dataclass
class PairResult:
    """driver.hpp/output.hpp PairResult: x, y (wrapped), y - x, chain, window."""
    x: tuple
    y: tuple
    yv: tuple
    chain: int
    window: int
    kernel_sum: Tuple[float, float] = (0.0, 0.0)


@dataclass
class Result2p2:
    """output.hpp Result2p2: the source w, its targets y and y - w, chain,
    window, and the pieces (p1 [4][4][4][Lmax], p234 [n_y][5][64])."""
    w: tuple
    y: list
    yv: list
    chain: int
    window: int
    p1: object = None
    p234: object = None


@dataclass
class RunStats:
    positions_solved: int = 0
    pairs: int = 0
    cache_peak: int = 0
    windows: List[int] = field(default_factory=list)
    pieces_2p2: int = 0
    targets_2p2: int = 0


def run_chain(steps, lattice, xunit: float, provider: Callable, contractor, cache: PropagatorCache,
              chain: int = 0, precision=0, batched: bool = False, graphs: bool = False,
              out_factory=None, sources_2p2=None, results_2p2=None, at_2p2=None, writer=None,
              timing=None):
    """One chain; returns ([PairResult], RunStats). With batched=True,
    out_factory(n) must return a device buffer of n x 2 doubles. 2+2: either
    `sources_2p2` ({global site: targets}, at the site's first solve in this
    chain) or `at_2p2` ({solve position as in the schedule: targets}, a
    plan over several chains, run_chains); results appended to `results_2p2`.
    `writer` (output.ResultWriter) gets each window's rows and 2+2 results,
    `timing` (output.TimingLog) a row per solve, kernel sum (the per-pair
    loop) and 2+2 source (driver.cpp:58-151)."""
    pending = {}
    for older, newer, _ in sch.all_pairs(steps):
        pending[older] = pending.get(older, 0) + 1
        pending[newer] = pending.get(newer, 0) + 1
    cache.reset(pending)
    wrap = lambda p: sch.mod_pos(p, lattice)  # noqa: E731
    results: List[PairResult] = []
    stats = RunStats()
    todo_2p2 = {tuple(wrap(k)): list(v) for k, v in (sources_2p2 or {}).items()}
    at = {tuple(k): list(v) for k, v in (at_2p2 or {}).items()}
    if (todo_2p2 or at) and results_2p2 is None:
        raise ValueError("run_chain: 2+2 sources need a results_2p2 list")

    window_2p2 = []

    def solve(window, position):
        dest = cache.begin_insert(position)
        site = tuple(wrap(position))
        t0 = time.perf_counter()
        provider(site, dest)
        if timing is not None:
            timing.solve(chain, window, site, time.perf_counter() - t0, 0)
        stats.positions_solved += 1
        # 2+2 at the site's first solve, from the block just solved
        targets = at.pop(tuple(position), None)
        if targets is None:
            targets = todo_2p2.pop(site, None)
        if targets is not None:
            t0 = time.perf_counter()
            pc = contractor.pieces_2p2(dest, site, targets, xunit, precision)
            if timing is not None:
                timing.pieces_2p2(chain, window, site, time.perf_counter() - t0)
            r = Result2p2(site, [tuple(t) for t in targets],
                          [tuple(sch.site_map_diff(t, site, lattice)) for t in targets],
                          chain, window, pc.p1, pc.p234)
            results_2p2.append(r)
            window_2p2.append(r)
            stats.pieces_2p2 += 1
            stats.targets_2p2 += len(targets)
        cache.end_insert(position)
    if batched and cache.residency not in ("device", "device32"):
        raise ValueError("the batched loop needs a device cache (every partner resident)")
    if cache.residency == "device32" and not batched:
        raise ValueError("the device32 cache (FP32 copies) feeds the batched FP32-copy loop only")
    f32 = cache.residency == "device32"
    for st in steps:
        window_rows = []
        if not batched:
            # the reference's order: each source contracted right after its
            # solve, pair by pair (driver.cpp:104-134); peak 16
            for src in st.sources:
                solve(st.index, src.position)
                if not src.partners:
                    continue
                gy = wrap(src.position)
                d_y = cache.device_ptr(src.position, 0)
                for q in src.partners:
                    d_x = cache.device_ptr(q, 1)
                    gx = wrap(q)
                    yv = sch.site_map_diff(src.position, q, lattice)
                    t0 = time.perf_counter()
                    ks = contractor.kernel_sum(d_x, d_y, gx, yv, xunit, precision)
                    if timing is not None:
                        timing.kernel_sum(chain, st.index, gx, gy, time.perf_counter() - t0)
                    window_rows.append(PairResult(gx, gy, yv, chain, st.index, tuple(ks)))
                    cache.pair_done(q, src.position)
                    stats.pairs += 1
        else:
            # the window's solves first (the reference's serial order, peak
            # 30), then one batched call per new source, optionally recorded
            # as one CUDA graph for the window
            for src in st.sources:
                solve(st.index, src.position)
            calls = []
            for src in st.sources:
                if not src.partners:
                    continue
                gy = wrap(src.position)
                xs = [cache.device_ptr(q, 1) for q in src.partners]
                gxs = [wrap(q) for q in src.partners]
                yvs = [sch.site_map_diff(src.position, q, lattice) for q in src.partners]
                rows = [PairResult(g, gy, v, chain, st.index) for g, v in zip(gxs, yvs)]
                calls.append((cache.device_ptr(src.position, 0), xs, gxs, yvs, rows,
                              out_factory(len(xs)), src))
            if graphs:
                contractor.graph_begin()
            for d_y, xs, gxs, yvs, _, buf, _ in calls:
                if f32:
                    contractor.kernel_sums_batched_f32(d_y, xs, gxs, yvs, xunit, buf)
                else:
                    contractor.kernel_sums_batched(d_y, xs, gxs, yvs, xunit, buf, precision)
            if graphs:
                g = contractor.graph_end()
                g.launch()
            contractor.check()  # the context's stream is done (and no kernel gave up)
            for _, _, _, _, rows, buf, src in calls:
                for r, v in zip(rows, buf.cpu().tolist()):
                    r.kernel_sum = (v[0], v[1])
                window_rows.extend(rows)
                for q in src.partners:
                    cache.pair_done(q, src.position)
                    stats.pairs += 1
            if graphs:
                g.close()
        results.extend(window_rows)
        stats.windows.append(len(window_rows))
        # the window's rows go to the result file as the window ends (driver.cpp:136-151)
        if writer is not None:
            writer.append(window_rows)
            if window_2p2:
                writer.append_2p2(window_2p2)
        window_2p2.clear()
    if cache.size() != 0:
        raise RuntimeError("run_chain: propagators left in the cache")
    stats.cache_peak = cache.peak
    return results, stats


def run_chains(chains, lattice, xunit: float, provider: Callable, contractor, cache: PropagatorCache,
               precision=0, batched: bool = False, graphs: bool = False, out_factory=None,
               sources_2p2=None, results_2p2=None, writer=None, timing=None):
    """Several chains over one cache (driver.cpp:169-208): the chains in
    order, the 2+2 of each source in `sources_2p2` ([(source, targets)]) at
    its first solve over all chains (schedule.plan_2p2). Returns
    ([PairResult], RunStats, [warning lines of the plan])."""
    if not chains:
        raise RuntimeError("run_chains: no chains")
    if not xunit > 0:
        raise RuntimeError("run_chains: xunit (m_mu a) is not set")
    srcs = [tuple(s) for s, _ in (sources_2p2 or [])]
    plan = sch.plan_2p2(chains, srcs, lattice)
    total = RunStats()
    results: List[PairResult] = []
    for c, steps in enumerate(chains):
        at = {pos: list(sources_2p2[i][1]) for pos, i in plan.at[c].items()}
        res, st = run_chain(steps, lattice, xunit, provider, contractor, cache, chain=c,
                            precision=precision, batched=batched, graphs=graphs,
                            out_factory=out_factory, results_2p2=results_2p2, at_2p2=at,
                            writer=writer, timing=timing)
        results.extend(res)
        total.positions_solved += st.positions_solved
        total.pairs += st.pairs
        total.cache_peak = max(total.cache_peak, st.cache_peak)
        total.windows.extend(st.windows)
        total.pieces_2p2 += st.pieces_2p2
        total.targets_2p2 += st.targets_2p2
    return results, total, sch.report_2p2(plan, srcs)
