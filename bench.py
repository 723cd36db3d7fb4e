#!/usr/bin/env python
"""Benchmark: connected-HLbL kernel sums (pairs/s) at 24^3 x 48 on GB300.

Workload (the reference's 24^3 x 48 configuration): lattice T=48, L=24
(V = 663,552 sites, 3.06 GB per propagator block), i.i.d. complex Gaussian
FP64 propagator blocks (seeded, generated on the device), the sliding-
hypercube schedule with stride 2, h = (+1,-1,+1,-1), K = 4 (76 propagators,
275 pairs). One step = every pair one newly solved source closes (the
sources of window 1 in solve order: up to 8 pairs each, 65 per window).

Printed (one JSON line, rank 0):
  value      pairs/s of the headline path (blocks as FP32 tile copies, FP32
             per-site products with pass 2 on the tensor cores, FP64 sums,
             batched per source, one CUDA graph for the timed sources) over K
             steps with the blocks resident in HBM (inputs are 3 GB each, far
             above the 129 MB L2, so no flush is needed between steps);
  fp64       pairs/s of the plain FP64 path on the same pairs;
  e2e        the same metric through the C ABI with host buffers: each step
             copies its new block from pinned host memory and reads back its
             kernel sums (median of seven passes);
  roofline   the dominant kernel (pass 2, against a cuBLAS TF32 GEMM measured
             in the run; pass 1 against the measured HBM bandwidth beside it);
  pieces_2p2 the 2+2 pieces of one source for 16 targets (compute_2p2_gpu);
  cpu_baseline  the CPU oracle (the reference's loops restated in C, plain
             summation, all host threads) on a bounded sample of one pair.

  python bench.py [--only-2p2] [--lattice T,LX,LY,LZ]   (profiling runs)
  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

LATTICE = (48, 24, 24, 24)
STRIDE, H, NSTEPS = 2, (1, -1, 1, -1), 4
RUN_SEED = 20261203
DENSE_SEED = 20261204  # table seed of the dense test QED weight
MUON_MEV, SPACING_FM = 105.658, 0.1
BYTES_PER_SITE_PASS = 2 * 2 * 12 * 24 * 8  # two blocks, both flavours, per pass
METRIC = "pairs/sec & HBM GB/s at 24^3x48: batched+surrogate vs plain FP64 at 1e-4 rel"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-chains16", action="store_true", help="skip the 16-chain driver run")
    ap.add_argument("--config5", action="store_true",
                    help="the 48^3x96 host-cache line alone (about 75 GB of pinned host memory)")
    ap.add_argument("--c5-partners", type=int, default=3)
    ap.add_argument("--config2-chain", action="store_true",
                    help="the whole 24^3x48 chain (275 pairs) in FP32 and FP64, every pair's error (minutes)")
    ap.add_argument("--c2-ref-pairs", type=int, default=8)
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip the baseline leg of the reference's own kernels on the GPU")
    ap.add_argument("--tc-tf32", action="store_true",
                    help="TF32 operands in the tensor-core pass 2 instead of FP16 (the library's default)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default kernel variants (profiling: the first launches are the timed ones)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--train-samples", type=int, default=4 * 1024 * 1024)
    ap.add_argument("--train-steps", type=int, default=12000)
    ap.add_argument("--only-2p2", action="store_true",
                    help="time only the 2+2 pieces of one source (profiling runs)")
    ap.add_argument("--lattice", default=None,
                    help="T,LX,LY,LZ of a smaller lattice (profiling runs); default 48,24,24,24")
    args = ap.parse_args()
    if args.lattice:
        global LATTICE
        LATTICE = tuple(int(a) for a in args.lattice.split(","))
        assert len(LATTICE) == 4
    return args


def volume(lat):
    return lat[0] * lat[1] * lat[2] * lat[3]


def workload() -> str:
    """The workload both arms report (config.workload)."""
    return (f"lattice {'x'.join(map(str, LATTICE))} (V={volume(LATTICE)}), stride 2, h=(+1,-1,+1,-1), K=4; "
            "step = the pairs one new source closes (window 1 sources)")


def window_steps():
    """(new source, [partners]) of windows >= 1, in solve order."""
    from hlbl_gb300 import schedule

    st = schedule.build_schedule(H, STRIDE, NSTEPS)
    return [(s.position, list(s.partners)) for w in st[1:] for s in w.sources if s.partners]


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def load_traffic():
    """Per-launch DRAM bytes of the pass-2 kernel from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "p2_kernel_traffic.json")) as fh:
            return json.load(fh)
    except OSError:
        return None


def measure_tf32_peak(torch):
    """cuBLAS TF32 GEMM throughput (8192^3, FP32 in/out with TF32 math), best of 10."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    try:
        n = 8192
        a = torch.randn(n, n, device="cuda")
        b = torch.randn(n, n, device="cuda")
        for _ in range(3):
            a @ b
        best = 1e30
        for _ in range(10):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            a @ b
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        del a, b
        return 2 * n ** 3 / (best * 1e-3) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs: every
    50 ms, started (and waited for until its first sample is written) before
    the region, so that the samples cover it."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "50"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        t_end = time.time() + 3.0
        while self.p is not None and time.time() < t_end and self.p.poll() is None:
            if os.path.getsize(self.f.name) > 0:
                break
            time.sleep(0.01)

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        sm, mx, reasons = [], None, set()
        for r in rows:
            try:
                sm.append(float(r[0]))
                mx = float(r[1])
                for n, v in zip(names, r[3:7]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle on a slab of time slices of one pair
# ---------------------------------------------------------------------------
def cpu_pair_seconds(src_h, y_h, gsx, yv, xu, n_slices, threads=None):
    """Seconds per pair from a slab sample: pass 1 + pass 2, both flavours,
    over n_slices time slices, scaled by T / n_slices."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import numpy as np
    import support as S

    o = S.oracle()
    if threads:
        o.oracle_set_threads(threads)
    o.oracle_set_compensated(0)  # the reference's plain loops
    T, L = LATTICE[0], LATTICE[1:]
    V = volume(LATTICE)
    vs = n_slices * L[0] * L[1] * L[2]
    sl_src = np.ascontiguousarray(src_h.reshape(24, V, 24)[:, :vs, :])
    sl_y = np.ascontiguousarray(y_h.reshape(24, V, 24)[:, :vs, :])
    local = (n_slices,) + L
    t0 = time.perf_counter()
    for f in (0, 1):
        dzu, dzsu = S.oracle_dz(sl_src, sl_y, f, gsx, LATTICE, local)
        g_dzu, g_dzsu = S.oracle_gammas(dzu, dzsu)
        S.oracle_4pt(g_dzu, g_dzsu, sl_src, sl_y, f, gsx, xu, yv, LATTICE, local)
    dt = time.perf_counter() - t0
    o.oracle_set_compensated(1)
    return dt * T / n_slices, int(o.oracle_get_threads())


def pick_slices(src_h, y_h, gsx, yv, xu, budget_s):
    t1, _ = cpu_pair_seconds(src_h, y_h, gsx, yv, xu, 1)
    per_slice = t1 / LATTICE[0]
    return max(1, min(LATTICE[0], int(round(budget_s / max(per_slice, 1e-6)))))


# ---------------------------------------------------------------------------
def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    import torch

    if args.impl == "reference":
        return run_reference(args, rank, world)

    import hlbl_gb300 as hg
    from hlbl_gb300 import schedule
    from hlbl_gb300.contract import measure_fma_peak

    torch.cuda.set_device(local_rank)
    if args.config5:
        return run_config5(args, hg, torch, rank)
    if args.config2_chain:
        return run_config2_chain(args, hg, torch, rank)
    if args.only_2p2:
        return run_2p2_only(args, hg, torch, rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    xu = hg.xunit(MUON_MEV, SPACING_FM)
    steps_all = window_steps()
    nst = len(steps_all)
    # weak scaling: rank r takes steps r, r+world, ... (pairs are independent)
    order = [steps_all[(rank + world * i) % nst] for i in range(args.warmup + args.steps)]
    warm, timed = order[:args.warmup], order[args.warmup:]

    c = hg.Contractor(LATTICE, device=local_rank)
    p2_fp16 = not args.tc_tf32
    c.set_tc_fp16(p2_fp16)
    stream = torch.cuda.Stream()
    c.set_stream(stream)
    blocks = {}

    def block(p):
        site = schedule.mod_pos(p, LATTICE)
        if site not in blocks:
            t = torch.empty(c.block_length, dtype=torch.float64, device="cuda")
            with torch.cuda.stream(stream):
                c.fill_gaussian_block(t, hg.Contractor.source_seed(RUN_SEED, site))
            blocks[site] = t
        return blocks[site]

    for p, qs in order:
        block(p)
        for q in qs:
            block(q)
    stream.synchronize()

    def pairs_of(step):
        p, qs = step
        return [(q, p, schedule.mod_pos(q, LATTICE), schedule.site_map_diff(p, q, LATTICE)) for q in qs]

    n_timed_pairs = sum(len(s[1]) for s in timed)
    n_rows = max(16, n_timed_pairs, sum(len(s[1]) for s in warm))
    res = torch.zeros((n_rows, 2), dtype=torch.float64, device="cuda")

    def step_args(st):
        pr = pairs_of(st)
        return (block(st[0]), [block(q) for q, _, _, _ in pr], [g for _, _, g, _ in pr],
                [v for _, _, _, v in pr])

    def run_batched(steps, prec, out):
        """One batched call per step (the pairs its new source closes)."""
        k = 0
        for st in steps:
            y_b, xs, gs, vs = step_args(st)
            c.kernel_sums_batched(y_b, xs, gs, vs, xu, out[k:k + len(xs)], prec)
            k += len(xs)
        return k

    # FP32 tile copies of the blocks, made once per block (as the driver
    # does when a solved block enters its cache): a step converts its new
    # source's block inside the timed region; partners were converted when
    # they were new
    blocks32 = {}

    def block32(p, make=True):
        site = schedule.mod_pos(p, LATTICE)
        if site not in blocks32:
            blocks32[site] = torch.empty(c.f32_block_length, dtype=torch.float32, device="cuda")
            if make:
                c.f32_tile_copy(block(p), blocks32[site])
        return blocks32[site]

    def run_batched32(steps, out):
        """The FP32-copy path: per step, convert the new block, then one
        batched call over the FP32 copies."""
        k = 0
        for st in steps:
            p, qs = st
            y32 = block32(p, make=False)
            c.f32_tile_copy(block(p), y32)
            pr = pairs_of(st)
            c.kernel_sums_batched_f32(y32, [block32(q) for q, _, _, _ in pr], [g for _, _, g, _ in pr],
                                      [v for _, _, _, v in pr], xu, out[k:k + len(pr)])
            k += len(pr)
        return k

    def run_pairs(steps, prec, out):
        """The per-pair API, one call per pair (the reference driver's loop)."""
        k = 0
        for st in steps:
            for q, p, gx, yv in pairs_of(st):
                c.kernel_sum_async(block(q), block(p), gx, yv, xu, out[k], precision=prec)
                k += 1
        return k

    def timeit(fn, *a):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        ev0.record(stream)
        n = fn(*a)
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        if dist:
            t = torch.tensor([ms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return n, ms

    def graph_timed():
        """Record the timed sources' work (conversion of each new block and
        one batched call) as one CUDA graph and time one replay (all K steps)."""
        c.graph_begin()
        run_batched32(timed, res)
        graph = c.graph_end()
        clocks = ClockSampler(local_rank)
        n, ms = timeit(lambda: (graph.launch(stream), n_timed_pairs)[1])
        graph.close()
        return n, ms, clocks.stop()

    # ---- headline: batched per new source on FP32 tile copies (one
    #      conversion per new block), FP32 products (pass 2 on the tensor
    #      cores), FP64 sums, the exact QED weight (FP32 quadrature, FP64 near
    #      the origin), one CUDA graph for the timed sources, autotuned -------
    c.set_qed(None)
    c.reserve(16)
    with torch.cuda.stream(stream):
        for p, qs in order:
            for q in qs:
                block32(q)  # partners were converted when they entered the cache
        for p, _ in order:
            block32(p, make=False)  # the new blocks' copies: buffers now, converted in their steps
    st0 = warm[0] if warm else timed[0]
    y32_0 = block32(st0[0])
    pr0 = pairs_of(st0)
    if args.no_autotune:
        tune = {"p1": "two stages, 1 CTA/SM", "p2": "tensor-core", "batch_group": 1, "ms": None}
    else:
        tune = c.autotune_f32(y32_0, [block32(q) for q, _, _, _ in pr0], [g for _, _, g, _ in pr0],
                              [v for _, _, _, v in pr0], xu, res[:len(pr0)])
    run_batched32(warm, res)
    stream.synchronize()
    n32, ms32, clk = graph_timed()
    res_main = res.clone()

    # ---- the same without the graph; the FP64-block batched API; per pair --
    res_b = torch.zeros_like(res)
    nb_, msb = timeit(run_batched32, timed, res_b)
    y0, xs0, gs0, vs0 = step_args(warm[0] if warm else timed[0])
    tune64 = {"no_autotune": True} if args.no_autotune else c.autotune(y0, xs0, gs0, vs0, xu, res[:len(xs0)])
    res_f64b = torch.zeros_like(res)
    run_batched(timed[:1], hg.FP32, res_f64b)
    nfb, msfb = timeit(run_batched, timed, hg.FP32, res_f64b)
    res_p = torch.zeros_like(res)
    run_pairs(timed[:1], hg.FP32, res_p)
    npp, mspp = timeit(run_pairs, timed, hg.FP32, res_p)

    # ---- the generic QED path: the coefficient stage (any QED kernel) and
    #      pass 2 with the generic epilogue, no structure of the tensor used;
    #      the stand-in through it, and the dense test weight (no closed form)
    #      checked against the FP64 path with the same weight ---------------------
    generic = {}
    n_first = len(timed[0][1])
    for name, kind in (("standin_generic", hg.QED_STANDIN_GENERIC), ("dense", hg.QED_DENSE)):
        c.set_qed_kernel(kind, DENSE_SEED)
        run_batched32(warm[:1] or timed[:1], res)
        stream.synchronize()
        ng, msg, _ = graph_timed()
        rg = res[:ng].clone()
        c.set_profiling(True)
        run_batched32(timed[:1], res_b)
        stream.synchronize()
        (g1ms, g1n), (g2ms, g2n) = c.kernel_times()
        c.set_profiling(False)
        ent = {"value": round(ng * world / (msg * 1e-3), 4), "unit": "pairs/s", "pairs_timed": ng,
               "p1_kernel_ms": round(g1ms / max(1, g1n), 3), "p2_kernel_ms": round(g2ms / max(1, g2n), 3)}
        if kind == hg.QED_STANDIN_GENERIC:
            a, b = rg.cpu().double(), res_main[:ng].cpu().double()
            ent["max_rel_err_vs_closed_form"] = (
                ((a - b).abs().max(1).values / b.abs().max(1).values.clamp_min(1e-300)).max().item())
        else:
            r64d = torch.zeros_like(res)
            run_batched(timed[:1], hg.FP64, r64d)
            stream.synchronize()
            a, b = rg[:n_first].cpu().double(), r64d[:n_first].cpu().double()
            ent["max_rel_err_vs_fp64_dense"] = (
                ((a - b).abs().max(1).values / b.abs().max(1).values.clamp_min(1e-300)).max().item())
            ent["pairs_checked"] = n_first
        generic[name] = ent
    c.set_qed_kernel(hg.QED_STANDIN)

    # ---- the learned QED weight, trained on this GPU, in the same path ------
    from hlbl_gb300.surrogate import Surrogate

    sur = Surrogate(device=local_rank, seed=3)
    t_train = time.perf_counter()
    train_rep = sur.train(n_samples=args.train_samples, batch=8192, steps=args.train_steps,
                          n_valid=1 << 18, bound=1e-4)
    train_rep["wall_seconds"] = round(time.perf_counter() - t_train, 2)
    train_rep["gain_max_err"] = train_rep["max_rel_err_base"] / max(train_rep["max_rel_err_net"], 1e-300)
    train_rep["gain_rms_err"] = train_rep["rms_rel_err_base"] / max(train_rep["rms_rel_err_net"], 1e-300)
    c.set_qed(sur)
    run_batched32(warm, res)
    c.set_qed(sur)  # fallback counter cleared: count the timed replay only
    nsur, mssur, _ = graph_timed()
    res_sur = res.clone()
    fallbacks = c.qed_fallbacks()
    c.set_qed(None)

    # ---- FP32 products with the FP64 weight everywhere -----------------------
    c.set_qed_fp32(False)
    res32x = torch.zeros_like(res)
    run_batched32(timed[:1], res32x)
    n32x, ms32x = timeit(run_batched32, timed, res32x)
    c.set_qed_fp32(True)

    # ---- plain FP64, per pair, exact weight (the reference's path) on the
    #      first fp64-steps steps; the other timed pairs untimed (batched) so
    #      every timed pair has its FP64 value --------------------------------
    f64_steps = timed[:max(1, args.fp64_steps)]
    res64 = torch.zeros_like(res)
    n64, ms64 = timeit(run_pairs, f64_steps, hg.FP64, res64)
    k = sum(len(s[1]) for s in f64_steps)
    rest = timed[len(f64_steps):]
    if rest:
        run_batched(rest, hg.FP64, res64[k:])
    stream.synchronize()
    a64 = res64[:n32].cpu().double()

    def errs(r):
        """(max per-pair error, the pair's two flavours as one vector;
        chain-total error of the timed pairs; max per-flavour error)."""
        a = r[:n32].cpu().double()
        d = (a - a64).abs()
        per_pair = (d.max(1).values / a64.abs().max(1).values.clamp_min(1e-300)).max().item()
        per_flavour = (d / a64.abs().clamp_min(1e-300)).max().item()
        chain = ((a.sum(0) - a64.sum(0)).abs() / a64.sum(0).abs()).max().item()
        return per_pair, chain, per_flavour

    rel, chain_rel, rel_fl = errs(res_main)
    rel_sur, chain_sur, rel_sur_fl = errs(res_sur)
    rel32x, chain32x, rel32x_fl = errs(res32x)
    relfb, chainfb, _ = errs(res_f64b)
    relp, _, _ = errs(res_p)

    # ---- per-kernel durations (CUDA events on the launching stream) --------
    c.set_profiling(True)
    run_batched32(timed[:1], res_b)
    stream.synchronize()
    (p1ms, p1n), (p2ms, p2n) = c.kernel_times()
    c.set_profiling(False)
    c.set_profiling(True)
    run_pairs([(timed[0][0], timed[0][1][:1])], hg.FP64, res_b)
    stream.synchronize()
    (p1ms64, p1n64), (p2ms64, p2n64) = c.kernel_times()
    c.set_profiling(False)
    n_prof = len(timed[0][1])
    g = tune["batch_group"]
    groups = [min(g, n_prof - i) for i in range(0, n_prof, g)]
    V = volume(LATTICE)
    blk = 2 * 12 * 24 * 8 * V  # bytes of one FP64 block (4,608 B/site)

    # ---- end to end through the C ABI with host buffers: each step stages
    #      its new block from pinned host memory on the side stream (the
    #      next one while this one computes) and reads its sums back ---------
    pinned = {}
    for p, _ in timed:
        site = schedule.mod_pos(p, LATTICE)
        if site not in pinned:
            h = torch.empty(c.block_length, dtype=torch.float64, pin_memory=True)
            h.copy_(block(p))
            pinned[site] = h
    host_out = torch.empty((n_timed_pairs, 2), dtype=torch.float64, pin_memory=True)

    def e2e_pass():
        h2d = d2h = 0
        # device timestamps on the compute stream: the pass's start and each
        # step's end (a step also waits there for its staged block)
        evs = [torch.cuda.Event(enable_timing=True)]
        evs[0].record(stream)
        site0 = schedule.mod_pos(timed[0][0], LATTICE)
        # each source's block has its own device buffer, idle while it is staged
        c.stage_async(block(timed[0][0]), pinned[site0], pinned[site0].numel() * 8, after_compute=False)
        h2d += pinned[site0].numel() * 8
        k = 0
        for i, st in enumerate(timed):
            pr = pairs_of(st)
            xs = [block32(q) for q, _, _, _ in pr]
            y32 = block32(st[0], make=False)
            c.f32_tile_copy(block(st[0]), y32)  # waits for the staged block
            c.kernel_sums_batched_f32(y32, xs, [g for _, _, g, _ in pr], [v for _, _, _, v in pr], xu,
                                      res[k:k + len(xs)])
            if i + 1 < len(timed):
                sn = schedule.mod_pos(timed[i + 1][0], LATTICE)
                c.stage_async(block(timed[i + 1][0]), pinned[sn], pinned[sn].numel() * 8, after_compute=False)
                h2d += pinned[sn].numel() * 8
            with torch.cuda.stream(stream):
                host_out[k:k + len(xs)].copy_(res[k:k + len(xs)], non_blocking=True)
            evs.append(torch.cuda.Event(enable_timing=True))
            evs[-1].record(stream)
            d2h += len(xs) * 16
            k += len(xs)
        enq = time.perf_counter()
        stream.synchronize()
        steps_ms = [round(a.elapsed_time(b), 1) for a, b in zip(evs[:-1], evs[1:])]
        return h2d, d2h, enq, steps_ms

    # one untimed pass first (the first copies from freshly pinned pages and
    # the first launches of this call sequence are not representative), then
    # seven timed passes: the host side of the box is shared (passes of the
    # same work have measured 45 and 139 pairs/s in one run), so the median
    # is reported and all seven are listed, each with the host time spent
    # enqueueing it (a slow pass with a short enqueue time waited on the device)
    e2e_pass()  # untimed
    # a 1 GB pinned host -> device copy just before each pass: the host link's
    # bandwidth at that moment (the machine's host side is shared)
    probe_h = torch.empty(1 << 30, dtype=torch.uint8, pin_memory=True)
    probe_d = torch.empty(1 << 30, dtype=torch.uint8, device="cuda")

    def h2d_probe():
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            probe_d.copy_(probe_h, non_blocking=True)
            e1.record(stream)
        e1.synchronize()
        return (1 << 30) / (e0.elapsed_time(e1) * 1e-3) / 1e9

    e2e_runs, e2e_enq, e2e_steps, h2d_gbs = [], [], [], []
    for _ in range(7):
        h2d_gbs.append(round(h2d_probe(), 1))
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        h2d, d2h, enq, steps_ms = e2e_pass()
        e2e_runs.append(time.perf_counter() - t0)
        e2e_enq.append(enq - t0)
        e2e_steps.append(steps_ms)
    del probe_h, probe_d
    e2e_s = statistics.median(e2e_runs)
    if dist:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())

    # ---- peaks and rooflines -------------------------------------------------
    peaks, peak_src = load_peaks()
    fp64_peak = measure_fma_peak(hg.FP64, local_rank)
    fp32_peak = measure_fma_peak(hg.FP32, local_rank)
    tf32_peak = measure_tf32_peak(torch)
    p2_avg_ms = p2ms / max(1, p2n)
    p1_avg_ms = p1ms / max(1, p1n)
    traffic = load_traffic()
    # the committed DRAM traffic is one pair's launch at 24^3 x 48 (V = 663,552);
    # the rows of the tile copies are read once, so it scales with the sites
    # and the pairs a launch covers
    def traffic_per_launch(key, launches):
        if not traffic or traffic.get(key) is None:
            return None
        return round(traffic[key] * (V / 663552) * (n_prof / max(1, launches)))
    # pass 1, per launch of g pairs: both FP64 blocks read (y once, each
    # partner once) and their FP32 tile copies written (half the bytes)
    p1_bytes = sum((1 + gi) for gi in groups) * blk * 0.5 / max(1, p1n)  # FP32 copies read
    p1_gbs = p1_bytes / (p1_avg_ms * 1e-3) / 1e9
    # pass 2, per pair: the 128 x 160 x 288 product per 32 sites per flavour
    # (FMA = 2 flops), algorithmic; the tensor cores issue 4x (FP16 operands)
    # or 3x (3xTF32)
    gemm_flop_pair = 2 * 2 * V * 4 * 288 * 160
    p2_tflops = gemm_flop_pair * n_prof / max(1, p2n) / (p2_avg_ms * 1e-3) / 1e12
    p2_bytes = sum((1 + gi) for gi in groups) * blk * 0.5 / max(1, p2n)  # FP32 tile copies read
    rl_p1 = {"bound": "hbm", "kernel": f"pass 1 on FP32 tile copies, p1f32_kernel ({tune['p1']}, batched)",
             "achieved": round(p1_gbs, 2), "peak": peaks["hbm_gbs"], "unit": "GB/s",
             "frac": round(p1_gbs / peaks["hbm_gbs"], 5),
             "traffic": traffic_per_launch("p1_bytes_per_launch", p1n),
             "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
             "kernel_ms": round(p1_avg_ms, 3), "bytes_per_launch": p1_bytes}
    # pass 2's operands are FP16 (the default: four FP16 MMAs per product,
    # hi.hi + hi.lo + lo.hi + hi.lo2) against the measured dense 16-bit GEMM
    # rate (bf16 and fp16 run at the same rate), or TF32 (three) against a
    # cuBLAS TF32 GEMM measured here
    if p2_fp16:
        p2_peak, p2_issue = peaks["bf16_tflops"], 4
        p2_peak_src = f"{peak_src} (MEASURED_PEAKS.json bf16_tflops: dense 16-bit GEMM, burst; FP16 operands)"
    else:
        p2_peak, p2_issue = tf32_peak, 3
        p2_peak_src = "measured here: cuBLAS TF32 GEMM 8192^3 (torch.matmul, allow_tf32); TF32 operands"
    rl_p2 = {"bound": "tensor", "kernel": f"pass 2, {tune['p2']}, {'FP16' if p2_fp16 else 'TF32'} operands (batched)",
             "achieved": round(p2_tflops, 2), "peak": round(p2_peak, 1), "unit": "TFLOP/s",
             "frac": round(p2_tflops / p2_peak, 5),
             "traffic": traffic_per_launch("p2_bytes_per_launch", p2n),
             "peak_source": p2_peak_src,
             "issued_tflops": round(p2_issue * p2_tflops, 2), "issued_per_product": p2_issue,
             "tf32_gemm_tflops_measured": round(tf32_peak, 1), "kernel_ms": round(p2_avg_ms, 3),
             "hbm_gbs": round(p2_bytes / (p2_avg_ms * 1e-3) / 1e9, 2)}
    dominant = rl_p1 if p1_avg_ms >= p2_avg_ms else rl_p2

    pairs_total = n32 * world
    value = pairs_total / (ms32 * 1e-3)
    out = {
        "metric": METRIC,
        "value": round(value, 4),
        "unit": "pairs/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms32 / max(1, len(timed)), 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32 products, fp64 sums",
        "data": "synthetic: seeded i.i.d. complex Gaussian FP64 propagator blocks, generated on the device",
        "config": {"workload": workload(),
                   "lattice": list(LATTICE), "pairs_timed": n32,
                   "path": "batched per source (autotuned), one CUDA graph for the timed sources; "
                           "blocks as FP32 tile copies (each new block converted once, in its step); "
                           + ("FP32 products (pass 2 on the tensor cores, FP16 operands split hi/lo with power-of-two "
                              "scales), FP64 sums" if p2_fp16
                              else "FP32 products (pass 2 on the tensor cores, 3xTF32), FP64 sums"),
                   "qed_weight": "stand-in (KQED unavailable), exact: FP32 quadrature, FP64 within "
                                 "0.1/m_mu of the origin; the learned weight is the 'surrogate' line",
                   "l2": "inputs 3.06 GB per block, larger than L2; no flush"},
        "max_rel_err_vs_fp64": rel,
        "max_rel_err_per_flavour_vs_fp64": rel_fl,
        "chain_total_rel_err_vs_fp64": chain_rel,
        "fp64": {"value": round(n64 / (ms64 * 1e-3), 4), "unit": "pairs/s", "pairs_timed": n64,
                 "path": "per pair, FP64 products, exact FP64 weight (the reference's algorithm)",
                 "p2_kernel_ms": round(p2ms64 / max(1, p2n64), 3),
                 "p1_kernel_ms": round(p1ms64 / max(1, p1n64), 3),
                 "fp64_fma_peak_tflops": round(fp64_peak, 3),
                 "p2_fp64_tflops": round(gemm_flop_pair / (p2ms64 / max(1, p2n64) * 1e-3) / 1e12, 4)},
        "speedup_vs_fp64": round(value / (n64 / (ms64 * 1e-3)), 2),
        "surrogate": {"value": round(nsur / (mssur * 1e-3), 4), "unit": "pairs/s",
                      "path": "the headline path with the MLP weight (the exact weight outside its validated region: FP32 quadrature, FP64 within 0.1/m_mu of the origin)",
                      "max_rel_err_vs_fp64": rel_sur, "chain_total_rel_err_vs_fp64": chain_sur,
                      "max_rel_err_per_flavour_vs_fp64": rel_sur_fl,
                      "train": train_rep, "fallback_rows_timed": fallbacks,
                      "rows_timed": nsur * 3 * V},
        "fp32_fp64_weight": {"value": round(n32x / (ms32x * 1e-3), 4), "unit": "pairs/s",
                             "path": "batched, no graph, FP64 QED weight everywhere",
                             "max_rel_err_vs_fp64": rel32x, "chain_total_rel_err_vs_fp64": chain32x,
                             "max_rel_err_per_flavour_vs_fp64": rel32x_fl},
        "batched_no_graph": {"value": round(nb_ / (msb * 1e-3), 4), "unit": "pairs/s"},
        "batched_fp64_blocks": {"value": round(nfb / (msfb * 1e-3), 4), "unit": "pairs/s",
                                "path": "hlbl_kernel_sums_batched on the FP64 blocks, no graph (pass 1 "
                                        "converts and writes the FP32 tile copies for every pair)",
                                "max_rel_err_vs_fp64": relfb, "chain_total_rel_err_vs_fp64": chainfb,
                                "autotune": tune64},
        "per_pair": {"value": round(npp / (mspp * 1e-3), 4), "unit": "pairs/s", "max_rel_err_vs_fp64": relp},
        "generic_qed": dict(generic, path="the headline path (graph, FP32 copies, tensor cores) with the QED "
                                          "weighting from the generic coefficient stage: 640 FP32 coefficients "
                                          "per site in HBM, dotted with F by pass 2's generic epilogue; "
                                          "'dense' is a test tensor with no index structure"),
        "autotune": tune,
        "e2e": {"value": round(pairs_total / e2e_s, 4), "unit": "pairs/s",
                "h2d_bytes_per_step": int(h2d / max(1, len(timed))),
                "d2h_bytes_per_step": int(d2h / max(1, len(timed))),
                "passes_pairs_per_s": [round(pairs_total / t, 2) for t in e2e_runs],
                "passes_enqueue_ms": [round(1e3 * t, 1) for t in e2e_enq],
                "passes_step_ms": e2e_steps,
                "h2d_probe_gbs_before_each_pass": h2d_gbs,
                "how": "median of seven passes over the timed steps after one untimed pass; each "
                       "step stages its new block from pinned host memory on the side stream while "
                       "the previous step computes"},
        "roofline": dominant,
        "rooflines": {"pass1": rl_p1, "pass2": rl_p2,
                      "fp32_fma_peak_tflops": round(fp32_peak, 2),
                      "fma_peak_source": "measured here (FMA-chain kernel, hlbl_measure_fma_peak)"},
        "clocks": clk,
        # per step: the new block's conversion, then per pair group pass 1,
        # its reduction, the gamma insertion, the B operand, the weights,
        # pass 2 and its reduction
        "gpu_launches": sum(1 + 7 * len(range(0, len(s[1]), tune["batch_group"])) for s in timed),
    }

    # ---- all 16 h directions as 16 chains over one cache (the reference's
    #      run_chains, driver.cpp:169-208), batched per source on FP32 copies,
    #      one CUDA graph per window -------------------------------------------
    if not args.no_chains16:
        out["chains16"] = bench_chains16(c, hg, torch, xu, res64_pairs=4)

    # ---- the 2+2 pieces of the first timed source (compute_2p2_gpu) ---------
    if rank == 0:
        p0 = timed[0][0]
        gsw = schedule.mod_pos(p0, LATTICE)
        out["pieces_2p2"] = bench_2p2(c, hg, torch, stream, block(p0), block32(p0), gsw, xu,
                                      max(3, args.steps))
        if not args.no_cpu_baseline:
            sec22, cores22 = cpu_2p2_seconds(block(p0).cpu().numpy(), gsw, xu)
            out["pieces_2p2"]["cpu_baseline"] = {
                "value": round(sec22 * 1e3, 1), "unit": "ms per source", "cores": cores22, "kind": "port",
                "sample": f"the oracle (FP64, OpenMP): Pi and P1 once plus P2_0..P4_1 of one target, "
                          f"the target part scaled by {N_TARGETS_2P2}"}

    if rank == 0 and not args.no_cpu_baseline:
        p, qs = timed[0]
        q = qs[0]
        gx = schedule.mod_pos(q, LATTICE)
        yv = schedule.site_map_diff(p, q, LATTICE)
        src_h = block(q).cpu().numpy()
        y_h = block(p).cpu().numpy()
        ns = pick_slices(src_h, y_h, gx, yv, xu, args.cpu_seconds)
        sec, cores = cpu_pair_seconds(src_h, y_h, gx, yv, xu, ns)
        out["cpu_baseline"] = {"value": round(1.0 / sec, 6), "unit": "pairs/s", "cores": cores,
                               "kind": "port",
                               "sample": f"one pair, pass 1 + pass 2 both flavours over {ns} of 48 "
                                         f"time slices, scaled by 48/{ns}; plain FP64 loops of the "
                                         f"reference restated in C (oracle), OpenMP"}
    if rank == 0 and not args.no_reference_gpu:
        p, qs = timed[0]
        q = qs[0]
        out["reference_gpu_baseline"] = reference_gpu_baseline(
            torch, c, hg, block(q), block(p), schedule.mod_pos(q, LATTICE), schedule.site_map_diff(p, q, LATTICE),
            xu, res64[0].cpu().tolist(), res_main[0].cpu().tolist(), schedule.mod_pos(p, LATTICE))
    if rank == 0:
        print(json.dumps(ordered(out)), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def ordered(out):
    """The contract's keys first, then a compact summary of every line (so a
    reader of a truncated line still has them), then the details."""
    def g(*path):
        v = out
        for k in path:
            if not isinstance(v, dict) or k not in v:
                return None
            v = v[k]
        return v

    summary = {
        "headline_pairs_per_s": g("value"), "e2e_pairs_per_s": g("e2e", "value"),
        "max_rel_err_vs_fp64": g("max_rel_err_vs_fp64"), "chain_total_rel_err_vs_fp64": g("chain_total_rel_err_vs_fp64"),
        "fp64_pairs_per_s": g("fp64", "value"),
        "reference_gpu_pairs_per_s": g("reference_gpu_baseline", "kernel_sum", "value"),
        "cpu_port_pairs_per_s": g("cpu_baseline", "value"),
        "surrogate": {"pairs_per_s": g("surrogate", "value"), "max_rel_err": g("surrogate", "max_rel_err_vs_fp64"),
                      "chain_total_rel_err": g("surrogate", "chain_total_rel_err_vs_fp64")},
        "generic_dense_pairs_per_s": g("generic_qed", "dense", "value"),
        "chains16_pairs_per_s": g("chains16", "value"),
        "pieces_2p2_ms_per_source": g("pieces_2p2", "value"),
        "reference_gpu_2p2_ms_per_source": g("reference_gpu_baseline", "pieces_2p2", "value"),
        "pass1_ms": g("rooflines", "pass1", "kernel_ms"), "pass2_ms": g("rooflines", "pass2", "kernel_ms"),
    }
    first = ["metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
             "vs_baseline", "dtype", "data", "config", "e2e", "roofline", "cpu_baseline", "clocks", "gpu_launches"]
    res = {k: out[k] for k in first if k in out}
    res["summary"] = summary
    res.update({k: v for k, v in out.items() if k not in res})
    return res


def bench_chains16(c, hg, torch, xu, res64_pairs):
    """The 24^3x48 configuration with every h in {+1,-1}^4 as its own chain
    (stride 2, K = 4: 16 x 275 pairs), run by the library's driver over one
    device cache of FP32 tile copies: solves (device fixtures), conversion as
    each block is stored, one batched FP32-copy call per new source, one CUDA
    graph per window, results read back per window. The solves stand in for
    the reference's solver (a 3 GB Gaussian fixture per solve, Box-Muller in
    FP64), so their time is measured on its own and reported apart; a few
    pairs are recomputed by the FP64 path for their error."""
    from hlbl_gb300 import schedule
    from hlbl_gb300.cache import PropagatorCache, TorchBuffers
    from hlbl_gb300.driver import run_chains

    hs = schedule.sign_vectors()
    chains = [schedule.build_schedule(h, STRIDE, NSTEPS) for h in hs]
    cache = PropagatorCache("device32", c.block_length, TorchBuffers(c))

    def provider(site, dest):
        c.fill_gaussian_block(dest, hg.Contractor.source_seed(RUN_SEED, site))

    def out_factory(n):
        return torch.zeros((n, 2), dtype=torch.float64, device="cuda")

    scratch = torch.empty(c.block_length, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(3):
        provider((i, 0, 0, 0), scratch)
    torch.cuda.synchronize()
    t_fill = (time.perf_counter() - t0) / 3
    del scratch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res, st, _ = run_chains(chains, LATTICE, xu, provider, c, cache, batched=True, graphs=True,
                            out_factory=out_factory)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    t_solves = t_fill * st.positions_solved
    per_chain = [sum(1 for r in res if r.chain == i) for i in range(len(chains))]
    # FP64 recomputation of the first pair of a few chains
    errs = []
    a = torch.empty(c.block_length, dtype=torch.float64, device="cuda")
    b = torch.empty(c.block_length, dtype=torch.float64, device="cuda")
    picks = [next(r for r in res if r.chain == i) for i in range(0, len(chains), max(1, len(chains) // res64_pairs))]
    for r in picks[:res64_pairs]:
        provider(tuple(r.x), a)
        provider(tuple(r.y), b)
        ks = c.kernel_sum(a, b, r.x, r.yv, xu, hg.FP64)
        errs.append(max(abs(r.kernel_sum[f] - ks[f]) for f in (0, 1)) / max(abs(ks[0]), abs(ks[1])))
    del a, b
    return {"value": round(len(res) / (dt - t_solves), 3), "unit": "pairs/s",
            "how": "pairs / (wall time of the run - the solves' fixture generation)",
            "with_solves": round(len(res) / dt, 3), "fixture_seconds_per_solve": round(t_fill, 4),
            "pairs": len(res), "seconds": round(dt, 2),
            "chains": len(chains), "pairs_per_chain": sorted(set(per_chain)),
            "positions_solved": st.positions_solved, "cache_peak": st.cache_peak,
            "max_rel_err_vs_fp64_sampled": max(errs) if errs else None, "pairs_checked_fp64": len(errs),
            "path": "library driver (run_chains) over a device cache of FP32 tile copies; per window the "
                    "solves (device fixtures) and conversions, then one batched FP32-copy call per new "
                    "source recorded as one CUDA graph; results read back per window"}


def reference_gpu_baseline(torch, c, hg, d_src, d_y, gsx, yv, xu, ours64, ours32, gsw):
    """Baseline leg: the reference's OWN Contractor and kernels
    (kernels/cuda_lattice.cu, kernels/hlbl_kernels/kernels.cu, src/contract.cpp),
    built for sm_103a by the committed recipe oracle/ref_gpu with the stand-in
    QED weight on the device, timed on this GPU: one pair (both flavours,
    Contractor::kernel_sum, which blocks on its host round trips) and one
    source's 2+2 pieces for the same targets as the pieces_2p2 line. The
    library's results for the same inputs are compared with it."""
    import platform

    import numpy as np

    path = os.path.join(ROOT, "oracle", "_ref", "gpu", platform.machine(), "libhlbl_ref_gpu.so")
    if not os.path.exists(path):
        return {"unavailable": "the reference's GPU build (oracle/_ref/gpu) is absent: no staged copy of its sources"}
    lib = C.CDLL(path)
    I4 = C.c_int * 4
    vpt = C.c_void_p
    lib.refgpu_last_error.restype = C.c_char_p
    lib.refgpu_create.argtypes = [C.POINTER(vpt), I4, C.c_int, C.c_ulonglong]
    lib.refgpu_destroy.argtypes = [vpt]
    lib.refgpu_kernel_sum.argtypes = [vpt, vpt, vpt, I4, I4, C.c_double, vpt]
    lib.refgpu_pieces_2p2.argtypes = [vpt, vpt, I4, vpt, C.c_int, C.c_double, vpt, vpt]
    lib.refgpu_reserve_kernel_memory.argtypes = [vpt, C.c_int, C.POINTER(C.c_size_t)]
    h = vpt()
    if lib.refgpu_create(C.byref(h), I4(*LATTICE), 0, 0) != 0:
        return {"unavailable": "refgpu_create: " + lib.refgpu_last_error().decode()}
    try:
        nb = C.c_size_t()
        torch.cuda.synchronize()
        # the reference's own preflight: the first launches reserve the kernels' stack
        if lib.refgpu_reserve_kernel_memory(h, 1, C.byref(nb)) != 0:
            return {"unavailable": "reserve_kernel_memory: " + lib.refgpu_last_error().decode()}
        ks = (C.c_double * 2)()
        t0 = time.perf_counter()
        rc = lib.refgpu_kernel_sum(h, vpt(d_src.data_ptr()), vpt(d_y.data_ptr()), I4(*gsx), I4(*yv),
                                   C.c_double(xu), ks)
        t_pair = time.perf_counter() - t0
        if rc != 0:
            return {"unavailable": "kernel_sum: " + lib.refgpu_last_error().decode()}
        ref = np.array([ks[0], ks[1]])
        targets = targets_2p2(gsw, N_TARGETS_2P2)
        tg = np.ascontiguousarray(np.asarray(targets, dtype=np.int32))
        p1 = np.zeros(64 * max(LATTICE))
        p234 = np.zeros(N_TARGETS_2P2 * 320)
        t0 = time.perf_counter()
        rc = lib.refgpu_pieces_2p2(h, vpt(d_y.data_ptr()), I4(*gsw), tg.ctypes.data_as(vpt), len(targets),
                                   C.c_double(xu), p1.ctypes.data_as(vpt), p234.ctypes.data_as(vpt))
        t_2p2 = time.perf_counter() - t0
        res = {"kernel_sum": {"value": round(1.0 / t_pair, 4), "unit": "pairs/s", "seconds_per_pair": round(t_pair, 3),
                              "reference_sums": ref.tolist(),
                              "fp64_rel_err_vs_reference": float(np.max(np.abs(np.asarray(ours64) - ref) / np.abs(ref))),
                              "headline_fp32_rel_err_vs_reference":
                                  float(np.max(np.abs(np.asarray(ours32) - ref)) / np.max(np.abs(ref)))},
               "kernel_memory_reserved_bytes": int(nb.value),
               "what": "the reference's Contractor::kernel_sum and Contractor::pieces_2p2 driving its own "
                       "kernels, built for sm_103a (oracle/ref_gpu), stand-in QED weight on the device; "
                       "one pair of the first timed step (wall time of the blocking call)"}
        if rc == 0:
            ours = c.pieces_2p2(d_y, gsw, targets, xu, hg.FP64)
            a = np.asarray(ours.p234).reshape(-1, 5, 64)
            b = p234.reshape(-1, 5, 64)
            err = max(float(np.abs(a[t, g] - b[t, g]).max() / max(np.abs(b[t, g]).max(), 1e-300))
                      for t in range(b.shape[0]) for g in range(5))
            res["pieces_2p2"] = {"value": round(t_2p2 * 1e3, 1), "unit": "ms per source",
                                 "targets": N_TARGETS_2P2, "fp64_max_row_rel_err_vs_reference": err}
        else:
            res["pieces_2p2"] = {"unavailable": lib.refgpu_last_error().decode()}
        return res
    finally:
        lib.refgpu_destroy(h)


N_TARGETS_2P2 = 16  # the README's 2+2 timing is quoted per 16 targets


def targets_2p2(gsw, n):
    """n distinct target sites around the source gsw, seeded."""
    import numpy as np

    rng = np.random.default_rng(2025)
    out = []
    while len(out) < n:
        t = [int(rng.integers(0, L)) for L in LATTICE]
        if t not in out and t != list(gsw):
            out.append(t)
    return out


def bench_2p2(c, hg, torch, stream, fwd, x32, gsw, xu, reps):
    """The 2+2 pieces of one source for N_TARGETS_2P2 targets
    (compute_2p2_gpu), timed with CUDA events on the context's stream."""
    import numpy as np

    targets = targets_2p2(gsw, N_TARGETS_2P2)
    d1 = torch.zeros(64 * c.lmax, dtype=torch.float64, device="cuda")
    d234 = torch.zeros(N_TARGETS_2P2 * 320, dtype=torch.float64, device="cuda")
    c.reserve_2p2()

    def timed(fn, n):
        fn()
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            fn()
        e1.record(stream)
        e1.synchronize()
        c.check()
        return e0.elapsed_time(e1) / n, d1.cpu().numpy().copy(), d234.cpu().numpy().copy()

    ms_copy, p1c, p234c = timed(lambda: c.pieces_2p2_f32(x32, gsw, targets, xu, d1, d234), reps)
    ms_blk, p1b, p234b = timed(lambda: c.pieces_2p2_async(fwd, gsw, targets, xu, d1, d234, hg.FP32), reps)
    ms64, p1d, p234d = timed(lambda: c.pieces_2p2_async(fwd, gsw, targets, xu, d1, d234, hg.FP64), 1)

    def row_err(a, b):
        a, b = a.reshape(-1, 5, 64), b.reshape(-1, 5, 64)
        return float(max(np.abs(a[t, g] - b[t, g]).max() / np.abs(b[t, g]).max()
                         for t in range(a.shape[0]) for g in range(5)))

    V = volume(LATTICE)
    evals = 4 * N_TARGETS_2P2 * V
    return {"value": round(ms_copy, 3), "unit": "ms per source", "targets": N_TARGETS_2P2,
            "path": "hlbl_pieces_2p2_f32: Pi from the source's FP32 tile copy, FP32 products and "
                    "QED weight (stand-in, FP32 quadrature), FP64 sums over CTAs",
            "qed_evaluations_per_s": round(evals / (ms_copy * 1e-3), 1),
            "fp32_from_fp64_block_ms": round(ms_blk, 3),
            "fp64_ms": round(ms64, 3),
            "speedup_vs_fp64": round(ms64 / ms_copy, 2),
            "max_row_rel_err_p234_vs_fp64": row_err(p234c, p234d),
            "max_rel_err_p1_vs_fp64": float(np.abs(p1c - p1d).max() / np.abs(p1d).max()),
            "fp32_paths_identical": bool(np.array_equal(p234c, p234b) and np.array_equal(p1c, p1b)),
            "gpu_launches_per_source": 3 + 5 * ((N_TARGETS_2P2 + 31) // 32),
            "reference_readme": "compute_2p2_gpu 4.6 s per 16 targets, one GH200, 262,144 sites, "
                                "real KQED (not comparable weight)"}


def run_config2_chain(args, hg, torch, rank):
    """The whole 24^3x48 chain (stride 2, h = (+1,-1,+1,-1), K = 4: 76
    propagators, 275 pairs) through the library's driver twice: the headline
    path (FP32 tile copies, batched, a graph per window) and the FP64 path pair
    by pair (the reference's algorithm and loop); every pair's error and the
    chain totals. Then a sample of pairs by the reference's own kernels built
    for sm_103a (oracle/ref_gpu, a baseline leg) against the FP64 path."""
    import platform

    import numpy as np

    from hlbl_gb300 import schedule
    from hlbl_gb300.cache import PropagatorCache, TorchBuffers
    from hlbl_gb300.driver import run_chain

    if rank != 0:
        return 0
    xu = hg.xunit(MUON_MEV, SPACING_FM)
    steps = schedule.build_schedule(H, STRIDE, NSTEPS)
    c = hg.Contractor(LATTICE)
    stream = torch.cuda.Stream()
    c.set_stream(stream)

    def provider(site, dest):
        c.fill_gaussian_block(dest, hg.Contractor.source_seed(RUN_SEED, site))

    def out_factory(n):
        return torch.zeros((n, 2), dtype=torch.float64, device="cuda")

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r32, st32 = run_chain(steps, LATTICE, xu, provider, c, PropagatorCache("device32", c.block_length, TorchBuffers(c)),
                          batched=True, graphs=True, out_factory=out_factory)
    torch.cuda.synchronize()
    t32 = time.perf_counter() - t0
    t0 = time.perf_counter()
    r64, st64 = run_chain(steps, LATTICE, xu, provider, c, PropagatorCache("device", c.block_length, TorchBuffers(c)),
                          precision=hg.FP64)
    torch.cuda.synchronize()
    t64 = time.perf_counter() - t0
    ref = {(r.x, r.y): np.array(r.kernel_sum) for r in r64}
    per_pair = [float(np.max(np.abs(np.array(r.kernel_sum) - ref[(r.x, r.y)])) / np.max(np.abs(ref[(r.x, r.y)])))
                for r in r32]
    tot32 = np.sum([r.kernel_sum for r in r32], axis=0)
    tot64 = np.sum([r.kernel_sum for r in r64], axis=0)
    scale = np.sum([np.abs(r.kernel_sum) for r in r64], axis=0)
    out = {"metric": "the 24^3x48 chain (275 pairs): FP32 headline path against FP64, every pair",
           "pairs": len(r32), "pairs_fp64": len(r64), "propagators": st32.positions_solved,
           "fp32_path_seconds": round(t32, 2), "fp64_path_seconds": round(t64, 2),
           "max_rel_err_per_pair": max(per_pair), "median_rel_err_per_pair": float(np.median(per_pair)),
           "chain_total_rel_err": float(np.max(np.abs(tot32 - tot64) / np.abs(tot64))),
           "chain_total_err_at_chain_scale": float(np.max(np.abs(tot32 - tot64) / scale)),
           "chain_totals_fp64": tot64.tolist()}
    path = os.path.join(ROOT, "oracle", "_ref", "gpu", platform.machine(), "libhlbl_ref_gpu.so")
    if os.path.exists(path) and args.c2_ref_pairs > 0:
        lib = C.CDLL(path)
        I4 = C.c_int * 4
        vpt = C.c_void_p
        lib.refgpu_last_error.restype = C.c_char_p
        lib.refgpu_create.argtypes = [C.POINTER(vpt), I4, C.c_int, C.c_ulonglong]
        lib.refgpu_destroy.argtypes = [vpt]
        lib.refgpu_kernel_sum.argtypes = [vpt, vpt, vpt, I4, I4, C.c_double, vpt]
        lib.refgpu_reserve_kernel_memory.argtypes = [vpt, C.c_int, C.POINTER(C.c_size_t)]
        h = vpt()
        assert lib.refgpu_create(C.byref(h), I4(*LATTICE), 0, 0) == 0, lib.refgpu_last_error()
        nb = C.c_size_t()
        assert lib.refgpu_reserve_kernel_memory(h, 1, C.byref(nb)) == 0, lib.refgpu_last_error()
        a = torch.empty(c.block_length, dtype=torch.float64, device="cuda")
        b = torch.empty(c.block_length, dtype=torch.float64, device="cuda")
        errs, secs = [], []
        for r in r64[:args.c2_ref_pairs]:
            provider(tuple(r.x), a)
            provider(tuple(r.y), b)
            stream.synchronize()
            ks = (C.c_double * 2)()
            t0 = time.perf_counter()
            assert lib.refgpu_kernel_sum(h, vpt(a.data_ptr()), vpt(b.data_ptr()), I4(*r.x), I4(*r.yv),
                                         C.c_double(xu), ks) == 0
            secs.append(time.perf_counter() - t0)
            errs.append(float(np.max(np.abs(np.array(r.kernel_sum) - np.array([ks[0], ks[1]])) /
                                     np.abs(np.array([ks[0], ks[1]])))))
        lib.refgpu_destroy(h)
        out["reference_gpu_sample"] = {"pairs": len(errs), "fp64_max_rel_err_vs_reference_kernels": max(errs),
                                       "reference_seconds_per_pair": round(float(np.mean(secs)), 3)}
    print(json.dumps(out), flush=True)
    return 0


def run_config5(args, hg, torch, rank):
    """The 48^3 x 96 configuration (V = 10,616,832; a 49 GB FP64 block, a
    24.5 GB FP32 tile copy) with a host-resident cache: stride 4,
    h = (-1,+1,+1,+1), K = 8, one source of window 1 and `c5_partners` of its
    partners. The partners' blocks are solved (device fixtures), converted to
    FP32 tile copies and stored in pinned host memory; in the timed loop each
    partner's copy streams into one of two device slots on a copy stream while
    the previous pair computes (one FP32-copy kernel-sum call per pair), so
    a pair costs max(copy, compute). Reported: pairs/s overlapped and with
    copy and compute in sequence, the host-to-device GB/s, and the first
    pair's error against the FP64 path. The GPU machine's host has 199 GB, so
    the reference's cache of FP64 blocks (16 live 49 GB blocks) cannot exist
    there; the host cache holds FP32 copies."""
    from hlbl_gb300 import schedule

    if rank != 0:
        return 0
    lat = (96, 48, 48, 48)
    h, stride, K = (-1, 1, 1, 1), 4, 8
    xu = hg.xunit(MUON_MEV, SPACING_FM)
    st = schedule.build_schedule(h, stride, K)
    src = next(s_ for s_ in st[1].sources if len(s_.partners) >= args.c5_partners)
    p = src.position
    qs = list(src.partners)[:args.c5_partners]
    c = hg.Contractor(lat)
    stream = torch.cuda.Stream()
    copy_stream = torch.cuda.Stream()
    c.set_stream(stream)
    n32 = c.f32_block_length
    site = lambda q: schedule.mod_pos(q, lat)  # noqa: E731
    seed = lambda q: hg.Contractor.source_seed(RUN_SEED, site(q))  # noqa: E731
    t0 = time.perf_counter()
    scratch = torch.empty(c.block_length, dtype=torch.float64, device="cuda")
    y32 = torch.empty(n32, dtype=torch.float32, device="cuda")
    slots = [torch.empty(n32, dtype=torch.float32, device="cuda") for _ in range(2)]
    host = []
    with torch.cuda.stream(stream):
        for q in qs:
            c.fill_gaussian_block(scratch, seed(q))
            c.f32_tile_copy(scratch, slots[0])
            hq = torch.empty(n32, dtype=torch.float32, pin_memory=True)
            hq.copy_(slots[0])
            host.append(hq)
        c.fill_gaussian_block(scratch, seed(p))
        c.f32_tile_copy(scratch, y32)
    stream.synchronize()
    del scratch
    t_setup = time.perf_counter() - t0
    out = torch.zeros((len(qs), 2), dtype=torch.float64, device="cuda")
    gsx = [site(q) for q in qs]
    yvs = [schedule.site_map_diff(p, q, lat) for q in qs]

    def one_pass():
        """Copy i goes to slot i % 2 on the copy stream once pair i - 2 (the
        slot's last reader) is done; pair i computes once copy i landed."""
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        staged = [torch.cuda.Event() for _ in qs]
        done = [torch.cuda.Event() for _ in qs]
        copy_ev = []
        torch.cuda.synchronize()
        ev0.record(stream)
        copy_stream.wait_stream(stream)

        def copy(i):
            if i >= 2:
                copy_stream.wait_event(done[i - 2])
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(copy_stream):
                e0.record(copy_stream)
                slots[i % 2].copy_(host[i], non_blocking=True)
                e1.record(copy_stream)
                staged[i].record(copy_stream)
            copy_ev.append((e0, e1))

        copy(0)
        for i in range(len(qs)):
            if i + 1 < len(qs):
                copy(i + 1)
            stream.wait_event(staged[i])
            c.kernel_sums_batched_f32(y32, [slots[i % 2]], [gsx[i]], [yvs[i]], xu, out[i:i + 1])
            done[i].record(stream)
        ev1.record(stream)
        torch.cuda.synchronize()
        gbs = [n32 * 4 / (a.elapsed_time(b) * 1e-3) / 1e9 for a, b in copy_ev]
        return ev0.elapsed_time(ev1), gbs

    one_pass()  # untimed: first launches at this size
    ms_ov, gbs_ov = one_pass()
    res32 = out.cpu().numpy().copy()
    # copies and computes in sequence: the reference's order (it copies
    # synchronously before each pair, propagator_cache.cpp:52-68)
    c.check()
    ms_seq, gbs_seq = [], []
    for i in range(len(qs)):
        torch.cuda.synchronize()
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        with torch.cuda.stream(stream):
            e0.record(stream)
            slots[0].copy_(host[i], non_blocking=True)
            e1.record(stream)
            c.kernel_sums_batched_f32(y32, [slots[0]], [gsx[i]], [yvs[i]], xu, out[i:i + 1])
            e2.record(stream)
        e2.synchronize()
        ms_seq.append(e0.elapsed_time(e2))
        gbs_seq.append(n32 * 4 / (e0.elapsed_time(e1) * 1e-3) / 1e9)
    del slots, y32
    torch.cuda.synchronize()
    # the first pair by the FP64 path on the FP64 blocks
    x64 = torch.empty(c.block_length, dtype=torch.float64, device="cuda")
    y64 = torch.empty(c.block_length, dtype=torch.float64, device="cuda")
    with torch.cuda.stream(stream):
        c.fill_gaussian_block(x64, seed(qs[0]))
        c.fill_gaussian_block(y64, seed(p))
    stream.synchronize()
    t0 = time.perf_counter()
    f64 = c.kernel_sum(x64, y64, gsx[0], yvs[0], xu, hg.FP64)
    t64 = time.perf_counter() - t0
    err = max(abs(res32[0][f] - f64[f]) for f in (0, 1)) / max(abs(f64[0]), abs(f64[1]))
    r = {"metric": "pairs/s at 48^3x96 with a host-resident cache (FP32 tile copies staged per pair)",
         "value": round(len(qs) / (ms_ov * 1e-3), 3), "unit": "pairs/s", "pairs": len(qs),
         "lattice": list(lat), "h": list(h), "stride": stride, "K": K,
         "source": list(site(p)), "partners": [list(site(q)) for q in qs],
         "sequential_pairs_per_s": round(len(qs) / (sum(ms_seq) * 1e-3), 3),
         "h2d_gbs_overlapped": [round(g, 1) for g in gbs_ov], "h2d_gbs_sequential": [round(g, 1) for g in gbs_seq],
         "bytes_staged_per_pair": n32 * 4, "setup_seconds": round(t_setup, 1),
         "fp64_seconds_per_pair": round(t64, 2), "fp32_rel_err_vs_fp64_first_pair": err,
         "path": "FP32 tile copies in pinned host memory, two device slots, copy stream overlapped with the "
                 "FP32-copy kernel sums (tensor-core pass 2)"}
    print(json.dumps(r), flush=True)
    return 0


def run_2p2_only(args, hg, torch, rank):
    """The 2+2 line alone: one source's Gaussian block, its FP32 tile copy,
    N_TARGETS_2P2 targets (profiling runs)."""
    from hlbl_gb300 import schedule

    if rank != 0:
        return 0
    xu = hg.xunit(MUON_MEV, SPACING_FM)
    c = hg.Contractor(LATTICE)
    stream = torch.cuda.Stream()
    c.set_stream(stream)
    gsw = schedule.mod_pos((1, 2, 3, 4), LATTICE)
    blk = torch.empty(c.block_length, dtype=torch.float64, device="cuda")
    x32 = torch.empty(c.f32_block_length, dtype=torch.float32, device="cuda")
    c.fill_gaussian_block(blk, hg.Contractor.source_seed(RUN_SEED, gsw))
    c.f32_tile_copy(blk, x32)
    r = bench_2p2(c, hg, torch, stream, blk, x32, gsw, xu, max(3, args.steps))
    r["lattice"] = list(LATTICE)
    print(json.dumps(r), flush=True)
    c.close()
    return 0


def cpu_2p2_seconds(fwd_h, gsw, xu):
    """The oracle's 2+2 (FP64, OpenMP) for one source: Pi + P1 once and P234
    of one target, scaled to N_TARGETS_2P2 targets."""
    import ctypes as C

    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import support as S

    o = S.oracle()
    V = volume(LATTICE)
    tg = np.ascontiguousarray(np.asarray(targets_2p2(gsw, 1), dtype=np.int32))
    pi = np.zeros(V * 16)
    p1 = np.zeros(64 * max(LATTICE))
    p234 = np.zeros(320)
    z = S.i4([0, 0, 0, 0])
    o.oracle_set_compensated(0)  # the reference's plain loops
    t0 = time.perf_counter()
    o.oracle_pi(S.vp(fwd_h), V, 0, S.vp(pi))
    o.oracle_p1_2p2(S.vp(pi), S.i4(LATTICE), S.i4(LATTICE), z, S.i4(gsw), max(LATTICE), S.vp(p1))
    t1 = time.perf_counter()
    o.oracle_p234(S.vp(pi), S.i4(LATTICE), S.i4(LATTICE), z, S.i4(gsw), S.vp(tg), 1, C.c_double(xu),
                  C.c_double(0.4), S.vp(p234))
    t2 = time.perf_counter()
    o.oracle_set_compensated(1)
    return (t1 - t0) + N_TARGETS_2P2 * (t2 - t1), int(o.oracle_get_threads())


def run_reference(args, rank, world):
    """The reference arm: the reference's contraction loops on the host cores
    (the oracle port; the reference has no CPU implementation of its own and
    its CUDA kernels need KQED), on the same workload, metric and unit."""
    if rank != 0:
        return 0
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import support as S
    from hlbl_gb300 import schedule

    xu = MUON_MEV / 197.3269804 * SPACING_FM
    steps_all = window_steps()
    p, qs = steps_all[0]
    q = qs[0]
    gx = schedule.mod_pos(q, LATTICE)
    yv = schedule.site_map_diff(p, q, LATTICE)
    src_h = S.gaussian_block(LATTICE, S.source_seed(RUN_SEED, schedule.mod_pos(q, LATTICE)))
    y_h = S.gaussian_block(LATTICE, S.source_seed(RUN_SEED, schedule.mod_pos(p, LATTICE)))
    budget = max(2.0, 120.0 / max(1, args.steps + args.warmup))
    ns = pick_slices(src_h, y_h, gx, yv, xu, budget)
    for _ in range(args.warmup):
        cpu_pair_seconds(src_h, y_h, gx, yv, xu, 1)
    secs = []
    cores = 1
    for _ in range(args.steps):
        s, cores = cpu_pair_seconds(src_h, y_h, gx, yv, xu, ns)
        secs.append(s)
    sec = statistics.mean(secs)
    v = 1.0 / sec
    sample = (f"per step: one pair, pass 1 + pass 2 both flavours over {ns} of 48 time slices, "
              f"scaled by 48/{ns}")
    print(json.dumps({
        "metric": METRIC, "value": round(v, 6), "unit": "pairs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(sec * 1e3 * ns / 48, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded i.i.d. complex Gaussian FP64 propagator blocks",
        "config": {"workload": workload(), "lattice": list(LATTICE)},
        "impl": "reference",
        "cpu_baseline": {"value": round(v, 6), "unit": "pairs/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(v, 6), "unit": "pairs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
