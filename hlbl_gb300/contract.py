"""The Contractor: hlbl::Contractor's interface (include/hlbl/contract.hpp:42-94
of the reference) over the C ABI of libhlbl_gb300.so.

Propagator blocks are device buffers (torch tensors or raw device addresses)
in the reference's layout [2][12][V][24] doubles. One Contractor per lattice;
it owns its work buffers and a CUDA stream.
"""
from __future__ import annotations

import ctypes as C
from typing import NamedTuple

import numpy as np

from ._lib import check, i4, lib, ptr

FP64 = 0  # per-site products in FP64 (the exact path)
FP32 = 1  # per-site products in FP32, FP64 site and volume sums
# QED kernels (hlbl_ctx_set_qed_kernel): the stand-in through its closed-form
# paths, the stand-in through the generic paths, the dense test weight (no
# index structure) entry by entry, and the same as a whole-tensor function
QED_STANDIN, QED_STANDIN_GENERIC, QED_DENSE, QED_DENSE_KERV, QED_KQED = 0, 1, 2, 3, 4
HBARC_MEV_FM = 197.3269804  # include/hlbl/physics.hpp:9


def xunit(muon_mass_mev: float, lattice_spacing_fm: float) -> float:
    """m_mu a, the lattice unit in units of the muon mass (physics.hpp:12-14)."""
    return muon_mass_mev / HBARC_MEV_FM * lattice_spacing_fm


def measure_fma_peak(precision=FP64, device: int = 0) -> float:
    """CUDA-core FMA throughput in TFLOP/s (FP64 or FP32)."""
    out = C.c_double()
    check(lib.hlbl_measure_fma_peak(int(device), _prec(precision), C.byref(out)))
    return out.value


class Pieces2p2(NamedTuple):
    """The 2+2 pieces of one source (include/hlbl/contract.hpp:27-37)."""
    p1: np.ndarray    # [4][4][4][lmax]
    p234: np.ndarray  # [n_y][5][4][4][4]: P2_0, P2_1, P3, P4_0, P4_1


def _targets(targets):
    """(int array [n][4], n) of a target list."""
    flat = [int(v) for t in targets for v in t]
    if len(flat) % 4:
        raise ValueError("targets must be 4-vectors")
    return (C.c_int * max(4, len(flat)))(*flat), len(flat) // 4


def _prec(p) -> int:
    """'fp64'/'fp32' names, or an integer passed to the C ABI as is (which
    rejects values other than HLBL_FP64/HLBL_FP32 with HLBL_EINVAL)."""
    if p == "fp64":
        return FP64
    if p == "fp32":
        return FP32
    if isinstance(p, int):
        return p
    raise ValueError(f"precision must be fp64 or fp32, not {p!r}")


class Graph:
    """A recorded window (hlbl_graph): replay with launch()."""

    def __init__(self, h):
        self._h = h

    def launch(self, stream=None) -> None:
        raw = getattr(stream, "cuda_stream", stream)
        check(lib.hlbl_graph_launch(self._h, C.c_void_p(raw) if raw else None))

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib.hlbl_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Contractor:
    """Kernel sums of pairs of point sources (src/contract.cpp of the reference)."""

    def __init__(self, global_extents, local_extents=None, proc_coords=(0, 0, 0, 0),
                 lam: float = 0.4, device: int = 0):
        local_extents = global_extents if local_extents is None else local_extents
        h = C.c_void_p()
        check(lib.hlbl_ctx_create(C.byref(h), i4(global_extents), i4(local_extents),
                                  i4(proc_coords), C.c_double(lam), int(device)))
        self._h = h
        self.global_extents = tuple(int(a) for a in global_extents)
        self.local_extents = tuple(int(a) for a in local_extents)
        self.proc_coords = tuple(int(a) for a in proc_coords)
        self.lam = lam
        self.device = device

    # -- lifetime --------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            lib.hlbl_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    @property
    def volume(self) -> int:
        v = 1
        for a in self.local_extents:
            v *= a
        return v

    @property
    def block_length(self) -> int:
        """Doubles in one propagator block (provider.hpp:18-20)."""
        return int(lib.hlbl_block_length(self._h))

    def check(self) -> None:
        """Raise if a kernel gave up a bounded wait since the last check."""
        check(lib.hlbl_ctx_check(self._h))

    def set_stream(self, stream) -> None:
        """Run on a CUDA stream (torch.cuda.Stream, a raw handle, or None)."""
        raw = getattr(stream, "cuda_stream", stream)
        check(lib.hlbl_ctx_set_stream(self._h, C.c_void_p(raw) if raw else None))

    # -- the hot path ----------------------------------------------------
    def kernel_sum(self, d_fwd_src, d_fwd_y, gsx, yv, xunit: float, precision=FP64):
        """Both flavours' kernel sums of the pair (x = gsx, y = gsx + yv).

        Contractor::kernel_sum, src/contract.cpp:104-114 (one rank; with more
        ranks sum the returned values over ranks)."""
        out = (C.c_double * 2)()
        check(lib.hlbl_kernel_sum(self._h, ptr(d_fwd_src), ptr(d_fwd_y), i4(gsx), i4(yv),
                                  C.c_double(xunit), _prec(precision), out))
        return out[0], out[1]

    def kernel_sum_async(self, d_fwd_src, d_fwd_y, gsx, yv, xunit: float, d_out,
                         precision=FP64) -> None:
        """As kernel_sum, results written to the device buffer d_out[2]."""
        check(lib.hlbl_kernel_sum_async(self._h, ptr(d_fwd_src), ptr(d_fwd_y), i4(gsx), i4(yv),
                                        C.c_double(xunit), _prec(precision), ptr(d_out)))

    def kernel_sums_batched(self, d_fwd_y, d_srcs, gsxs, yvs, xunit: float, d_out,
                            precision=FP64) -> None:
        """All pairs one new source closes: pair i = (gsxs[i], gsxs[i] + yvs[i])
        with partner block d_srcs[i]; sums to the device buffer d_out[n][2].
        Asynchronous on the context's stream (batched launches share y)."""
        n = len(d_srcs)
        srcs = (C.c_void_p * max(1, n))(*[ptr(s) for s in d_srcs])
        g = (C.c_int * (4 * max(1, n)))(*[int(v) for p in gsxs for v in p])
        y = (C.c_int * (4 * max(1, n)))(*[int(v) for p in yvs for v in p])
        check(lib.hlbl_kernel_sums_batched(self._h, ptr(d_fwd_y), n, srcs, g, y, C.c_double(xunit),
                                           _prec(precision), ptr(d_out)))

    def reserve(self, max_pairs: int) -> None:
        check(lib.hlbl_ctx_reserve(self._h, int(max_pairs)))

    def stage_async(self, d_dst, h_src, nbytes: int, after_compute: bool = True) -> None:
        """Copy a pinned host block to the device on the side stream; the next
        contraction waits for it (host-cache staging). after_compute: wait
        first for contraction work already enqueued (d_dst may be in use)."""
        check(lib.hlbl_stage_async(self._h, ptr(d_dst), ptr(h_src), int(nbytes),
                                   1 if after_compute else 0))

    def autotune(self, d_fwd_y, d_srcs, gsxs, yvs, xunit: float, d_out) -> dict:
        """Pick the FP32 tile variants and batch group on this batch."""
        n = len(d_srcs)
        srcs = (C.c_void_p * n)(*[ptr(s) for s in d_srcs])
        g = (C.c_int * (4 * n))(*[int(v) for p in gsxs for v in p])
        y = (C.c_int * (4 * n))(*[int(v) for p in yvs for v in p])
        p1, p2, grp, ms = C.c_int(), C.c_int(), C.c_int(), C.c_double()
        check(lib.hlbl_autotune(self._h, ptr(d_fwd_y), n, srcs, g, y, C.c_double(xunit), ptr(d_out),
                                C.byref(p1), C.byref(p2), C.byref(grp), C.byref(ms)))
        return {"p1_tile": 4 if p1.value else 8,
                "p2": ("cuda-core tile 4", "cuda-core tile 2", "tensor-core")[p2.value],
                "batch_group": grp.value, "ms": ms.value}

    def set_qed_fp32(self, on: bool = True, r64: float = 0.1) -> None:
        """FP32 path's exact QED weight: FP32 quadrature outside min(|x|,|y|) < r64
        (FP64 inside), or FP64 everywhere."""
        check(lib.hlbl_ctx_set_qed_fp32(self._h, 1 if on else 0, float(r64)))

    @property
    def f32_block_length(self) -> int:
        """Floats in one FP32 tile copy of a block."""
        return int(lib.hlbl_f32_block_length(self._h))

    def kernel_sums_batched_f32(self, d_y32, d_x32s, gsxs, yvs, xunit: float, d_out) -> None:
        """kernel_sums_batched on FP32 tile copies (f32_tile_copy) of the blocks."""
        n = len(d_x32s)
        xs = (C.c_void_p * max(1, n))(*[ptr(s) for s in d_x32s])
        g = (C.c_int * (4 * max(1, n)))(*[int(v) for p in gsxs for v in p])
        y = (C.c_int * (4 * max(1, n)))(*[int(v) for p in yvs for v in p])
        check(lib.hlbl_kernel_sums_batched_f32(self._h, ptr(d_y32), n, xs, g, y, C.c_double(xunit),
                                               ptr(d_out)))

    def autotune_f32(self, d_y32, d_x32s, gsxs, yvs, xunit: float, d_out) -> dict:
        """Pick the FP32-copy path's pass-1 variant and pair group on this batch."""
        n = len(d_x32s)
        xs = (C.c_void_p * n)(*[ptr(s) for s in d_x32s])
        g = (C.c_int * (4 * n))(*[int(v) for p in gsxs for v in p])
        y = (C.c_int * (4 * n))(*[int(v) for p in yvs for v in p])
        v, grp, ms = C.c_int(), C.c_int(), C.c_double()
        check(lib.hlbl_autotune_f32(self._h, ptr(d_y32), n, xs, g, y, C.c_double(xunit), ptr(d_out),
                                    C.byref(v), C.byref(grp), C.byref(ms)))
        return {"p1": ("one stage, 2 CTAs/SM", "two stages, 1 CTA/SM",
                       "one flavour per CTA, two stages, 3 CTAs/SM",
                       "one flavour per CTA, producer warp, empty/full barriers")[v.value],
                "p1_variant": v.value,
                "p2": "tensor-core",
                "batch_group": grp.value, "ms": ms.value}

    def set_p1f32_variant(self, variant: int, group: int = 0) -> None:
        """The FP32-copy path's pass-1 variant (0-3, hlbl_gb300.h) and pairs per launch."""
        check(lib.hlbl_ctx_set_p1f32_variant(self._h, int(variant), int(group)))

    def f32_tile_copy(self, d_block, d_out) -> None:
        """The FP32 tile copy of a block (the tensor-core pass 2's input layout)."""
        check(lib.hlbl_f32_tile_copy(self._h, ptr(d_block), ptr(d_out)))

    def set_tensor_cores(self, on: bool) -> None:
        """FP32 two-flavour pass 2 on the tensor cores (default) or the CUDA cores."""
        check(lib.hlbl_ctx_set_tensor_cores(self._h, 1 if on else 0))

    def set_tc_fp16(self, on: bool = True) -> None:
        """FP16 (on) or TF32 operands in the FP32-copy path's tensor-core pass 2."""
        check(lib.hlbl_ctx_set_tc_fp16(self._h, 1 if on else 0))

    def graph_begin(self) -> None:
        check(lib.hlbl_graph_begin(self._h))

    def graph_end(self) -> "Graph":
        g = C.c_void_p()
        check(lib.hlbl_graph_end(self._h, C.byref(g)))
        return Graph(g)

    def set_batch_group(self, group: int) -> None:
        """Pairs per batched launch (1..16; 0 = 16)."""
        check(lib.hlbl_ctx_set_batch_group(self._h, int(group)))

    # -- the vendored launchers (kernels/cuda_lattice.h:49-57) -------------
    def cu_dzu_dzsu(self, d_dzu, d_dzsu, fwd_src, fwd_y, iflavor, proc_coords, gsx,
                    global_geom, local_geom) -> None:
        check(lib.hlbl_cu_dzu_dzsu(self._h, ptr(d_dzu), ptr(d_dzsu), ptr(fwd_src), ptr(fwd_y),
                                   int(iflavor), i4(proc_coords), i4(gsx), i4(global_geom),
                                   i4(local_geom)))

    def cu_4pt_contraction(self, d_kernel_sum, d_g_dzu, d_g_dzsu, fwd_src, fwd_y, iflavor,
                           proc_coords, gsx, xunit, yv, global_geom, local_geom) -> None:
        check(lib.hlbl_cu_4pt_contraction(self._h, ptr(d_kernel_sum), ptr(d_g_dzu),
                                          ptr(d_g_dzsu), ptr(fwd_src), ptr(fwd_y), int(iflavor),
                                          i4(proc_coords), i4(gsx), C.c_double(xunit), i4(yv),
                                          i4(global_geom), i4(local_geom)))

    def insert_gammas(self, d_dzu, d_dzsu, d_g_dzu, d_g_dzsu) -> None:
        """contract.cpp:58-77 on the device."""
        check(lib.hlbl_insert_gammas(self._h, ptr(d_dzu), ptr(d_dzsu), ptr(d_g_dzu),
                                     ptr(d_g_dzsu)))

    def reserve_kernel_memory(self) -> int:
        """Contractor::reserve_kernel_memory (contract.cpp:158-197)."""
        n = C.c_size_t()
        check(lib.hlbl_reserve_kernel_memory(self._h, C.byref(n)))
        return int(n.value)

    # -- the 2+2 pieces ----------------------------------------------------------
    @property
    def lmax(self) -> int:
        """The last dimension of P1: the largest global extent."""
        return int(lib.hlbl_2p2_lmax(self._h))

    def set_2p2_r64(self, r64: float) -> None:
        """FP32 2+2 path: the FP64 QED weight where an argument is shorter
        than r64 (units of 1/m_mu); 0, the default: FP32 everywhere."""
        check(lib.hlbl_ctx_set_2p2_r64(self._h, C.c_double(r64)))

    def reserve_2p2(self) -> None:
        """Allocate the 2+2 work buffers now (before a graph capture)."""
        check(lib.hlbl_2p2_reserve(self._h))

    def pieces_2p2(self, d_fwd, gsw, targets, xunit: float, precision=FP64) -> "Pieces2p2":
        """The 2+2 pieces of the source w = gsw for `targets` (global sites in
        [0, L)) from the device block of w, flavour 0: Contractor::pieces_2p2
        (src/contract.cpp:116-156). This rank's part (sum over ranks with
        more than one). p1 flat [4][4][4][lmax], p234 flat [n_y][5][4][4][4]."""
        tg, n = _targets(targets)
        p1 = np.zeros(64 * self.lmax)
        p234 = np.zeros(n * 5 * 64)
        check(lib.hlbl_pieces_2p2(self._h, ptr(d_fwd), i4(gsw), tg, n, C.c_double(xunit),
                                  _prec(precision), p1.ctypes.data_as(C.c_void_p),
                                  p234.ctypes.data_as(C.c_void_p)))
        return Pieces2p2(p1, p234)

    def pieces_2p2_async(self, d_fwd, gsw, targets, xunit: float, d_p1, d_p234,
                         precision=FP64) -> None:
        """As pieces_2p2, asynchronous, into the device buffers d_p1 and d_p234."""
        tg, n = _targets(targets)
        check(lib.hlbl_pieces_2p2_async(self._h, ptr(d_fwd), i4(gsw), tg, n,
                                        C.c_double(xunit), _prec(precision), ptr(d_p1),
                                        ptr(d_p234)))

    def pieces_2p2_f32(self, d_x32, gsw, targets, xunit: float, d_p1, d_p234) -> None:
        """As pieces_2p2_async in FP32, from the block's FP32 tile copy."""
        tg, n = _targets(targets)
        check(lib.hlbl_pieces_2p2_f32(self._h, ptr(d_x32), i4(gsw), tg, n, C.c_double(xunit),
                                      ptr(d_p1), ptr(d_p234)))

    def compute_2p2(self, d_fwd_y, iflavor: int, gsw, gycoords, xunit: float, precision=FP64):
        """compute_2p2_gpu (kernels/hlbl_kernels/kernels.cu:753-870) without its
        MPI reduction: (P1 flat [4][4][4][lmax], P234 flat [5][n_y][64])."""
        tg, n = _targets(gycoords)
        p1 = np.zeros(64 * self.lmax)
        p234 = np.zeros(n * 5 * 64)
        check(lib.hlbl_compute_2p2(self._h, ptr(d_fwd_y), p1.ctypes.data_as(C.c_void_p),
                                   p234.ctypes.data_as(C.c_void_p), int(iflavor), i4(gsw), tg, n,
                                   C.c_double(xunit), _prec(precision)))
        return p1, p234

    # -- the QED weight ------------------------------------------------------
    def set_qed_kernel(self, kind: int, seed: int = 0) -> None:
        """The QED kernel pass 2 and the 2+2 pieces weight with (QED_STANDIN,
        QED_STANDIN_GENERIC, QED_DENSE with its table seed, QED_DENSE_KERV,
        QED_KQED in a build linked with a KQED)."""
        check(lib.hlbl_ctx_set_qed_kernel(self._h, int(kind), C.c_uint64(seed)))

    def set_qed(self, surrogate=None, r0: float = -1.0) -> None:
        """Pass 2's QED weight: the exact stand-in (surrogate None) or the
        learned surrogate with fallback radius r0 (< 0: its validated radius)."""
        if surrogate is None:
            check(lib.hlbl_ctx_set_qed(self._h, 0, None, C.c_double(0.0)))
        else:
            check(lib.hlbl_ctx_set_qed(self._h, 1, surrogate.handle, C.c_double(r0)))

    def qed_fallbacks(self) -> int:
        n = C.c_ulonglong()
        check(lib.hlbl_ctx_qed_fallbacks(self._h, C.byref(n)))
        return int(n.value)

    # -- measurement ---------------------------------------------------------
    def set_profiling(self, on: bool) -> None:
        """Time every pass-1/pass-2 kernel with CUDA events (resets totals)."""
        check(lib.hlbl_ctx_set_profiling(self._h, 1 if on else 0))

    def kernel_times(self):
        """((pass-1 ms, launches), (pass-2 ms, launches)) since profiling began."""
        ms = (C.c_double * 2)()
        n = (C.c_longlong * 2)()
        check(lib.hlbl_ctx_kernel_times(self._h, ms, n))
        return (ms[0], n[0]), (ms[1], n[1])

    # -- fixtures (src/provider.cpp) ---------------------------------------
    def fill_random_block(self, d_out, seed: int) -> None:
        """fill_random_block with a per-source seed, on the device."""
        check(lib.hlbl_fill_random_block(self._h, ptr(d_out), C.c_uint64(seed)))

    def fill_gaussian_block(self, d_out, seed: int) -> None:
        check(lib.hlbl_fill_gaussian_block(self._h, ptr(d_out), C.c_uint64(seed)))

    @staticmethod
    def source_seed(run_seed: int, gsx) -> int:
        """RandomProvider's per-source seed (provider.cpp:59-64)."""
        return int(lib.hlbl_source_seed(C.c_uint64(run_seed), i4(gsx)))
