"""The propagators the schedule still needs: hlbl::PropagatorCache
(include/hlbl/propagator_cache.hpp, src/propagator_cache.cpp of the
reference), same states, same errors, same peak accounting.

  device    blocks on the GPU, read in place.
  host      blocks in pinned host memory; a contraction gets its block through
            one of two device staging slots. Unlike the reference's
            synchronous cudaMemcpy (propagator_cache.cpp:63-66), the copy is
            issued on the contractor's side stream (hlbl_stage_async), so the
            next source's block streams in while the current one computes.
  device32  the FP32 tile copy of each block on the GPU (half the bytes):
            the solve fills one FP64 scratch block, which is converted into
            the entry's copy as it is stored (hlbl_f32_tile_copy); the
            FP32-copy contraction path (kernel_sums_batched_f32) reads them.

Buffers come from an allocator object, so the bookkeeping is testable
without a GPU: TorchBuffers (the product) or any object with the same three
methods.
"""
from __future__ import annotations

from typing import Dict, Optional, Tuple

Vec4 = Tuple[int, int, int, int]
DEVICE, HOST, DEVICE32 = "device", "host", "device32"


class TorchBuffers:
    """Device blocks, pinned host blocks and staging through a Contractor."""

    def __init__(self, contractor):
        import torch

        self.torch = torch
        self.c = contractor

    def device(self, n):
        return self.torch.empty(n, dtype=self.torch.float64, device="cuda")

    def pinned(self, n):
        return self.torch.empty(n, dtype=self.torch.float64, pin_memory=True)

    def stage(self, dst, src):
        self.c.stage_async(dst, src, src.numel() * 8)

    def store(self, dst_host, src_dev):
        self.c.check()  # the solve that filled src_dev ran on the contractor's stream
        dst_host.copy_(src_dev)

    def device32(self):
        return self.torch.empty(self.c.f32_block_length, dtype=self.torch.float32, device="cuda")

    def convert(self, dst32, src_dev):
        self.c.f32_tile_copy(src_dev, dst32)  # on the contractor's stream, after the solve


class PropagatorCache:
    """Mirror of hlbl::PropagatorCache (propagator_cache.hpp:24-75)."""

    def __init__(self, residency: str, block_len: int, buffers, pending: Optional[Dict] = None):
        if residency not in (DEVICE, HOST, DEVICE32):
            raise ValueError("residency is 'device', 'host' or 'device32'")
        self.residency = residency
        self.block_len = block_len
        self.buf = buffers
        self.pending: Dict[Vec4, int] = dict(pending or {})
        self.entries: Dict[Vec4, object] = {}
        self.peak = 0
        self.pool = []          # host: freed pinned blocks, reused
        self.scratch = None     # host: the solve target
        self.staging = [None, None]
        self.staged = [None, None]

    def reset(self, pending: Dict[Vec4, int]) -> None:
        """propagator_cache.cpp:15-20"""
        if self.entries:
            raise RuntimeError("PropagatorCache: reset with positions still cached")
        self.pending = dict(pending)
        self.peak = 0

    def begin_insert(self, position: Vec4):
        """The device buffer the solve fills (propagator_cache.cpp:23-34)."""
        if position in self.entries:
            raise RuntimeError("PropagatorCache: position inserted twice")
        if self.residency == DEVICE:
            self.entries[position] = self.buf.device(self.block_len)
            return self.entries[position]
        if self.scratch is None:
            self.scratch = self.buf.device(self.block_len)
        return self.scratch

    def end_insert(self, position: Vec4) -> None:
        """propagator_cache.cpp:36-50"""
        if self.residency == HOST:
            h = self.pool.pop() if self.pool else self.buf.pinned(self.block_len)
            self.buf.store(h, self.scratch)
            self.entries[position] = h
        elif self.residency == DEVICE32:
            h = self.pool.pop() if self.pool else self.buf.device32()
            self.buf.convert(h, self.scratch)
            self.entries[position] = h
        self.peak = max(self.peak, len(self.entries))
        if self.pending.get(position, 0) == 0:
            self._evict(position)

    def device_ptr(self, position: Vec4, slot: int):
        """The block on the device; host mode stages it into slot 0 or 1
        unless it is there already (propagator_cache.cpp:52-68)."""
        if position not in self.entries:
            raise RuntimeError("PropagatorCache: position is not cached")
        if self.residency in (DEVICE, DEVICE32):
            return self.entries[position]
        if slot not in (0, 1):
            raise RuntimeError("PropagatorCache: bad slot")
        if self.staging[slot] is None:
            self.staging[slot] = self.buf.device(self.block_len)
        if self.staged[slot] != position:
            self.buf.stage(self.staging[slot], self.entries[position])
            self.staged[slot] = position
        return self.staging[slot]

    def pair_done(self, older: Vec4, newer: Vec4) -> None:
        """propagator_cache.cpp:70-74"""
        for p in (older, newer):
            self.pending[p] = self.pending.get(p, 0) - 1
            if self.pending[p] == 0:
                self._evict(p)

    def contains(self, position: Vec4) -> bool:
        return position in self.entries

    def size(self) -> int:
        return len(self.entries)

    def _evict(self, position: Vec4) -> None:
        """propagator_cache.cpp:80-91"""
        e = self.entries.pop(position, None)
        if e is not None and self.residency in (HOST, DEVICE32):
            self.pool.append(e)
        for i in (0, 1):
            if self.staged[i] == position:
                self.staged[i] = None
