"""Site sharding over ranks: the reference's domain decomposition
(src/geometry.cpp:21-36) and its one exchange step, the all-reduce of the
2,880 pass-1 sums between the passes and of the final sums
(src/contract.cpp:53-56, :100). The 2+2 pieces shard the same way: every
rank computes its sites' part of P1 and P234, and one all-reduce of each
gives the totals (compute_2p2_gpu's MPI_Iallreduce, kernels.cu:824-860).

Each rank holds its sub-lattice's blocks; ShardedContractor runs pass 1 on
them, all-reduces the sums over the process group, inserts the gammas, runs
pass 2 and all-reduces the two results. The per-rank compute is a backend:
GpuBackend (this library's interface-B entry points) or, in the CPU tests,
the oracle.
"""
from __future__ import annotations

import torch
import torch.distributed as dist


class GpuBackend:
    """Pass 1, gamma insertion and pass 2 of one rank through the C ABI."""

    def __init__(self, contractor, global_extents, local_extents, proc_coords):
        self.c = contractor
        self.glob, self.loc, self.pc = global_extents, local_extents, proc_coords

    def pass1(self, src, y, f, gsx):
        dzu = torch.zeros(1728, dtype=torch.float64, device="cuda")
        dzsu = torch.zeros(1152, dtype=torch.float64, device="cuda")
        self.c.cu_dzu_dzsu(dzu, dzsu, src, y, f, self.pc, gsx, self.glob, self.loc)
        self.c.check()
        return torch.cat([dzu, dzsu])

    def pass2(self, dz, src, y, f, gsx, xunit, yv):
        dzu, dzsu = dz[:1728].contiguous(), dz[1728:].contiguous()
        g_dzu = torch.empty(6912, dtype=torch.float64, device="cuda")
        g_dzsu = torch.empty(4608, dtype=torch.float64, device="cuda")
        self.c.insert_gammas(dzu, dzsu, g_dzu, g_dzsu)
        ks = torch.zeros(1, dtype=torch.float64, device="cuda")
        self.c.cu_4pt_contraction(ks, g_dzu, g_dzsu, src, y, f, self.pc, gsx, xunit, yv, self.glob,
                                  self.loc)
        self.c.check()
        return ks


    def pieces(self, fwd, gsw, targets, xunit, iflavor):
        """This rank's P1 [4][4][4][Lmax] and P234 [n_y][5][64] on the device."""
        p1, p234 = self.c.compute_2p2(fwd, iflavor, gsw, targets, xunit)
        n = len(targets)
        p234 = p234.reshape(5, n, 64).transpose(1, 0, 2).copy()
        return torch.from_numpy(p1).cuda(), torch.from_numpy(p234).cuda()


class ShardedContractor:
    """kernel_sum over all ranks of `group`; every rank gets the totals."""

    def __init__(self, backend, group=None):
        self.b = backend
        self.group = group

    def kernel_sum(self, src, y, gsx, yv, xunit):
        out = []
        for f in (0, 1):
            dz = self.b.pass1(src, y, f, gsx)
            dist.all_reduce(dz, op=dist.ReduceOp.SUM, group=self.group)  # the exchange step
            part = self.b.pass2(dz, src, y, f, gsx, xunit, yv)
            dist.all_reduce(part, op=dist.ReduceOp.SUM, group=self.group)
            out.append(float(part.item()))
        return tuple(out)

    def pieces_2p2(self, fwd, gsw, targets, xunit, iflavor=0):
        """The 2+2 pieces over all ranks of `group`: (P1 [4][4][4][Lmax],
        P234 [n_y][5][64]) on every rank."""
        p1, p234 = self.b.pieces(fwd, gsw, targets, xunit, iflavor)
        dist.all_reduce(p1, op=dist.ReduceOp.SUM, group=self.group)
        dist.all_reduce(p234, op=dist.ReduceOp.SUM, group=self.group)
        return p1, p234
