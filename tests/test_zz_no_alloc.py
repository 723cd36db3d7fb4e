"""The allocation-free pass 1 (hlbl_cu_dzu_dzsu_noalloc).

It serves callers that cannot allocate device memory when they contract --
a process whose solver already holds nearly all device memory in its own
pool, or one measuring free memory around the kernels. Its scratch is a
fixed array inside the library that every call reuses, so this test calls
it several times in a row with different inputs and checks each result
against the context-based entry point, hlbl_cu_dzu_dzsu, and against the CPU
oracle, at the FP64 bar of the other parity tests (1e-12 relative). One case
has far more tiles than thread blocks (each block walks many tiles, with the
next tile's copy in flight). The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

import support as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
TOL64 = 1e-12


def _with_context(hg, src, y, f, gsx, glob, loc, pc):
    with hg.Contractor(glob, loc, pc) as c:
        dzu = torch.zeros(1728, dtype=torch.float64, device="cuda")
        dzsu = torch.zeros(1152, dtype=torch.float64, device="cuda")
        c.cu_dzu_dzsu(dzu, dzsu, src, y, f, pc, gsx, glob, loc)
        torch.cuda.synchronize()
        return torch.cat([dzu, dzsu]).cpu().numpy()


def _without_allocation(lib, src, y, f, gsx, glob, loc, pc):
    from hlbl_gb300._lib import i4

    dzu = torch.zeros(1728, dtype=torch.float64, device="cuda")
    dzsu = torch.zeros(1152, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.hlbl_cu_dzu_dzsu_noalloc(dzu.data_ptr(), dzsu.data_ptr(), src.data_ptr(),
                                      y.data_ptr(), f, i4(pc), i4(gsx), i4(glob), i4(loc),
                                      C.c_void_p(stream))
    assert rc == 0, lib.hlbl_last_error().decode()
    torch.cuda.synchronize()
    return torch.cat([dzu, dzsu]).cpu().numpy()


def test_noalloc_pass1_matches_context_entry_twice_in_a_row():
    import hlbl_gb300 as hg
    from hlbl_gb300._lib import lib

    cases = [
        # (lattice, local, proc coords, seeds, flavour, gsx)
        ((8, 6, 6, 6), (8, 6, 6, 6), (0, 0, 0, 0), (41, 42), 0, (3, 1, 5, 2)),
        ((8, 4, 4, 4), (4, 4, 4, 4), (1, 0, 0, 0), (43, 44), 1, (6, 0, 3, 1)),
        # 8,192 tiles of 8 sites: many more than the resident blocks
        ((16, 16, 16, 16), (16, 16, 16, 16), (0, 0, 0, 0), (45, 46), 1, (9, 2, 15, 7)),
    ]
    for glob, loc, pc, seeds, f, gsx in cases:
        h_src, h_y = S.random_block(loc, seeds[0], pc), S.random_block(loc, seeds[1], pc)
        src, y = torch.from_numpy(h_src).cuda(), torch.from_numpy(h_y).cuda()
        want = _with_context(hg, src, y, f, gsx, glob, loc, pc)
        dzu, dzsu = S.oracle_dz(h_src, h_y, f, gsx, glob, loc, pc)
        oracle = np.concatenate([np.ravel(dzu), np.ravel(dzsu)])
        got = _without_allocation(lib, src, y, f, gsx, glob, loc, pc)
        assert np.all(np.isfinite(got))
        scale = np.max(np.abs(want))
        assert scale > 0
        assert np.max(np.abs(got - want)) <= TOL64 * scale
        assert np.max(np.abs(got - oracle)) <= TOL64 * np.max(np.abs(oracle))
