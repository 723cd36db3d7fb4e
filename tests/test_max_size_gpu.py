"""The largest configuration's lattice, 48^3 x 96 (V = 10,616,832 sites, 49 GB
per FP64 block): one pair's kernel sums, FP32 against FP64, and one source's
2+2 pieces for two targets, FP32 against FP64. Checks that every index and
buffer size holds at this volume (block offsets past 2^32 elements) and that
the FP32 bars hold there too. Needs a GPU with ~200 GB free."""
import numpy as np
import pytest

import support as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_48cubed_x_96_pair_and_2p2():
    import hlbl_gb300 as hg

    lat = (96, 48, 48, 48)
    free, _ = torch.cuda.mem_get_info()
    if free < 200 * 2**30:
        pytest.skip("needs ~200 GB of free device memory")
    xu = hg.xunit(105.658, 0.1)
    with hg.Contractor(lat) as c:
        n = c.block_length
        assert n == 2 * 12 * 24 * 10616832  # 6.1e9 doubles: 64-bit offsets
        x = torch.empty(n, dtype=torch.float64, device="cuda")
        y = torch.empty(n, dtype=torch.float64, device="cuda")
        c.fill_gaussian_block(x, hg.Contractor.source_seed(5, (0, 0, 0, 0)))
        c.fill_gaussian_block(y, hg.Contractor.source_seed(5, (4, 4, 4, 4)))
        gsx, yv = (0, 0, 0, 0), (4, 4, 4, 4)
        k64 = c.kernel_sum(x, y, gsx, yv, xu, hg.FP64)
        k32 = c.kernel_sum(x, y, gsx, yv, xu, hg.FP32)
        assert np.all(np.isfinite(k64)) and np.all(np.isfinite(k32))
        assert S.pair_rel_err(k32, k64) <= 1e-4
        targets = [(4, 4, 4, 4), (60, 30, 2, 47)]
        p64 = c.pieces_2p2(y, (4, 4, 4, 4), targets, xu, hg.FP64)
        p32 = c.pieces_2p2(y, (4, 4, 4, 4), targets, xu, hg.FP32)
        a, b = p32.p234.reshape(-1, 5, 64), p64.p234.reshape(-1, 5, 64)
        for t in range(2):
            for g in range(5):
                assert np.abs(a[t, g] - b[t, g]).max() <= 1e-5 * np.abs(b[t, g]).max()
        assert np.abs(p32.p1 - p64.p1).max() <= 1e-6 * np.abs(p64.p1).max()
        del x, y
    torch.cuda.empty_cache()
