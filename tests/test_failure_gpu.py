"""Failure detection without a GPU fault: a kernel's bounded wait runs out (a
transfer nothing performs), the kernel sets the context's error flag and
returns, the host reports it, and the context keeps working."""
import time

import pytest

import support as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_bounded_wait_reports_and_context_survives():
    import hlbl_gb300 as hg
    from hlbl_gb300._lib import check, lib

    lat = (4, 4, 4, 4)
    src, y = S.random_block(lat, 1), S.random_block(lat, 2)
    with hg.Contractor(lat) as c:
        t0 = time.time()
        check(lib.hlbl_selftest_wait_timeout(c.handle))
        with pytest.raises(hg.HlblError, match="gave up waiting"):
            c.check()
        assert time.time() - t0 < 30
        c.check()  # the flag was cleared
        got = c.kernel_sum(torch.from_numpy(src).cuda(), torch.from_numpy(y).cuda(), (0, 0, 0, 0),
                           (1, 1, 1, 1), 0.5, hg.FP64)
        assert S.rel_err(got, S.oracle_kernel_sum(src, y, (0, 0, 0, 0), (1, 1, 1, 1), 0.5, lat)) <= 1e-12
