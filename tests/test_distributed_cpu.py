"""Site sharding over two gloo ranks on CPU (the oracle as each rank's
compute): the totals and the exchange match the reference's own two-rank
split (tests/golden), and a rank that fails is reported to the other."""
import os
import sys

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))


class OracleBackend:
    def __init__(self, glob, loc, pc):
        self.glob, self.loc, self.pc = glob, loc, pc

    def pass1(self, src, y, f, gsx):
        import support as S

        dzu, dzsu = S.oracle_dz(src, y, f, gsx, self.glob, self.loc, self.pc)
        return torch.from_numpy(np.concatenate([dzu, dzsu]))

    def pass2(self, dz, src, y, f, gsx, xunit, yv):
        import support as S

        d = dz.numpy()
        g_dzu, g_dzsu = S.oracle_gammas(d[:1728], d[1728:])
        v = S.oracle_4pt(g_dzu, g_dzsu, src, y, f, gsx, xunit, yv, self.glob, self.loc, self.pc)
        return torch.tensor([v], dtype=torch.float64)


def _rank(rank, world, port, q, fail_rank):
    sys.path.insert(0, HERE)
    sys.path.insert(0, os.path.dirname(HERE))
    import datetime

    import torch.distributed as dist

    import support as S
    from hlbl_gb300.distributed import ShardedContractor

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world,
                            timeout=datetime.timedelta(seconds=20))
    try:
        sp = S.golden()["two_rank_split"]
        pc = [rank, 0, 0, 0]
        src = S.random_block(sp["local"], sp["seeds"][0], pc)
        y = S.random_block(sp["local"], sp["seeds"][1], pc)
        if rank == fail_rank:
            raise RuntimeError("rank fails before the exchange")
        sc = ShardedContractor(OracleBackend(sp["global"], sp["local"], pc))
        q.put((rank, sc.kernel_sum(src, y, sp["gsx"], sp["yv"], sp["xunit"])))
    except Exception as e:  # reported to the test, not raised in the child
        q.put((rank, repr(e)))
    finally:
        dist.destroy_process_group() if dist.is_initialized() else None


def _run(fail_rank, port):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q, fail_rank)) for r in range(2)]
    for p in ps:
        p.start()
    out = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
    return out


def test_two_gloo_ranks_match_reference_split():
    sys.path.insert(0, HERE)
    import support as S

    sp = S.golden()["two_rank_split"]
    out = _run(-1, 29517)
    for r in (0, 1):
        assert isinstance(out[r], tuple), out[r]
        assert S.rel_err(out[r], sp["single_rank_kernel_sum"]) <= 1e-12


def test_failed_rank_is_reported_not_hung():
    out = _run(1, 29518)
    assert "rank fails" in out[1]
    # the surviving rank's collective ends with an error (peer gone), not a hang
    assert isinstance(out[0], str)
