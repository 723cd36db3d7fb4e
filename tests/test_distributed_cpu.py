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

    def pieces(self, fwd, gsw, targets, xunit, iflavor):
        import support as S

        p1, p234 = S.oracle_pieces_2p2(fwd, gsw, targets, xunit, self.glob, self.loc, self.pc,
                                       iflavor=iflavor)
        return torch.from_numpy(p1.copy()), torch.from_numpy(p234.copy())


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


def _rank_2p2(rank, world, port, q):
    sys.path.insert(0, HERE)
    sys.path.insert(0, os.path.dirname(HERE))
    import datetime
    import json

    import torch.distributed as dist

    import support as S
    from hlbl_gb300.distributed import ShardedContractor

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world,
                            timeout=datetime.timedelta(seconds=20))
    try:
        with open(os.path.join(HERE, "golden", "reference_2p2.json")) as fh:
            sp = json.load(fh)["compute_2p2_split"]
        glob, loc = sp["global"], sp["local"]
        pc = [rank, 0, 0, 0]
        full = S.random_block(glob, sp["seed"])
        V, Vl = int(np.prod(glob)), int(np.prod(loc))
        fwd = np.ascontiguousarray(full.reshape(2, 12, V, 24)[:, :, rank * Vl:(rank + 1) * Vl, :]).ravel()
        sc = ShardedContractor(OracleBackend(glob, loc, pc))
        p1, p234 = sc.pieces_2p2(fwd, sp["gsw"], sp["targets"], sp["xunit"], sp["iflavor"])
        q.put((rank, (p1.numpy(), p234.numpy())))
    except Exception as e:
        q.put((rank, repr(e)))
    finally:
        dist.destroy_process_group() if dist.is_initialized() else None


def _run(fail_rank, port, target=None):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    if target is None:
        ps = [ctx.Process(target=_rank, args=(r, 2, port, q, fail_rank)) for r in range(2)]
    else:
        ps = [ctx.Process(target=target, args=(r, 2, port, q)) for r in range(2)]
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


def test_two_gloo_ranks_2p2_pieces_match_reference_split():
    """P1 and P234 summed over two gloo ranks (each its half of an 8x4^3
    lattice, flavour 1) equal the sum of the reference's per-rank partials."""
    import json

    with open(os.path.join(HERE, "golden", "reference_2p2.json")) as fh:
        sp = json.load(fh)["compute_2p2_split"]
    n_y = len(sp["targets"])
    want1 = sum(np.asarray(r["p1"]) for r in sp["ranks"]).reshape(4, 4, 4, -1)
    want234 = sum(np.asarray(r["p234_raw"]).reshape(5, n_y, 64).transpose(1, 0, 2) for r in sp["ranks"])
    out = _run(-1, 29519, _rank_2p2)
    for r in (0, 1):
        assert isinstance(out[r], tuple), out[r]
        p1, p234 = out[r]
        assert np.abs(p1 - want1).max() <= 1e-12 * np.abs(want1).max()
        assert np.abs(p234 - want234).max() <= 1e-12 * np.abs(want234).max()
