"""ResultWriter and TimingLog (src/output.cpp:131-332): the reference's
dataset layout, shapes, dtypes and attributes, flushed per window, written by
the driver loop (CPU, fake contraction)."""
import numpy as np
import pytest

from hlbl_gb300 import schedule
from hlbl_gb300.cache import PropagatorCache
from hlbl_gb300.driver import run_chains
from hlbl_gb300.output import Chain, ResultWriter, RunInfo, TimingLog, read_results
from test_cache_driver import NumpyBuffers, Recorder, provider


class ShapedRecorder(Recorder):
    """Pieces of the reference's shapes: P1 [4][4][4][Lmax] holding the source
    block's first value, P234 [n_y][5][64] holding the target index."""

    def __init__(self, lmax):
        self.lmax = lmax

    def pieces_2p2(self, d_fwd, gsw, targets, xunit, precision):
        from hlbl_gb300.contract import Pieces2p2

        p234 = np.repeat(np.arange(len(targets), dtype=float), 5 * 64).reshape(len(targets), 5, 64)
        return Pieces2p2(np.full((4, 4, 4, self.lmax), float(d_fwd[0])), p234)


def test_driver_writes_the_reference_layout(tmp_path):
    lat = (6, 6, 6, 6)
    hs = [(1, 1, 1, 1), (-1, 1, -1, 1)]
    chains = [schedule.build_schedule(h, 1, 1) for h in hs]
    srcs = [((1, 1, 1, 1), [(0, 0, 0, 0), (2, 3, 4, 5)])]
    info = RunInfo(lattice=lat, chains=[Chain((0, 0, 0, 0), h, 1, 1) for h in hs], muon_mass=105.658,
                   lattice_spacing=0.1, xunit=0.0535, with_2p2=True)
    path = str(tmp_path / "run.npz")
    w = ResultWriter(path, info)
    log = TimingLog(str(tmp_path / "timing.csv"))
    out22 = []
    res, st, _ = run_chains(chains, lat, 0.0535, provider, ShapedRecorder(max(lat)),
                            PropagatorCache("device", 4, NumpyBuffers()), sources_2p2=srcs,
                            results_2p2=out22, writer=w, timing=log)
    log.close()
    f = read_results(path)
    n = len(res)
    assert f["kernel_sum/x"].shape == (n, 4) and f["kernel_sum/x"].dtype == np.int32
    assert f["kernel_sum/kernel_sum"].shape == (n, 2) and f["kernel_sum/kernel_sum"].dtype == np.float64
    assert [tuple(r) for r in f["kernel_sum/y"]] == [r.y for r in res]
    assert list(f["kernel_sum/window"]) == [r.window for r in res]
    assert np.array_equal(f["kernel_sum/kernel_sum"], np.array([r.kernel_sum for r in res]))
    assert f["2p2/w"].shape == (1, 4) and f["2p2/P1"].shape == (1, 4, 4, 4, 6)
    assert [tuple(r) for r in f["2p2/w"]] == [out22[0].w] and f["2p2/P1"][0, 0, 0, 0, 0] == hash(out22[0].w) % 1000
    assert f["2p2/pair_y"].shape == (2, 4) and f["2p2/P234"].shape == (2, 5, 4, 4, 4)
    assert [tuple(r) for r in f["2p2/pair_y"]] == [(0, 0, 0, 0), (2, 3, 4, 5)]
    assert np.all(f["2p2/P234"][1] == 1) and np.all(f["2p2/P234"][0] == 0)
    assert [tuple(r) for r in f["2p2/pair_yv"]] == [tuple(v) for v in out22[0].yv]
    assert f["chains"].tolist() == [[0, 0, 0, 0] + list(h) + [1, 1] for h in hs]
    a = f["attrs:/"]
    assert a["lattice"] == list(lat) and a["kernel"] == "LLambda0.4" and "direction" not in a
    assert "P1_index" in f["attrs:2p2"]
    lines = open(tmp_path / "timing.csv").read().splitlines()
    assert lines[0] == "kind,chain,window,x0,x1,x2,x3,y0,y1,y2,y3,seconds,iterations"
    kinds = [l.split(",")[0] for l in lines[1:]]
    assert kinds.count("solve") == st.positions_solved
    assert kinds.count("kernel_sum") == st.pairs and kinds.count("2p2") == 1
    sol = next(l for l in lines[1:] if l.startswith("solve"))
    assert sol.split(",")[7:11] == ["", "", "", ""]  # a solve leaves y empty


def test_writer_rejects_what_the_reference_rejects(tmp_path):
    with pytest.raises(RuntimeError):
        ResultWriter(str(tmp_path / "a.npz"), RunInfo(lattice=(4, 4, 4, 4)))
    w = ResultWriter(str(tmp_path / "b.npz"), RunInfo(lattice=(4, 4, 4, 4), chains=[Chain()]))
    with pytest.raises(RuntimeError):
        w.append_2p2([])  # no 2p2 group in this run
    f = read_results(str(tmp_path / "b.npz"))
    assert f["kernel_sum/x"].shape == (0, 4) and f["attrs:/"]["stride"] == 1


def test_flush_every_and_close(tmp_path):
    from hlbl_gb300.driver import PairResult

    path = str(tmp_path / "c.npz")
    w = ResultWriter(path, RunInfo(lattice=(4, 4, 4, 4), chains=[Chain()]), flush_every=3)
    row = PairResult((0, 0, 0, 0), (1, 1, 1, 1), (1, 1, 1, 1), 0, 0, (1.0, 2.0))
    w.append([row])
    w.append([row])
    assert read_results(path)["kernel_sum/x"].shape == (0, 4)  # not yet rewritten
    w.append([row])
    assert read_results(path)["kernel_sum/x"].shape == (3, 4)
    w.append([row])
    w.close()
    f = read_results(path)
    assert f["kernel_sum/kernel_sum"].shape == (4, 2) and f["kernel_sum/kernel_sum"][3, 1] == 2.0
    with pytest.raises(ValueError):
        ResultWriter(path, RunInfo(lattice=(4, 4, 4, 4), chains=[Chain()]), flush_every=0)
