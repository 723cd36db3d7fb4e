"""Result file and timing log of a run (the reference's ResultWriter and
TimingLog, src/output.cpp:131-332, include/hlbl/output.hpp).

The reference writes one HDF5 file per run. No HDF5 library is available to
this package, so ResultWriter keeps the same datasets, shapes, dtypes and
attributes in a NumPy .npz container: dataset "group/name" is the array under
that key, the attributes of the file and of a group are a JSON object under
"attrs:/" and "attrs:<group>". As in the reference every append is flushed
(the file is rewritten in full and renamed into place), so a killed job keeps
its finished windows; `flush_every` = n > 1 rewrites after every n-th append
instead (the container has no in-place append, so a rewrite costs the whole
file), and `close()` writes what is pending.

  kernel_sum/  one row per pair
    x[N][4], y[N][4], yv[N][4], chain[N], window[N]   int32
    kernel_sum[N][2]                                   float64 (flavour 0, 1)
  2p2/         with RunInfo.with_2p2; one row per 2+2 source
    w[M][4], chain[M], window[M]                       int32
    P1[M][4][4][4][Lmax]                               float64
               and one row per (source, target)
    pair_w[R][4], pair_y[R][4], pair_yv[R][4]          int32
    P234[R][5][4][4][4]                                float64 (P2_0, P2_1, P3, P4_0, P4_1)
  chains[C][10]  start0..3, dir0..3, stride, steps     int32
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass, field
from typing import List

import numpy as np


@dataclass
class Chain:
    """One chain of the input (input.hpp Chain)."""
    start: tuple = (0, 0, 0, 0)
    direction: tuple = (1, 1, 1, 1)
    stride: int = 1
    steps: int = -1


@dataclass
class RunInfo:
    """What identifies a run (output.hpp RunInfo)."""
    lattice: tuple = (0, 0, 0, 0)
    procs: tuple = (1, 1, 1, 1)
    nconf: int = -1
    chains: List[Chain] = field(default_factory=list)
    kernel: str = "LLambda0.4"
    muon_mass: float = 0.0
    lattice_spacing: float = 0.0
    xunit: float = 0.0
    with_2p2: bool = False


class ResultWriter:
    """output.cpp:131-297 in a .npz container (module docstring)."""

    def __init__(self, path: str, info: RunInfo, flush_every: int = 1):
        if not info.chains:
            raise RuntimeError("ResultWriter: no chains")
        if flush_every < 1:
            raise ValueError("ResultWriter: flush_every must be >= 1")
        self.path = path
        self.info = info
        self.flush_every = flush_every
        self._pending = 0
        self.lmax = max(int(a) for a in info.lattice)
        self._ks = {"x": [], "y": [], "yv": [], "chain": [], "window": [], "kernel_sum": []}
        self._p22 = {"w": [], "chain": [], "window": [], "P1": [], "pair_w": [], "pair_y": [],
                     "pair_yv": [], "P234": []}
        self._attrs = {"/": self._file_attrs()}
        if info.with_2p2:
            self._attrs["2p2"] = {
                "rows": "w, chain, window, P1: one row per 2+2 source, at its first solve; "
                        "pair_w, pair_y, pair_yv, P234: one row per (source, target)",
                "P1_index": "P1[row][rho][sigma][nu][zeta]: Pi_{sigma nu}(z) summed over the "
                            "sites z with (z - w)_rho mod L_rho = zeta; 0 for zeta >= L_rho",
                "P234_index": "P234[row][geometry][rho][sigma][nu], geometry P2_0, P2_1, P3, "
                              "P4_0, P4_1; only rho < sigma is filled (P4_1: rho != sigma)",
                "flavour": "operator 0 only (iflavor 0 of compute_2p2_gpu, as cvc): the "
                           "two-point function is the same for both flavours"}
        self._flush()

    def _file_attrs(self):
        i = self.info
        a = {"chains_columns": "start0..3, dir0..3, stride, steps; row = chain index",
             "lattice": [int(v) for v in i.lattice], "procs": [int(v) for v in i.procs],
             "nconf": int(i.nconf), "muon_mass_MeV": float(i.muon_mass),
             "lattice_spacing_fm": float(i.lattice_spacing), "xunit": float(i.xunit),
             "kernel": i.kernel,
             "flavour_order": "kernel_sum/kernel_sum[:,0] = operator 0, [:,1] = operator 1",
             "coordinate_ranges": "x, y, w, pair_w, pair_y: [0, L); yv, pair_yv: minimum image "
                                  "of y - x, pair_y - pair_w in [-L/2, L/2)",
             "container": "npz (the reference's HDF5 layout)"}
        if len(i.chains) == 1:  # as in files from before chain lists
            c = i.chains[0]
            a.update({"direction": list(c.direction), "origin": list(c.start), "stride": c.stride})
        return a

    @property
    def rows(self) -> int:
        return len(self._ks["chain"])

    @property
    def rows_2p2(self) -> int:
        return len(self._p22["chain"])

    def append(self, rows) -> None:
        """PairResult rows (driver.PairResult)."""
        for r in rows:
            self._ks["x"].append(r.x)
            self._ks["y"].append(r.y)
            self._ks["yv"].append(r.yv)
            self._ks["chain"].append(r.chain)
            self._ks["window"].append(r.window)
            self._ks["kernel_sum"].append(r.kernel_sum)
        self._appended()

    def append_2p2(self, rows) -> None:
        """Result2p2 rows (driver.Result2p2); needs RunInfo.with_2p2."""
        if not self.info.with_2p2:
            raise RuntimeError("ResultWriter: the run has no 2p2 group")
        for r in rows:
            self._p22["w"].append(r.w)
            self._p22["chain"].append(r.chain)
            self._p22["window"].append(r.window)
            self._p22["P1"].append(np.asarray(r.p1, dtype=np.float64).reshape(4, 4, 4, self.lmax))
            p234 = np.asarray(r.p234, dtype=np.float64).reshape(len(r.y), 5, 4, 4, 4)
            for t, (y, yv) in enumerate(zip(r.y, r.yv)):
                self._p22["pair_w"].append(r.w)
                self._p22["pair_y"].append(y)
                self._p22["pair_yv"].append(yv)
                self._p22["P234"].append(p234[t])
        self._appended()

    def _arrays(self):
        def ints(v, shape):
            return np.asarray(v, dtype=np.int32).reshape((-1,) + shape)

        def dbl(v, shape):
            return np.asarray(v, dtype=np.float64).reshape((-1,) + shape)

        k = self._ks
        out = {"kernel_sum/x": ints(k["x"], (4,)), "kernel_sum/y": ints(k["y"], (4,)),
               "kernel_sum/yv": ints(k["yv"], (4,)), "kernel_sum/chain": ints(k["chain"], ()),
               "kernel_sum/window": ints(k["window"], ()),
               "kernel_sum/kernel_sum": dbl(k["kernel_sum"], (2,))}
        if self.info.with_2p2:
            p = self._p22
            out.update({"2p2/w": ints(p["w"], (4,)), "2p2/chain": ints(p["chain"], ()),
                        "2p2/window": ints(p["window"], ()),
                        "2p2/P1": dbl(p["P1"], (4, 4, 4, self.lmax)),
                        "2p2/pair_w": ints(p["pair_w"], (4,)), "2p2/pair_y": ints(p["pair_y"], (4,)),
                        "2p2/pair_yv": ints(p["pair_yv"], (4,)),
                        "2p2/P234": dbl(p["P234"], (5, 4, 4, 4))})
        out["chains"] = np.asarray([list(c.start) + list(c.direction) + [c.stride, c.steps]
                                    for c in self.info.chains], dtype=np.int32).reshape(-1, 10)
        for g, a in self._attrs.items():
            out["attrs:" + g] = np.asarray(json.dumps(a))
        return out

    def _appended(self) -> None:
        self._pending += 1
        if self._pending >= self.flush_every:
            self._flush()

    def close(self) -> None:
        """Write what is pending (a no-op when every append was flushed)."""
        if self._pending:
            self._flush()

    def _flush(self) -> None:
        self._pending = 0
        tmp = self.path + ".tmp.npz"
        with open(tmp, "wb") as fh:
            np.savez(fh, **self._arrays())
        os.replace(tmp, self.path)


def read_results(path: str) -> dict:
    """The datasets ("group/name" -> array) and attributes ("attrs:<group>" ->
    dict) of a result file."""
    with np.load(path) as z:
        out = {}
        for k in z.files:
            out[k] = json.loads(str(z[k])) if k.startswith("attrs:") else z[k]
    return out


class TimingLog:
    """One CSV row per solve, per kernel sum and per 2+2 source
    (output.cpp:300-332): kind,chain,window,x0..x3,y0..y3,seconds,iterations.
    A solve leaves y empty; a kernel sum leaves iterations empty; a 2+2 row
    (kind 2p2) has the source as x and leaves y and iterations empty."""

    HEADER = "kind,chain,window,x0,x1,x2,x3,y0,y1,y2,y3,seconds,iterations\n"

    def __init__(self, path: str):
        self.fh = open(path, "w")
        self.fh.write(self.HEADER)
        self.fh.flush()

    def _row(self, kind, chain, window, x, y, seconds, iterations):
        xs = ",".join(str(int(a)) for a in x)
        ys = ",".join(str(int(a)) for a in y) if y is not None else ",,,"
        it = "" if iterations is None else str(int(iterations))
        self.fh.write(f"{kind},{chain},{window},{xs},{ys},{seconds:.6f},{it}\n")
        self.fh.flush()

    def solve(self, chain, window, site, seconds, iterations):
        self._row("solve", chain, window, site, None, seconds, iterations)

    def kernel_sum(self, chain, window, x, y, seconds):
        self._row("kernel_sum", chain, window, x, y, seconds, None)

    def pieces_2p2(self, chain, window, site, seconds):
        self._row("2p2", chain, window, site, None, seconds, None)

    def close(self):
        self.fh.close()
