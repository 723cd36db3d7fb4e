"""Generate the golden fixtures of the 2+2 pieces (tests/golden/reference_2p2.json).

Runs the reference's OWN 2+2 code -- kernels/hlbl_kernels/kernels.cu
(compute_2p2_gpu and its kernels) and Contractor::pieces_2p2
(src/contract.cpp:116-156) -- built as a host emulation by
oracle/ref_host/Makefile into oracle/_ref/libhlbl_ref_host.so. The emulation
runs each CUDA block as blockDim threads (kernel_pi synchronises its block,
kernel_p2x/p3/p4 reduce with warp shuffles), block after block. The QED
weight is the project's stand-in (include/hlbl_gb300_qed.h), as KQED is not
available.

Inputs are fill_random_block (src/provider.cpp:25-57), integer arithmetic
the tests regenerate bit-exactly, so only outputs are stored.

Usage (needs the reference sources, i.e. only where they are mounted):
    make -C oracle/ref_host REF=<reference checkout>
    python tests/golden/make_golden_2p2.py
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libhlbl_ref_host.so")
OUT = os.path.join(HERE, "reference_2p2.json")

I4 = C.c_int * 4
XUNIT_PHYS = 105.6583745 / 197.3269804 * 0.07957


def i4(v):
    return I4(*[int(a) for a in v])


def vp(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def load_ref():
    lib = C.CDLL(REF_LIB)
    lib.ref_pieces_2p2.restype = C.c_int
    lib.ref_pieces_2p2.argtypes = [I4, C.c_void_p, I4, C.c_void_p, C.c_int, C.c_double,
                                   C.c_void_p, C.c_void_p]
    lib.ref_compute_2p2.argtypes = [C.c_void_p, C.c_int, I4, C.c_void_p, C.c_int, C.c_double,
                                    I4, I4, I4, C.c_void_p, C.c_void_p]
    lib.ref_fill_random_block.argtypes = [I4, C.c_uint64, C.c_void_p]
    lib.ref_plan_2p2.restype = C.c_int
    lib.ref_plan_2p2.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                 I4, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                 C.c_void_p, C.c_int, C.c_void_p, C.c_char_p, C.c_int]
    return lib


def sign_vectors():
    return [[a, b, c, d] for a in (1, -1) for b in (1, -1) for c in (1, -1) for d in (1, -1)]


# plan_2p2 cases (schedule.cpp:284-347): (name, lattice, hs, stride, n_steps, origins, sources)
PLANS = [
    # all 16 h as 16 chains (the 24^3x48 multi-chain configuration's shape),
    # sources: solved sites, one given twice, one never solved
    ("16chains_l6", [6, 6, 6, 6], sign_vectors(), 1, 1, [[0, 0, 0, 0]] * 16,
     [[1, 1, 1, 1], [0, 0, 0, 0], [5, 5, 5, 5], [7, 1, 1, 1], [3, 3, 3, 3], [2, 0, 1, 5]]),
    # three chains whose windows wrap onto each other; more than 10 warnings
    ("3chains_wrap", [8, 4, 4, 4], [[1, 1, 1, 1], [1, -1, 1, -1], [-1, 1, 1, 1]], 2, 2,
     [[0, 0, 0, 0], [4, 0, 0, 0], [2, 2, 2, 2]],
     [[2, 2, 2, 2], [6, 2, 2, 2], [0, 1, 0, 1], [4, 0, 0, 0], [12, 4, 4, 4]]),
]


def ref_plan(lib, lat, hs, stride, n_steps, origins, sources):
    n = len(hs)
    h = np.ascontiguousarray(np.asarray(hs, dtype=np.int32))
    o = np.ascontiguousarray(np.asarray(origins, dtype=np.int32))
    sv = np.ascontiguousarray(np.asarray(sources, dtype=np.int32).reshape(-1, 4))
    at = np.zeros((4096, 6), dtype=np.int32)
    ns = np.zeros((4096, 6), dtype=np.int32)
    un = np.zeros(256, dtype=np.int32)
    n_at, n_ns, n_un = C.c_int(), C.c_int(), C.c_int()
    rep = C.create_string_buffer(1 << 16)
    rc = lib.ref_plan_2p2(n, vp(h), stride, n_steps, vp(o), len(sv), vp(sv), i4(lat), vp(at), 4096,
                          C.byref(n_at), vp(ns), 4096, C.byref(n_ns), vp(un), 256, C.byref(n_un), rep,
                          1 << 16)
    assert rc == 0
    return {"at": at[:n_at.value].tolist(), "not_sources": ns[:n_ns.value].tolist(),
            "unsolved": un[:n_un.value].tolist(), "report": rep.value.decode().splitlines()}


def volume(v):
    return int(v[0]) * int(v[1]) * int(v[2]) * int(v[3])


def block(lib, lat, seed):
    out = np.zeros(2 * 12 * 24 * volume(lat))
    lib.ref_fill_random_block(i4(lat), C.c_uint64(seed), vp(out))
    return out


# Contractor::pieces_2p2 cases (flavour 0, per-target layout [n_y][5][64]):
# (name, lattice, seed, gsw, targets, xunit)
PIECES = [
    # a target at the source itself (y = 0) and one at L/2 in every direction
    ("l4", [4, 4, 4, 4], 3, [1, 0, 2, 3], [[1, 2, 3, 0], [1, 0, 2, 3], [3, 2, 0, 1]], 0.5),
    # odd and unequal extents (L/2 rounds down), Lmax = 6
    ("odd_5x3x4x6", [5, 3, 4, 6], 5, [4, 1, 0, 5], [[0, 0, 0, 0], [4, 2, 3, 1], [2, 1, 2, 3]], 0.7),
    # physical xunit, the driver test lattice, four targets
    ("l6_phys", [6, 6, 6, 6], 7, [0, 0, 0, 0],
     [[1, 1, 1, 1], [3, 3, 3, 3], [5, 0, 2, 4], [0, 3, 0, 3]], XUNIT_PHYS),
]


def main() -> int:
    if not os.path.exists(REF_LIB):
        print("missing", REF_LIB, "- run make -C oracle/ref_host first", file=sys.stderr)
        return 1
    lib = load_ref()
    out: dict = {"what": "outputs of the reference's own 2+2 code (kernels.cu compute_2p2_gpu, "
                         "contract.cpp pieces_2p2; host emulation, stand-in QED weight, "
                         "Lambda=0.4)",
                 "generator": "tests/golden/make_golden_2p2.py",
                 "input": "fill_random_block(lattice, seed)"}
    cases = []
    for name, lat, seed, gsw, targets, xu in PIECES:
        t0 = time.time()
        fwd = block(lib, lat, seed)
        lmax = max(lat)
        tg = np.ascontiguousarray(np.asarray(targets, dtype=np.int32))
        p1 = np.zeros(64 * lmax)
        p234 = np.zeros(len(targets) * 5 * 64)
        rc = lib.ref_pieces_2p2(i4(lat), vp(fwd), i4(gsw), vp(tg), len(targets), C.c_double(xu),
                                vp(p1), vp(p234))
        assert rc == 0, name
        cases.append({"name": name, "lattice": lat, "seed": seed, "gsw": gsw, "targets": targets,
                      "xunit": xu, "p1": p1.tolist(), "p234": p234.tolist()})
        print(name, "%.1f s" % (time.time() - t0), flush=True)
    out["pieces_2p2"] = cases

    # compute_2p2_gpu itself (its [5][n_y][64] layout), flavour 1, and its
    # per-rank partials on a 2-rank split along t of an 8x4x4x4 lattice
    glob, loc = [8, 4, 4, 4], [4, 4, 4, 4]
    seed, gsw, targets, xu = 21, [5, 1, 2, 3], [[0, 0, 0, 0], [6, 3, 1, 2]], 0.6
    full = block(lib, glob, seed)
    V, Vl = volume(glob), volume(loc)
    tg = np.ascontiguousarray(np.asarray(targets, dtype=np.int32))
    ranks = []
    for r in (0, 1):
        sl = np.ascontiguousarray(full.reshape(2, 12, V, 24)[:, :, r * Vl:(r + 1) * Vl, :])
        p1 = np.zeros(64 * 8)
        p234 = np.zeros(len(targets) * 5 * 64)
        lib.ref_compute_2p2(vp(sl), 1, i4(gsw), vp(tg), len(targets), C.c_double(xu),
                            i4([r, 0, 0, 0]), i4(glob), i4(loc), vp(p1), vp(p234))
        ranks.append({"proc_coords": [r, 0, 0, 0], "p1": p1.tolist(), "p234_raw": p234.tolist()})
        print("split rank", r, flush=True)
    out["compute_2p2_split"] = {"global": glob, "local": loc, "seed": seed, "gsw": gsw,
                                "targets": targets, "xunit": xu, "iflavor": 1,
                                "layout": "p1 [4][4][4][Lmax]; p234_raw [5][n_y][64]",
                                "ranks": ranks}
    plans = []
    for name, lat, hs, stride, n_steps, origins, sources in PLANS:
        r = ref_plan(lib, lat, hs, stride, n_steps, origins, sources)
        plans.append({"name": name, "lattice": lat, "h": hs, "stride": stride, "n_steps": n_steps,
                      "origins": origins, "sources": sources, **r})
        print("plan", name, len(r["at"]), "at,", len(r["not_sources"]), "not sources,",
              len(r["unsolved"]), "unsolved", flush=True)
    out["plan_2p2"] = plans
    with open(OUT, "w") as fh:
        json.dump(out, fh)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main())
