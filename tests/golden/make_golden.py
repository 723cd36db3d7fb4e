"""Generate the golden fixtures that pin the oracle.

Runs the reference's OWN sources (kernels/cuda_lattice.cu, src/contract.cpp,
src/provider.cpp, src/gamma.cpp, src/schedule.cpp), built as a host emulation
by oracle/ref_host/Makefile into oracle/_ref/libhlbl_ref_host.so, on small
lattices, and writes what they return to tests/golden/*.json. The QED weight
in these runs is the project's stand-in (include/hlbl_gb300_qed.h) because
KQED is not available; the reference's own golden values
(sanity_check/test_contract_random.cpp:58) need real KQED and cannot be
reproduced.

Inputs are the reference's uniform random fixture (fill_random_block,
src/provider.cpp:25-57), which is pure integer arithmetic, so the tests can
regenerate them bit-exactly instead of storing them.

Usage (needs the reference sources, i.e. only where they are mounted):
    make -C oracle/ref_host REF=<reference checkout>
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libhlbl_ref_host.so")

I4 = C.c_int * 4


def i4(v):
    return I4(*[int(a) for a in v])


def vp(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def load_ref():
    lib = C.CDLL(REF_LIB)
    lib.ref_kernel_sum.restype = C.c_int
    lib.ref_kernel_sum.argtypes = [I4, C.c_void_p, C.c_void_p, I4, I4, C.c_double, C.c_void_p]
    lib.ref_dzu_dzsu.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                 I4, I4, I4, I4]
    lib.ref_4pt.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                            C.c_int, I4, I4, C.c_double, I4, I4, I4]
    lib.ref_fill_random_block.argtypes = [I4, C.c_uint64, C.c_void_p]
    lib.ref_random_provider.argtypes = [I4, C.c_uint64, I4, C.c_void_p]
    lib.ref_apply_gamma.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
    lib.ref_schedule_pairs.restype = C.c_int
    lib.ref_schedule_pairs.argtypes = [I4, C.c_int, C.c_int, I4, C.c_void_p, C.c_int]
    lib.ref_schedule_stats.argtypes = [I4, C.c_int, C.c_int, C.c_void_p]
    return lib


def volume(v):
    return int(v[0]) * int(v[1]) * int(v[2]) * int(v[3])


def ref_block(lib, local, seed):
    out = np.zeros(2 * 12 * 24 * volume(local))
    lib.ref_fill_random_block(i4(local), C.c_uint64(seed), vp(out))
    return out


def ref_source_block(lib, local, seed, gsx):
    out = np.zeros(2 * 12 * 24 * volume(local))
    lib.ref_random_provider(i4(local), C.c_uint64(seed), i4(gsx), vp(out))
    return out


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


# Kernel-sum cases: (name, lattice (T,LX,LY,LZ), input spec, gsx, yv, xunit).
# Input spec ("seeds", s_src, s_y): fill_random_block with those seeds, as in
# test_contract_random.cpp:42-46; ("provider", run_seed, x, y): the blocks
# RandomProvider::compute makes for source positions x and y.
XUNIT_PHYS = 105.6583745 / 197.3269804 * 0.07957  # test_driver_random.cpp inputs
CASES = [
    # the reference's golden configuration (test_contract_random.cpp:37-51)
    ("golden_8x4x4x4", [8, 4, 4, 4], ("seeds", 1, 2), [0, 0, 0, 0], [1, 1, 1, 1], 1.0),
    # gsx off the origin; yv with a component at L/2 (maps to -L/2)
    ("l4_halfL", [4, 4, 4, 4], ("seeds", 3, 4), [1, 2, 3, 0], [2, -1, 2, 1], 1.0),
    # odd and unequal extents (L/2 rounds down; zerohalf never hits)
    ("odd_5x3x4x6", [5, 3, 4, 6], ("seeds", 5, 6), [4, 1, 0, 5], [-2, 1, 2, -3], 0.7),
    # the driver test lattice with the provider's per-source blocks
    ("driver_6x6x6x6", [6, 6, 6, 6], ("provider", 7, [0, 0, 0, 0], [1, 1, 1, 1]),
     [0, 0, 0, 0], [1, 1, 1, 1], XUNIT_PHYS),
    ("driver_6x6x6x6_b", [6, 6, 6, 6], ("provider", 7, [1, 1, 1, 1], [0, 2, 0, 2]),
     [1, 1, 1, 1], [-1, 1, -1, 1], XUNIT_PHYS),
    # yv wraps (negative and beyond L): the kernels map it themselves
    ("wrap_8x4x4x4", [8, 4, 4, 4], ("seeds", 11, 12), [7, 3, 0, 2], [-7, 5, -2, 2], 0.5),
]


def ref_insert_gammas(lib, dzu, dzsu):
    """g_dzu, g_dzsu from pass 1's sums by the reference's apply_gamma
    (src/gamma.cpp), in the order of contract.cpp:58-77."""
    g_dzu, g_dzsu = np.zeros(6912), np.zeros(4608)
    for src, dst, n in ((dzu, g_dzu, 6), (dzsu, g_dzsu, 4)):
        for k in range(n):
            for ia in range(12):
                for mu in range(4):
                    t = np.ascontiguousarray(src[(k * 12 + ia) * 24:(k * 12 + ia + 1) * 24])
                    t5 = np.zeros(24)
                    lib.ref_apply_gamma(5, vp(t), vp(t5))
                    o = np.zeros(24)
                    lib.ref_apply_gamma(mu, vp(t5), vp(o))
                    dst[((k * 4 + mu) * 12 + ia) * 24:((k * 4 + mu) * 12 + ia + 1) * 24] = o
    return g_dzu, g_dzsu


def inputs(lib, lat, spec):
    if spec[0] == "seeds":
        return ref_block(lib, lat, spec[1]), ref_block(lib, lat, spec[2])
    _, seed, gx, gy = spec
    return ref_source_block(lib, lat, seed, gx), ref_source_block(lib, lat, seed, gy)


def main() -> int:
    if not os.path.exists(REF_LIB):
        print("missing", REF_LIB, "- run make -C oracle/ref_host first", file=sys.stderr)
        return 1
    lib = load_ref()
    out: dict = {"what": "outputs of the reference's own sources (host emulation, "
                         "stand-in QED weight, Lambda=0.4)",
                 "generator": "tests/golden/make_golden.py"}

    # gamma matrices: columns are images of unit 24-vectors
    gam = {}
    for g in (0, 1, 2, 3, 5):
        m = np.zeros((24, 24))
        for j in range(24):
            e = np.zeros(24)
            e[j] = 1.0
            o = np.zeros(24)
            lib.ref_apply_gamma(g, vp(e), vp(o))
            m[:, j] = o
        gam[str(g)] = m.astype(int).tolist()
    out["gamma"] = gam

    # fixtures: checksums and a few values
    blk = ref_block(lib, [8, 4, 4, 4], 1)
    out["fill_random_block"] = {"lattice": [8, 4, 4, 4], "seed": 1, "sha256": sha(blk),
                                "first": blk[:8].tolist(), "index_1000": blk[1000]}
    pb = ref_source_block(lib, [6, 6, 6, 6], 7, [1, 1, 1, 1])
    out["random_provider"] = {"lattice": [6, 6, 6, 6], "seed": 7, "gsx": [1, 1, 1, 1],
                              "sha256": sha(pb)}

    # kernel sums through Contractor::kernel_sum
    cases = []
    for name, lat, spec, gsx, yv, xu in CASES:
        src, y = inputs(lib, lat, spec)
        r = (C.c_double * 2)()
        rc = lib.ref_kernel_sum(i4(lat), vp(src), vp(y), i4(gsx), i4(yv), C.c_double(xu), r)
        assert rc == 0, name
        cases.append({"name": name, "lattice": lat, "input": list(spec), "gsx": gsx, "yv": yv,
                      "xunit": xu, "kernel_sum": [r[0], r[1]]})
        print(name, r[0], r[1])
    out["kernel_sum"] = cases

    # pass-1 output and pass-2 sum of one flavour, for the per-pass tests
    lat, gsx = [4, 4, 4, 4], [1, 2, 3, 0]
    src, y = ref_block(lib, lat, 3), ref_block(lib, lat, 4)
    passes = []
    for f in (0, 1):
        dzu, dzsu = np.zeros(1728), np.zeros(1152)
        lib.ref_dzu_dzsu(vp(dzu), vp(dzsu), vp(src), vp(y), f, i4([0] * 4), i4(gsx), i4(lat),
                         i4(lat))
        passes.append({"flavour": f, "dzu": dzu.tolist(), "dzsu": dzsu.tolist()})
    out["pass1"] = {"lattice": lat, "seeds": [3, 4], "gsx": gsx, "flavours": passes}

    # two-rank split along t of a 8x4x4x4 lattice: each rank's partial sums
    glob, loc = [8, 4, 4, 4], [4, 4, 4, 4]
    full_src, full_y = ref_block(lib, glob, 21), ref_block(lib, glob, 22)
    V, Vl = volume(glob), volume(loc)
    gsx2, yv2 = [5, 1, 2, 3], [1, -1, 1, -1]
    ranks = []
    for r in (0, 1):
        sl = [full_src.reshape(2, 12, V, 24)[:, :, r * Vl:(r + 1) * Vl, :].copy(),
              full_y.reshape(2, 12, V, 24)[:, :, r * Vl:(r + 1) * Vl, :].copy()]
        dz = []
        for f in (0, 1):
            dzu, dzsu = np.zeros(1728), np.zeros(1152)
            lib.ref_dzu_dzsu(vp(dzu), vp(dzsu), vp(sl[0]), vp(sl[1]), f, i4([r, 0, 0, 0]),
                             i4(gsx2), i4(glob), i4(loc))
            dz.append((dzu, dzsu))
        ranks.append((sl, dz))
    split = {"global": glob, "local": loc, "seeds": [21, 22], "gsx": gsx2, "yv": yv2,
             "xunit": 1.0, "ranks": []}
    # the all-reduced pass-1 sums, then each rank's pass-2 partial
    for r in (0, 1):
        sl = ranks[r][0]
        parts = []
        for f in (0, 1):
            dzu = ranks[0][1][f][0] + ranks[1][1][f][0]
            dzsu = ranks[0][1][f][1] + ranks[1][1][f][1]
            g_dzu, g_dzsu = ref_insert_gammas(lib, dzu, dzsu)
            ks = np.zeros(1)
            lib.ref_4pt(vp(ks), vp(g_dzu), vp(g_dzsu), vp(sl[0]), vp(sl[1]), f, i4([r, 0, 0, 0]),
                        i4(gsx2), C.c_double(1.0), i4(yv2), i4(glob), i4(loc))
            parts.append(float(ks[0]))
        split["ranks"].append({"proc_coords": [r, 0, 0, 0], "kernel_sum_partial": parts})
    r = (C.c_double * 2)()
    lib.ref_kernel_sum(i4(glob), vp(full_src), vp(full_y), i4(gsx2), i4(yv2), C.c_double(1.0), r)
    split["single_rank_kernel_sum"] = [r[0], r[1]]
    out["two_rank_split"] = split

    # schedules: pair lists and interleaved statistics (src/schedule.cpp)
    sched = []
    for h, stride, k in (([1, 1, 1, 1], 1, 1), ([1, -1, 1, -1], 2, 4), ([-1, 1, 1, 1], 4, 8)):
        buf = np.zeros(9 * 4096, dtype=np.int32)
        n = lib.ref_schedule_pairs(i4(h), stride, k, i4([0] * 4), vp(buf), 4096)
        assert n > 0
        sched.append({"h": h, "stride": stride, "steps": k,
                      "pairs": buf[:9 * n].reshape(n, 9).tolist()})
    out["schedule"] = sched
    stats = []
    for a in (-1, 1):
        for b in (-1, 1):
            for c in (-1, 1):
                for d in (-1, 1):
                    for k in (1, 2, 5):
                        s = np.zeros(3, dtype=np.int64)
                        lib.ref_schedule_stats(i4([a, b, c, d]), 4, k, vp(s))
                        stats.append({"h": [a, b, c, d], "stride": 4, "steps": k,
                                      "propagators": int(s[0]), "pairs": int(s[1]),
                                      "peak": int(s[2])})
    out["schedule_stats"] = stats

    path = os.path.join(HERE, "reference_host_emulation.json")
    with open(path, "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote", path, os.path.getsize(path), "bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main())
