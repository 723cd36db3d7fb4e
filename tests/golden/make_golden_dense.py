"""Golden fixtures for the dense test weight (a QED tensor with no closed form).

Runs the reference's OWN sources (Contractor::kernel_sum, cu_dzu_dzsu +
cu_4pt_contraction, Contractor::pieces_2p2), built as a host emulation by
oracle/ref_host/Makefile into oracle/_ref/libhlbl_ref_host.so, with KQED's
QED_Mkernel_L2 served by the dense test weight of include/hlbl_gb300_qed.h
(every entry of kerv[6][4][4][4] its own seeded combination of smooth
functions, seed tests/support.py:DENSE_SEED), and writes what they return to
tests/golden/reference_dense_qed.json. These pin the oracle and the library's
generic-weight paths for a tensor that no contraction shortcut applies to.

Usage (needs the reference sources, i.e. only where they are mounted):
    make -C oracle/ref_host REF=<reference checkout>
    python tests/golden/make_golden_dense.py
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
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import make_golden as mg  # noqa: E402
import make_golden_2p2 as m2  # noqa: E402
from support import DENSE_SEED  # noqa: E402

OUT = os.path.join(HERE, "reference_dense_qed.json")


def main() -> int:
    if not os.path.exists(mg.REF_LIB):
        print("missing", mg.REF_LIB, "- run make -C oracle/ref_host first", file=sys.stderr)
        return 1
    lib = mg.load_ref()
    lib2 = m2.load_ref()
    lib.ref_set_qed_dense.argtypes = [C.c_int, C.c_ulonglong]
    lib.ref_set_qed_dense(1, DENSE_SEED)
    out: dict = {"what": "outputs of the reference's own sources (host emulation) with "
                         "QED_Mkernel_L2 served by the dense test weight",
                 "generator": "tests/golden/make_golden_dense.py", "dense_seed": DENSE_SEED}
    cases = []
    for name, lat, spec, gsx, yv, xu in mg.CASES:
        src, y = mg.inputs(lib, lat, spec)
        r = (C.c_double * 2)()
        rc = lib.ref_kernel_sum(mg.i4(lat), mg.vp(src), mg.vp(y), mg.i4(gsx), mg.i4(yv),
                                C.c_double(xu), r)
        assert rc == 0, name
        cases.append({"name": name, "lattice": lat, "input": list(spec), "gsx": gsx, "yv": yv,
                      "xunit": xu, "kernel_sum": [r[0], r[1]]})
        print(name, r[0], r[1], flush=True)
    out["kernel_sum"] = cases

    # one flavour's pass 2 alone (cu_4pt_contraction) from the reference's own
    # pass-1 sums and gamma insertion
    lat, gsx, yv, xu = [4, 4, 4, 4], [1, 2, 3, 0], [2, -1, 2, 1], 0.8
    src, y = mg.ref_block(lib, lat, 3), mg.ref_block(lib, lat, 4)
    per_f = []
    for f in (0, 1):
        dzu, dzsu = np.zeros(1728), np.zeros(1152)
        lib.ref_dzu_dzsu(mg.vp(dzu), mg.vp(dzsu), mg.vp(src), mg.vp(y), f, mg.i4([0] * 4),
                         mg.i4(gsx), mg.i4(lat), mg.i4(lat))
        g_dzu, g_dzsu = mg.ref_insert_gammas(lib, dzu, dzsu)
        ks = np.zeros(1)
        lib.ref_4pt(mg.vp(ks), mg.vp(g_dzu), mg.vp(g_dzsu), mg.vp(src), mg.vp(y), f,
                    mg.i4([0] * 4), mg.i4(gsx), C.c_double(xu), mg.i4(yv), mg.i4(lat), mg.i4(lat))
        per_f.append(float(ks[0]))
    out["pass2"] = {"lattice": lat, "seeds": [3, 4], "gsx": gsx, "yv": yv, "xunit": xu,
                    "kernel_sum_per_flavour": per_f}

    # Contractor::pieces_2p2 (flavour 0, per-target layout [n_y][5][64])
    lib2.ref_set_qed_dense.argtypes = [C.c_int, C.c_ulonglong]
    lib2.ref_set_qed_dense(1, DENSE_SEED)
    pcs = []
    for name, lat, seed, gsw, targets, xu in m2.PIECES[:2]:
        t0 = time.time()
        fwd = m2.block(lib2, lat, seed)
        lmax = max(lat)
        tg = np.ascontiguousarray(np.asarray(targets, dtype=np.int32))
        p1 = np.zeros(64 * lmax)
        p234 = np.zeros(len(targets) * 5 * 64)
        rc = lib2.ref_pieces_2p2(m2.i4(lat), m2.vp(fwd), m2.i4(gsw), m2.vp(tg), len(targets),
                                 C.c_double(xu), m2.vp(p1), m2.vp(p234))
        assert rc == 0, name
        pcs.append({"name": name, "lattice": lat, "seed": seed, "gsw": gsw, "targets": targets,
                    "xunit": xu, "p1": p1.tolist(), "p234": p234.tolist()})
        print(name, "%.1f s" % (time.time() - t0), flush=True)
    out["pieces_2p2"] = pcs
    lib.ref_set_qed_dense(0, 0)
    with open(OUT, "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main())
