"""HLBL_QEDK_KQED on the GPU: the library linked with a KQED install (the
stand-in install of tests/kqed_build.py, whose device QED_Mkernel_L2 is the
project's stand-in weight, compiled apart as a real KQED's would be) weights
through the generic paths with that separately linked device function. Its
kernel sums and 2+2 pieces must equal the reference's own results with the
same weight (tests/golden): FP64 1e-12, FP32 1e-4 per pair, 2+2 rows FP64
1e-12. Runs in a child process, which loads that build of the library."""
import json
import os
import subprocess
import sys

import pytest

import kqed_build as K

pytestmark = pytest.mark.gpu

CHILD = r'''
import json, sys
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[2])
import numpy as np, torch
import support as S, hlbl_gb300 as hg
out = {"kernel_sum": [], "pieces": []}
for case in S.golden()["kernel_sum"]:
    src, y = S.case_inputs(case)
    with hg.Contractor(case["lattice"]) as c:
        c.set_qed_kernel(hg.QED_KQED)
        d_src, d_y = torch.from_numpy(src).cuda(), torch.from_numpy(y).cuda()
        a = c.kernel_sum(d_src, d_y, case["gsx"], case["yv"], case["xunit"], hg.FP64)
        b = c.kernel_sum(d_src, d_y, case["gsx"], case["yv"], case["xunit"], hg.FP32)
    out["kernel_sum"].append([list(a), list(b), case["kernel_sum"]])
g2 = json.load(open(sys.argv[3]))["pieces_2p2"][0]
fwd = S.random_block(g2["lattice"], g2["seed"])
with hg.Contractor(g2["lattice"]) as c:
    c.set_qed_kernel(hg.QED_KQED)
    p = c.pieces_2p2(torch.from_numpy(fwd).cuda(), g2["gsw"], g2["targets"], g2["xunit"], hg.FP64)
out["pieces"] = [np.asarray(p.p234).ravel().tolist(), g2["p234"]]
print("RESULT " + json.dumps(out))
'''


def test_kqed_linked_library_matches_reference():
    lib = K.build_linked_library()
    env = dict(os.environ, HLBL_GB300_LIB=lib)
    tests = os.path.dirname(os.path.abspath(__file__))
    r = subprocess.run([sys.executable, "-c", CHILD, K.ROOT, tests,
                        os.path.join(tests, "golden", "reference_2p2.json")],
                       capture_output=True, text=True, env=env, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    res = json.loads(next(ln for ln in r.stdout.splitlines() if ln.startswith("RESULT "))[7:])
    import numpy as np

    import support as S

    for f64, f32, want in res["kernel_sum"]:
        assert S.rel_err(f64, want) <= 1e-12, (f64, want)
        assert S.pair_rel_err(f32, want) <= 1e-4, (f32, want)
    got, want = (np.asarray(v).reshape(-1, 5, 64) for v in res["pieces"])
    for t in range(want.shape[0]):
        for g in range(5):
            scale = max(np.abs(want[t, g]).max(), 1e-300)
            assert np.abs(got[t, g] - want[t, g]).max() <= 1e-12 * scale, (t, g)
