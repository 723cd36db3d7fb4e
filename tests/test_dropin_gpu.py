"""The reference's own driver loop (run_chains, src/driver.cpp) on the library:
tests/dropin/run_chains_main.cpp runs it on the configuration of
sanity_check/test_driver_random.cpp (6^4, stride 1, two steps, 2+2 sources)
with the device and the host cache, once linked with the reference's own
kernels (built for sm_103a by oracle/ref_gpu) and once with the library's
drop-in launchers. The pair lists, cache peaks and 2+2 sources must be the
same, and every kernel sum and 2+2 piece equal to 1e-10 relative (the
reference's own tolerance for its unordered FP64 atomics,
sanity_check/test_contract_random.cpp:55-66). Skipped where the reference's
GPU build is absent."""
import json
import subprocess

import numpy as np
import pytest

import dropin_build as D
import support as S

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.fixture(scope="module")
def runs():
    if S.ref_gpu_lib() is None or D.sources() is None:
        pytest.skip("the reference's GPU build or its sources are absent")
    out = {}
    for variant in ("ref", "gb300"):
        exe = D.build(variant)
        path = exe + ".json"
        r = subprocess.run([exe, path], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
        with open(path) as fh:
            out[variant] = {x["run"]: x for x in json.load(fh)}
    return out


@pytest.mark.parametrize("cache", ["device_cache", "host_cache"])
def test_reference_driver_on_the_library_matches_its_own_kernels(runs, cache):
    a, b = runs["gb300"][cache], runs["ref"][cache]
    for k in ("pairs", "cache_peak", "positions_solved"):
        assert a[k] == b[k], k
    assert a["pairs"] == len(a["kernel_sums"]) > 0
    for ra, rb in zip(a["kernel_sums"], b["kernel_sums"]):
        assert ra[:4] == rb[:4]  # x, y, chain, window: the same pair in the same order
        assert S.rel_err(ra[4:], rb[4:]) <= TOL, (ra, rb)
    assert len(a["pieces_2p2"]) == len(b["pieces_2p2"]) == 3
    for pa, pb in zip(a["pieces_2p2"], b["pieces_2p2"]):
        assert pa["w"] == pb["w"]
        for key in ("p1", "p234"):
            x, y = np.asarray(pa[key]), np.asarray(pb[key])
            assert np.max(np.abs(x - y)) <= TOL * np.max(np.abs(y)), key


def test_device_and_host_cache_agree_on_the_library(runs):
    """test_driver_random.cpp:210-220: the two caches give the same sums."""
    a, b = runs["gb300"]["device_cache"], runs["gb300"]["host_cache"]
    assert [r[:4] for r in a["kernel_sums"]] == [r[:4] for r in b["kernel_sums"]]
    for ra, rb in zip(a["kernel_sums"], b["kernel_sums"]):
        assert ra[4:] == rb[4:]  # same inputs, fixed-order reductions: bit-identical
