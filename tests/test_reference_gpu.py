"""The library against the reference's OWN kernels on the GPU: its Contractor
(src/contract.cpp) driving kernels/cuda_lattice.cu and
kernels/hlbl_kernels/kernels.cu, built for sm_103a by oracle/ref_gpu with
KQED's QED_Mkernel_L2 served on the device by the project's test weights.
First the reference's GPU build against its own host-emulation goldens (so
the build itself is pinned), then the library's FP64 path against it.

Tolerance 1e-10 relative per flavour: the reference adds its per-site
values with FP64 atomics in no fixed order and pins its own results to 1e-10
for that reason (sanity_check/test_contract_random.cpp:55-66). Skipped where
the reference's GPU build is absent (no staged copy of its sources)."""
import json
import os

import numpy as np
import pytest

import support as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
TOL_REF = 1e-10

if S.ref_gpu_lib() is None:
    pytest.skip("the reference's GPU build (oracle/_ref/gpu) is absent", allow_module_level=True)

with open(os.path.join(os.path.dirname(__file__), "golden", "reference_dense_qed.json")) as fh:
    GD = json.load(fh)
with open(os.path.join(os.path.dirname(__file__), "golden", "reference_2p2.json")) as fh:
    G2 = json.load(fh)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("dense", [False, True], ids=["standin", "dense"])
def test_reference_gpu_build_matches_its_host_emulation(dense):
    cases = GD["kernel_sum"] if dense else S.golden()["kernel_sum"]
    for case in cases:
        src, y = S.case_inputs(case)
        with S.RefGpu(case["lattice"], dense=dense) as r:
            got = r.kernel_sum(dev(src), dev(y), case["gsx"], case["yv"], case["xunit"])
        assert S.rel_err(got, case["kernel_sum"]) <= TOL_REF, (case["name"], got, case["kernel_sum"])


@pytest.mark.parametrize("dense", [False, True], ids=["standin", "dense"])
@pytest.mark.parametrize("lat", [(8, 8, 8, 8), (16, 8, 8, 12)])
def test_fp64_path_matches_reference_kernels(lat, dense):
    import hlbl_gb300 as hg

    xu = hg.xunit(105.658, 0.1)
    src, y = S.gaussian_block(lat, 301), S.gaussian_block(lat, 302)
    gsx, yv = (3, 1, 7, 2), (2, -3, 1, 4)
    d_src, d_y = dev(src), dev(y)
    with S.RefGpu(lat, dense=dense) as r:
        want = r.kernel_sum(d_src, d_y, gsx, yv, xu)
    with hg.Contractor(lat) as c:
        if dense:
            c.set_qed_kernel(hg.QED_DENSE, S.DENSE_SEED)
        got64 = c.kernel_sum(d_src, d_y, gsx, yv, xu, hg.FP64)
        got32 = c.kernel_sum(d_src, d_y, gsx, yv, xu, hg.FP32)
    assert S.rel_err(got64, want) <= TOL_REF, (got64, want)
    assert S.pair_rel_err(got32, want) <= 1e-4, (got32, want)


def test_reference_gpu_pieces_2p2_match_host_emulation_and_library():
    import hlbl_gb300 as hg

    for case in G2["pieces_2p2"][:2]:
        lat = case["lattice"]
        fwd = dev(S.random_block(lat, case["seed"]))
        with S.RefGpu(lat) as r:
            p1, p234 = r.pieces_2p2(fwd, case["gsw"], case["targets"], case["xunit"], max(lat))
        ref = np.asarray(case["p234"]).reshape(-1, 5, 64)
        with hg.Contractor(lat) as c:
            ours = c.pieces_2p2(fwd, case["gsw"], case["targets"], case["xunit"], hg.FP64)
        o234 = np.asarray(ours.p234).reshape(-1, 5, 64)
        scale = lambda a: max(np.max(np.abs(a)), 1e-300)
        assert np.max(np.abs(p1 - np.asarray(case["p1"]))) <= TOL_REF * scale(case["p1"])
        for t in range(ref.shape[0]):
            for g in range(5):
                assert np.max(np.abs(p234[t, g] - ref[t, g])) <= TOL_REF * scale(ref[t, g]), (t, g)
                assert np.max(np.abs(o234[t, g] - p234[t, g])) <= TOL_REF * scale(p234[t, g]), (t, g)


@pytest.mark.parametrize("dense", [False, True], ids=["standin", "dense"])
def test_config1_chain_matches_reference_kernels(dense):
    """The 8^3 x 16 chain (stride 1, h = (1,1,1,1), K = 1: 31 propagators, 80
    pairs x 2 flavours) through the library's driver on the host cache, the
    reference's loop (each source's pairs right after its solve, FP64), and
    every pair's sums against the reference's own kernels on the same blocks."""
    import hlbl_gb300 as hg
    from hlbl_gb300 import schedule
    from hlbl_gb300.cache import PropagatorCache, TorchBuffers
    from hlbl_gb300.driver import run_chain

    lat = (16, 8, 8, 8)
    xu = hg.xunit(105.658, 0.1)
    steps = schedule.build_schedule((1, 1, 1, 1), 1, 1)
    blocks = {}

    def block(site):
        site = tuple(site)
        if site not in blocks:
            blocks[site] = S.gaussian_block(lat, S.source_seed(1234, site))
        return blocks[site]

    with hg.Contractor(lat) as c:
        if dense:
            c.set_qed_kernel(hg.QED_DENSE, S.DENSE_SEED)

        def provider(site, dest):
            dest.copy_(torch.from_numpy(block(site)))

        res, st = run_chain(steps, lat, xu, provider, c, PropagatorCache("host", c.block_length, TorchBuffers(c)),
                            precision=hg.FP64)
    assert len(res) == 80 and st.positions_solved == 31
    worst = 0.0
    with S.RefGpu(lat, dense=dense) as r:
        for p in res:
            want = r.kernel_sum(dev(block(p.x)), dev(block(p.y)), p.x, p.yv, xu)
            worst = max(worst, S.rel_err(p.kernel_sum, want))
    assert worst <= TOL_REF, worst
