"""The learned QED weight on the GPU: its training gradients and its inference
kernel against the CPU oracle of the network (oracle/mlp_oracle.py), what
training gains over the coarse quadrature it corrects, and kernel sums with
it against the exact weight."""
import os
import sys

import numpy as np
import pytest

import support as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
sys.path.insert(0, os.path.join(S.ROOT, "oracle"))
import mlp_oracle as M  # noqa: E402


@pytest.fixture(scope="module")
def sur():
    from hlbl_gb300.surrogate import Surrogate

    s = Surrogate(seed=11)
    yield s
    s.close()


def _rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_gradients_match_oracle(sur):
    rng = np.random.default_rng(5)
    p, _ = sur.params()
    x = rng.uniform(-1, 1, (512, 3)).astype(np.float32)
    t = rng.normal(0, 1, (512, 6)).astype(np.float32)
    loss, g = sur.gradients(x, t)
    loss_o, g_o = M.loss_and_grad(p.astype(np.float64), x, t, round_bf16=True)
    assert abs(loss - loss_o) <= 1e-3 * abs(loss_o)
    o = 0
    for name, shp in M.SHAPES:
        n = int(np.prod(shp))
        # BF16 operands, FP32 accumulation (GPU) vs FP64 accumulation (oracle)
        assert _rel_l2(g[o:o + n], g_o[o:o + n]) <= 2e-2, name
        o += n


def test_inference_kernel_matches_oracle(sur):
    rng = np.random.default_rng(6)
    p, _ = sur.params()
    x = rng.uniform(-1, 1, (1000, 3)).astype(np.float32)
    got = sur.eval(x)
    want = M.forward(p.astype(np.float64), x, round_bf16=True)
    assert np.max(np.abs(got - want)) <= 1e-2 * np.max(np.abs(want))


def test_training_gains_over_base_and_keeps_pairs_within_1e4(sur):
    import hlbl_gb300 as hg

    rep = sur.train(n_samples=1 << 20, batch=8192, steps=4000, n_valid=1 << 16, bound=1e-4)
    print("surrogate training report:", rep)
    # what the trained network gains over the coarse quadrature it corrects,
    # inside the accepted region that validation chose
    assert rep["max_rel_err_net"] * 2 <= rep["max_rel_err_base"], rep
    assert rep["rms_rel_err_net"] * 2 <= rep["rms_rel_err_base"], rep
    assert rep["max_rel_err_net"] <= 1e-4, rep
    assert rep["r0"] < 0.1 and rep["r1"] > 0.5, rep
    lat = (16, 8, 8, 8)
    xu = hg.xunit(105.658, 0.1)
    src = torch.from_numpy(S.gaussian_block(lat, 101)).cuda()
    y = torch.from_numpy(S.gaussian_block(lat, 102)).cuda()
    with hg.Contractor(lat) as c:
        exact = c.kernel_sum(src, y, (3, 1, 4, 1), (1, -1, 1, -1), xu, hg.FP64)
        # r0 = 0.05: the three evaluations at x = gsx and K(x, x - y) at x = y
        # fall back to the exact weight, four rows per pair
        c.set_qed(sur, r0=0.05)
        learned = c.kernel_sum(src, y, (3, 1, 4, 1), (1, -1, 1, -1), xu, hg.FP64)
        learned32 = c.kernel_sum(src, y, (3, 1, 4, 1), (1, -1, 1, -1), xu, hg.FP32)
        assert c.qed_fallbacks() >= 8
        c.set_qed(None)
        again = c.kernel_sum(src, y, (3, 1, 4, 1), (1, -1, 1, -1), xu, hg.FP64)
    assert again == exact
    assert S.pair_rel_err(learned, exact) <= 1e-4
    assert S.pair_rel_err(learned32, exact) <= 1e-4
