"""The network oracle (oracle/mlp_oracle.py) against finite differences, in
FP64 without BF16 rounding. CPU only."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import mlp_oracle as M  # noqa: E402


def test_parameter_count_matches_library_header():
    hdr = open(os.path.join(os.path.dirname(M.__file__), "..", "include", "hlbl_gb300.h")).read()
    assert f"#define HLBL_SURROGATE_NPARAM {M.NPARAM}" in hdr


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = rng.normal(0, 0.2, M.NPARAM)
    x = rng.uniform(-1, 1, (16, 3))
    t = rng.normal(0, 1, (16, 6))
    _, g = M.loss_and_grad(p, x, t, round_bf16=False)
    idx = rng.choice(M.NPARAM, 60, replace=False)
    for i in idx:
        e = np.zeros(M.NPARAM)
        e[i] = 1e-6
        lp, _ = M.loss_and_grad(p + e, x, t, round_bf16=False)
        lm, _ = M.loss_and_grad(p - e, x, t, round_bf16=False)
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9], dtype=np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == 1.0
