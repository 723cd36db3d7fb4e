"""The learned QED weight (an MLP correcting a coarse quadrature of the six
weight functions), trained on the GPU by the library's own kernels.

    s = Surrogate(); report = s.train(); contractor.set_qed(s)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import TrainConfig, TrainReport, check, lib

NPARAM = 34310
RADIUS = 6.43  # 12 fm in units of 1/m_mu: the training range of |x|, |y|
QED_EXACT, QED_SURROGATE = 0, 1


class Surrogate:
    """hlbl_surrogate (include/hlbl_gb300.h)."""

    def __init__(self, device: int = 0, lam: float = 0.4, seed: int = 1):
        h = C.c_void_p()
        check(lib.hlbl_surrogate_create(C.byref(h), int(device), C.c_double(lam), C.c_uint64(seed)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib.hlbl_surrogate_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def handle(self):
        return self._h

    def train(self, n_samples=4 * 1024 * 1024, batch=8192, steps=4000, lr=1e-3, seed=7,
              radius=RADIUS, n_valid=262144, bound=1e-5) -> dict:
        """Generate labelled samples, train (Adam), validate; returns the report."""
        cfg = TrainConfig(n_samples, batch, steps, lr, seed, radius, n_valid, bound)
        rep = TrainReport()
        check(lib.hlbl_surrogate_train(self._h, C.byref(cfg), C.byref(rep)))
        return {k: getattr(rep, k) for k, _ in TrainReport._fields_}

    def params(self):
        p = np.zeros(NPARAM, dtype=np.float32)
        sg = np.zeros(6, dtype=np.float32)
        check(lib.hlbl_surrogate_params(self._h, p.ctypes.data, sg.ctypes.data, 0))
        return p, sg

    def set_params(self, p, sigma) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        sg = np.ascontiguousarray(sigma, dtype=np.float32)
        assert p.size == NPARAM and sg.size == 6
        check(lib.hlbl_surrogate_params(self._h, p.ctypes.data, sg.ctypes.data, 1))

    def gradients(self, feat, target):
        """(loss, grad) of one training step on host rows (no update)."""
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        target = np.ascontiguousarray(target, dtype=np.float32)
        n = feat.shape[0]
        g = np.zeros(NPARAM, dtype=np.float32)
        loss = C.c_float()
        check(lib.hlbl_surrogate_gradients(self._h, feat.ctypes.data, target.ctypes.data, n,
                                           g.ctypes.data, C.byref(loss)))
        return float(loss.value), g

    def eval(self, feat):
        """Raw network outputs of the inference kernel for host rows."""
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        out = np.zeros((feat.shape[0], 6), dtype=np.float32)
        check(lib.hlbl_surrogate_eval(self._h, feat.ctypes.data, feat.shape[0], out.ctypes.data))
        return out
