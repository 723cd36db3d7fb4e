"""Test helpers: the CPU oracle (oracle/hlbl_oracle.c) through ctypes, and the
golden fixtures of tests/golden. Test infrastructure only."""
from __future__ import annotations

import contextlib
import ctypes as C
import json
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_host_emulation.json")
I4 = C.c_int * 4


def i4(v):
    return I4(*[int(a) for a in v])


def vp(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


def volume(v) -> int:
    return int(v[0]) * int(v[1]) * int(v[2]) * int(v[3])


def block_len(v) -> int:
    return 2 * 12 * 24 * volume(v)


_oracle = None


def oracle():
    """The oracle library, built on demand."""
    global _oracle
    if _oracle is None:
        from hlbl_gb300.build import build_oracle

        lib = C.CDLL(build_oracle())
        vpt, dp = C.c_void_p, C.c_double
        lib.oracle_fill_random_block.argtypes = [I4, I4, C.c_uint64, vpt]
        lib.oracle_fill_gaussian_block.argtypes = [I4, I4, C.c_uint64, vpt]
        lib.oracle_source_seed.restype = C.c_uint64
        lib.oracle_source_seed.argtypes = [C.c_uint64, I4]
        lib.oracle_kernel_sum.argtypes = [vpt, vpt, I4, I4, dp, dp, I4, I4, I4, vpt]
        lib.oracle_dzu_dzsu.argtypes = [vpt, vpt, vpt, vpt, C.c_int, I4, I4, I4, I4]
        lib.oracle_insert_gammas.argtypes = [vpt, vpt, vpt, vpt]
        lib.oracle_4pt.restype = dp
        lib.oracle_4pt.argtypes = [vpt, vpt, vpt, vpt, C.c_int, I4, I4, dp, I4, dp, I4, I4]
        lib.oracle_apply_gamma.argtypes = [C.c_int, vpt, vpt]
        lib.oracle_qed_kernel.argtypes = [dp, vpt, vpt, vpt]
        lib.oracle_qed_weights.argtypes = [dp, dp, dp, dp, vpt]
        lib.oracle_coord_map.argtypes = [C.c_int, C.c_int]
        lib.oracle_coord_map_zerohalf.argtypes = [C.c_int, C.c_int]
        lib.oracle_coord_map_diff.argtypes = [C.c_int, C.c_int, C.c_int]
        lib.oracle_set_threads.argtypes = [C.c_int]
        lib.oracle_get_threads.restype = C.c_int
        lib.oracle_set_compensated.argtypes = [C.c_int]
        lib.oracle_get_compensated.restype = C.c_int
        lib.oracle_pi.argtypes = [vpt, C.c_longlong, C.c_int, vpt]
        lib.oracle_p1_2p2.argtypes = [vpt, I4, I4, I4, I4, C.c_int, vpt]
        lib.oracle_p234.argtypes = [vpt, I4, I4, I4, I4, vpt, C.c_int, dp, dp, vpt]
        lib.oracle_pieces_2p2.argtypes = [vpt, C.c_int, I4, vpt, C.c_int, dp, dp, I4, I4, I4, vpt,
                                          vpt]
        lib.oracle_set_qed_dense.argtypes = [C.c_int, C.c_ulonglong]
        lib.oracle_get_qed_dense.restype = C.c_int
        _oracle = lib
    return _oracle


# Seed of the dense test weight (include/hlbl_gb300_qed.h) in every test
# and fixture that uses it.
DENSE_SEED = 20261204


@contextlib.contextmanager
def dense_qed(seed=DENSE_SEED):
    """Within the block the oracle weights with the dense test tensor."""
    lib = oracle()
    lib.oracle_set_qed_dense(1, seed)
    try:
        yield
    finally:
        lib.oracle_set_qed_dense(0, 0)


def random_block(local, seed, pc=(0, 0, 0, 0)) -> np.ndarray:
    """fill_random_block (src/provider.cpp:25-57) via the oracle."""
    out = np.zeros(block_len(local))
    oracle().oracle_fill_random_block(i4(local), i4(pc), C.c_uint64(seed), vp(out))
    return out


def gaussian_block(local, seed, pc=(0, 0, 0, 0)) -> np.ndarray:
    out = np.zeros(block_len(local))
    oracle().oracle_fill_gaussian_block(i4(local), i4(pc), C.c_uint64(seed), vp(out))
    return out


def source_seed(run_seed, gsx) -> int:
    return int(oracle().oracle_source_seed(C.c_uint64(run_seed), i4(gsx)))


def oracle_kernel_sum(src, y, gsx, yv, xunit, lattice, lam=0.4, local=None, pc=(0, 0, 0, 0)):
    local = lattice if local is None else local
    out = np.zeros(2)
    oracle().oracle_kernel_sum(vp(src), vp(y), i4(gsx), i4(yv), C.c_double(xunit),
                               C.c_double(lam), i4(lattice), i4(local), i4(pc), vp(out))
    return out


def oracle_dz(src, y, f, gsx, lattice, local=None, pc=(0, 0, 0, 0)):
    local = lattice if local is None else local
    dzu, dzsu = np.zeros(1728), np.zeros(1152)
    oracle().oracle_dzu_dzsu(vp(dzu), vp(dzsu), vp(src), vp(y), int(f), i4(pc), i4(gsx),
                             i4(lattice), i4(local))
    return dzu, dzsu


def oracle_gammas(dzu, dzsu):
    g_dzu, g_dzsu = np.zeros(6912), np.zeros(4608)
    oracle().oracle_insert_gammas(vp(np.ascontiguousarray(dzu)), vp(np.ascontiguousarray(dzsu)),
                                  vp(g_dzu), vp(g_dzsu))
    return g_dzu, g_dzsu


def oracle_4pt(g_dzu, g_dzsu, src, y, f, gsx, xunit, yv, lattice, local=None, pc=(0, 0, 0, 0),
               lam=0.4):
    local = lattice if local is None else local
    return float(oracle().oracle_4pt(vp(g_dzu), vp(g_dzsu), vp(src), vp(y), int(f), i4(pc),
                                     i4(gsx), C.c_double(xunit), i4(yv), C.c_double(lam),
                                     i4(lattice), i4(local)))


def oracle_pieces_2p2(fwd, gsw, targets, xunit, lattice, local=None, pc=(0, 0, 0, 0),
                      iflavor=0, lam=0.4):
    """The 2+2 pieces of one rank: p1 [4,4,4,Lmax], p234 [n_y,5,64]."""
    local = lattice if local is None else local
    lmax = max(lattice)
    tg = np.ascontiguousarray(np.asarray(targets, dtype=np.int32).reshape(-1, 4))
    p1 = np.zeros(64 * lmax)
    p234 = np.zeros(len(tg) * 5 * 64)
    oracle().oracle_pieces_2p2(vp(fwd), int(iflavor), i4(gsw), vp(tg), len(tg), C.c_double(xunit),
                               C.c_double(lam), i4(lattice), i4(local), i4(pc), vp(p1), vp(p234))
    return p1.reshape(4, 4, 4, lmax), p234.reshape(len(tg), 5, 64)


def golden() -> dict:
    with open(GOLDEN) as fh:
        return json.load(fh)


def case_inputs(case):
    """The two blocks of a golden kernel-sum case, regenerated bit-exactly."""
    lat, spec = case["lattice"], case["input"]
    if spec[0] == "seeds":
        return random_block(lat, spec[1]), random_block(lat, spec[2])
    _, seed, gx, gy = spec
    return random_block(lat, source_seed(seed, gx)), random_block(lat, source_seed(seed, gy))


def pair_rel_err(a, b) -> float:
    """Relative error of a pair's kernel sum as a 2-vector (both flavours):
    max |a_f - b_f| / max |b_f|. The bar of the FP32 path: a flavour whose
    sum nearly cancels is measured against the pair's scale."""
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def rel_err(a, b) -> float:
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


# ---- the reference's own kernels built for the GPU (oracle/ref_gpu) ---------
_ref_gpu = None


def ref_gpu_lib():
    """The GPU build of the reference's Contractor and kernels, or None where
    no staged copy of its sources was built (a machine without the reference
    checkout and without the copy)."""
    global _ref_gpu
    if _ref_gpu is None:
        import platform

        path = os.path.join(ROOT, "oracle", "_ref", "gpu", platform.machine(), "libhlbl_ref_gpu.so")
        if not os.path.exists(path):
            return None
        lib = C.CDLL(path)
        vpt = C.c_void_p
        lib.refgpu_last_error.restype = C.c_char_p
        lib.refgpu_create.argtypes = [C.POINTER(vpt), I4, C.c_int, C.c_ulonglong]
        lib.refgpu_destroy.argtypes = [vpt]
        lib.refgpu_kernel_sum.argtypes = [vpt, vpt, vpt, I4, I4, C.c_double, vpt]
        lib.refgpu_pieces_2p2.argtypes = [vpt, vpt, I4, vpt, C.c_int, C.c_double, vpt, vpt]
        lib.refgpu_reserve_kernel_memory.argtypes = [vpt, C.c_int, C.POINTER(C.c_size_t)]
        _ref_gpu = lib
    return _ref_gpu


class RefGpu:
    """The reference's Contractor on the GPU (one rank, whole lattice), with
    the stand-in weight or (dense) the dense test weight."""

    def __init__(self, lattice, dense=False, seed=DENSE_SEED):
        self.lib = ref_gpu_lib()
        self.h = C.c_void_p()
        self._check(self.lib.refgpu_create(C.byref(self.h), i4(lattice), int(bool(dense)), seed))

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(self.lib.refgpu_last_error().decode())

    def kernel_sum(self, d_src, d_y, gsx, yv, xunit):
        out = (C.c_double * 2)()
        self._check(self.lib.refgpu_kernel_sum(self.h, C.c_void_p(d_src.data_ptr()),
                                               C.c_void_p(d_y.data_ptr()), i4(gsx), i4(yv),
                                               C.c_double(xunit), out))
        return out[0], out[1]

    def pieces_2p2(self, d_fwd, gsw, targets, xunit, lmax):
        tg = np.ascontiguousarray(np.asarray(targets, dtype=np.int32).reshape(-1, 4))
        p1, p234 = np.zeros(64 * lmax), np.zeros(len(tg) * 5 * 64)
        self._check(self.lib.refgpu_pieces_2p2(self.h, C.c_void_p(d_fwd.data_ptr()), i4(gsw), vp(tg),
                                               len(tg), C.c_double(xunit), vp(p1), vp(p234)))
        return p1, p234.reshape(len(tg), 5, 64)

    def close(self):
        if self.h:
            self.lib.refgpu_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
