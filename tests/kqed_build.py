"""Test infrastructure: a stand-in KQED install and the library linked with it.

KQED (libKQED_cuda.a + KQED.h) is not available here. To exercise the
library's KQED link path (HLBL_KQED_DIR, HLBL_QEDK_KQED), this builds a
directory with KQED's layout -- include/KQED.h (oracle/ref_gpu/shim/KQED.h)
and lib/libKQED_cuda.a holding a device QED_Mkernel_L2 and a host
initialise() (oracle/ref_gpu/qed_device.cu, the project's stand-in weight) --
and the library linked with it, both under oracle/_build."""
from __future__ import annotations

import os
import shutil
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KQED_DIR = os.path.join(ROOT, "oracle", "_build", "kqed_standin")
KQED_LIB_OUT = os.path.join(ROOT, "oracle", "_build", "kqed_linked", "libhlbl_gb300.so")


def build_standin_kqed() -> str:
    from hlbl_gb300.build import ARCH, _nvcc

    inc, lib = os.path.join(KQED_DIR, "include"), os.path.join(KQED_DIR, "lib")
    os.makedirs(inc, exist_ok=True)
    os.makedirs(lib, exist_ok=True)
    shutil.copyfile(os.path.join(ROOT, "oracle", "ref_gpu", "shim", "KQED.h"), os.path.join(inc, "KQED.h"))
    obj = os.path.join(lib, "qed_device.o")
    subprocess.run([_nvcc()] + ARCH + ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-rdc=true", "-I", inc,
                                       "-I", os.path.join(ROOT, "include"), "-c",
                                       os.path.join(ROOT, "oracle", "ref_gpu", "qed_device.cu"), "-o", obj],
                   check=True, capture_output=True)
    a = os.path.join(lib, "libKQED_cuda.a")
    if os.path.exists(a):
        os.remove(a)
    subprocess.run(["ar", "rcs", a, obj], check=True)
    return KQED_DIR


def build_linked_library() -> str:
    from hlbl_gb300.build import build_library

    return build_library(kqed_dir=build_standin_kqed(), out=KQED_LIB_OUT)
