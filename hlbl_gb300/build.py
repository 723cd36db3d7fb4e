"""Build the native parts: the CUDA library for sm_103a and the C oracle.

    python -m hlbl_gb300.build          # library + oracle
    python -m hlbl_gb300.build --lib    # library only

The library is built in-tree under hlbl_gb300/_build/ (one nvcc process per
translation unit, in parallel, then one link). The oracle (test
infrastructure) goes to oracle/_build/. Where the reference sources are
mounted, the host-emulation build of them (oracle/ref_host) is made too.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libhlbl_gb300.so")
ORACLE_SRC = os.path.join(ROOT, "oracle", "hlbl_oracle.c")
ORACLE_LIB = os.path.join(ROOT, "oracle", "_build", "libhlbl_oracle.so")
REF_DIR = os.environ.get("HLBL_REFERENCE_DIR", "/root/reference")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build_library(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
                     + glob.glob(os.path.join(ROOT, "include", "*.h")))
    if not force and _newer(LIB, sources + headers):
        return LIB
    nvcc = _nvcc()
    objs = []
    jobs = []
    for s in sources:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        jobs.append([nvcc] + ARCH + NVCC_FLAGS + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    tmp = LIB + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs)
    os.replace(tmp, LIB)
    return LIB


def build_oracle(force: bool = False) -> str:
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    deps = [ORACLE_SRC] + glob.glob(os.path.join(ROOT, "include", "*.h"))
    if not force and _newer(ORACLE_LIB, deps):
        return ORACLE_LIB
    cc = shutil.which("gcc") or "cc"
    tmp = ORACLE_LIB + ".tmp"
    _run([cc, "-std=c11", "-O2", "-fopenmp", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"),
          ORACLE_SRC, "-o", tmp, "-lm"])
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_reference_emulation() -> str | None:
    """The reference's own sources as a host emulation (only where mounted)."""
    if not os.path.isdir(os.path.join(REF_DIR, "kernels")):
        return None
    _run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref_host"), "REF=" + REF_DIR])
    return os.path.join(ROOT, "oracle", "_ref", "libhlbl_ref_host.so")


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    force = "--force" in argv
    print(build_library(force))
    if "--lib" not in argv:
        print(build_oracle(force))
        r = build_reference_emulation()
        if r:
            print(r)
    return 0


if __name__ == "__main__":
    sys.exit(main())
