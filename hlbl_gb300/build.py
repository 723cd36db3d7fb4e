"""Build the native parts: the CUDA library for sm_103a and the C oracle.

    python -m hlbl_gb300.build          # library + oracle
    python -m hlbl_gb300.build --lib    # library only

The library is built in-tree under hlbl_gb300/_build/ (one nvcc process per
translation unit, in parallel, then one link); a stamp beside it records the
host architecture and compiler it was built for, and a library built for
another is rebuilt. The oracle (test infrastructure) goes to oracle/_build/.
Where the reference sources are found (HLBL_REFERENCE_DIR, else a `reference`
directory beside the repository), the host-emulation build of them
(oracle/ref_host) is made and the files of their GPU build are staged
(oracle/ref_gpu); wherever a staged copy exists, the GPU build of the
reference's kernels (oracle/_ref/gpu) is made too, alongside the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import platform
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
REF_DIR = os.environ.get("HLBL_REFERENCE_DIR", os.path.join(os.path.dirname(ROOT), "reference"))
REF_GPU_SRC = os.path.join(ROOT, "oracle", "_ref", "gpu", "src")
REF_GPU_LIB = os.path.join(ROOT, "oracle", "_ref", "gpu", platform.machine(), "libhlbl_ref_gpu.so")

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


def _stamp(flags) -> str:
    """What the library was built for: host architecture, compiler, flags."""
    r = subprocess.run([_nvcc(), "--version"], capture_output=True, text=True)
    ver = r.stdout.strip().splitlines()[-1] if r.stdout.strip() else "?"
    return "\n".join([platform.machine(), ver, " ".join(ARCH + flags)]) + "\n"


def _kqed_flags(kqed_dir):
    """A linked KQED: its header directory and static library (include/KQED.h,
    lib/libKQED_cuda.a under kqed_dir); its device code needs relocatable
    device code and a device link."""
    inc, lib = os.path.join(kqed_dir, "include"), os.path.join(kqed_dir, "lib", "libKQED_cuda.a")
    for p in (os.path.join(inc, "KQED.h"), lib):
        if not os.path.exists(p):
            raise RuntimeError(f"HLBL_KQED_DIR: {p} is missing")
    return ["-DHLBL_WITH_KQED", "-rdc=true", "-I", inc], [lib], [inc, lib]


def build_library(force: bool = False, kqed_dir: str | None = None, out: str | None = None) -> str:
    """The library; with kqed_dir (default: the HLBL_KQED_DIR environment
    variable) linked with that KQED, so that HLBL_QEDK_KQED weights with its
    QED_Mkernel_L2. `out`: the library's path (default hlbl_gb300/_build)."""
    kqed_dir = kqed_dir if kqed_dir is not None else os.environ.get("HLBL_KQED_DIR") or None
    lib_path = out or LIB
    build_dir = os.path.dirname(lib_path)
    os.makedirs(build_dir, exist_ok=True)
    extra, link_extra, deps_extra = _kqed_flags(kqed_dir) if kqed_dir else ([], [], [])
    flags = NVCC_FLAGS + extra
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
                     + glob.glob(os.path.join(ROOT, "include", "*.h")))
    deps = sources + headers + [d for d in deps_extra if os.path.isfile(d)]
    stamp_path = lib_path + ".stamp"
    stamp = _stamp(flags + link_extra)
    try:
        with open(stamp_path) as fh:
            same = fh.read() == stamp
    except OSError:
        same = False
    if not force and same and _newer(lib_path, deps):
        return lib_path
    nvcc = _nvcc()
    objs = []
    jobs = []
    for s in sources:
        o = os.path.join(build_dir, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        jobs.append([nvcc] + ARCH + flags + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    tmp = lib_path + ".tmp"
    _run([nvcc] + ARCH + (["-rdc=true"] if kqed_dir else []) + ["-shared", "-o", tmp] + objs + link_extra)
    os.replace(tmp, lib_path)
    with open(stamp_path, "w") as fh:
        fh.write(stamp)
    return lib_path


def build_oracle(force: bool = False) -> str:
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    deps = [ORACLE_SRC] + glob.glob(os.path.join(ROOT, "include", "*.h"))
    if not force and _newer(ORACLE_LIB, deps):
        return ORACLE_LIB
    cc = shutil.which("gcc") or "cc"
    tmp = ORACLE_LIB + ".tmp"
    _run([cc, "-std=c11", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"),
          ORACLE_SRC, "-o", tmp, "-lm"])
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_reference_emulation() -> str | None:
    """The reference's own sources as a host emulation, and the staged copy of
    the files of their GPU build (only where the sources are found)."""
    if not os.path.isdir(os.path.join(REF_DIR, "kernels")):
        return None
    _run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref_host"), "REF=" + REF_DIR])
    _run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref_gpu"), "stage", "REF=" + REF_DIR])
    return os.path.join(ROOT, "oracle", "_ref", "libhlbl_ref_host.so")


def build_reference_gpu() -> str | None:
    """The reference's own kernels built for sm_103a from the staged copy
    (the GPU baseline; None where no copy is staged or the build fails)."""
    if not os.path.isdir(REF_GPU_SRC):
        return None
    r = subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle", "ref_gpu")],
                       capture_output=True, text=True)
    if r.returncode != 0:
        print("reference GPU build failed:\n" + r.stdout[-2000:] + r.stderr[-2000:], file=sys.stderr)
        return None
    return REF_GPU_LIB


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    force = "--force" in argv
    print(build_library(force))
    if "--lib" not in argv:
        print(build_oracle(force))
        r = build_reference_emulation()
        if r:
            print(r)
        r = build_reference_gpu()
        if r:
            print(r)
    return 0


if __name__ == "__main__":
    sys.exit(main())
