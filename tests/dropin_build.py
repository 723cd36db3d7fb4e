"""Build helper of the drop-in tests (test infrastructure): makes
tests/dropin/run_chains_main.cpp against the library (variant "gb300") or the
reference's own kernels (variant "ref") with tests/dropin/Makefile, from the
staged copy of the reference's sources or a reference checkout."""
from __future__ import annotations

import os
import platform
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STAGED = os.path.join(ROOT, "oracle", "_ref", "gpu", "src")
OUT = os.path.join(ROOT, "oracle", "_ref", "dropin", platform.machine())


def sources() -> str | None:
    """The reference sources to compile: the staged copy, else a checkout."""
    if os.path.exists(os.path.join(STAGED, "src", "driver.cpp")):
        return STAGED
    from hlbl_gb300.build import REF_DIR

    if os.path.exists(os.path.join(REF_DIR, "src", "driver.cpp")):
        return REF_DIR
    return None


def build(variant: str) -> str:
    """Path of the built program; raises with make's output on failure."""
    src = sources()
    if src is None:
        raise FileNotFoundError("no reference sources (staged copy or checkout)")
    from hlbl_gb300.build import build_library

    build_library()
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "tests", "dropin"), variant, "S=" + src],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("make %s failed:\n%s%s" % (variant, r.stdout[-3000:], r.stderr[-3000:]))
    return os.path.join(OUT, "run_chains_" + variant)
