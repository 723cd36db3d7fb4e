"""The C ABI without a GPU: libhlbl_gb300.so loads, exports every function
include/hlbl_gb300.h declares (and no other hlbl_ symbol), the ctypes binding
gives each one the header's number of arguments, and a call that needs the
GPU fails with a status and a message instead of falling back to anything."""
import ctypes as C
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "hlbl_gb300.h")


def declared():
    """name -> number of parameters, for the header's function declarations."""
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    src = re.sub(r"^\s*#[^\n]*", "", src, flags=re.M)
    out = {}
    for stmt in re.split(r"[;{}]", src):
        m = re.fullmatch(r"\s*((?:const\s+)?\w+[\s\*]+)(hlbl_\w+)\s*\((.*)\)\s*", stmt, flags=re.S)
        if not m:
            continue
        ret, name, params = m.groups()
        if "static" in ret or "typedef" in ret:
            continue
        params = " ".join(params.split())
        out[name] = 0 if params in ("", "void") else params.count(",") + 1
    return out


@pytest.fixture(scope="module")
def lib():
    from hlbl_gb300 import build

    build.build_library()
    from hlbl_gb300 import _lib

    return _lib.lib


def test_header_parses_to_the_whole_api():
    d = declared()
    assert len(d) >= 50
    for name in ("hlbl_ctx_create", "hlbl_kernel_sum", "hlbl_kernel_sums_batched_f32", "hlbl_cu_dzu_dzsu",
                 "hlbl_cu_4pt_contraction", "hlbl_compute_2p2", "hlbl_pieces_2p2", "hlbl_stage_async"):
        assert name in d, name
    assert d["hlbl_version"] == 0 and d["hlbl_ctx_create"] == 6


def test_every_declared_function_is_exported_and_bound(lib):
    for name, n in declared().items():
        f = getattr(lib, name)  # AttributeError if not exported
        assert f.argtypes is not None, f"{name} has no ctypes signature"
        assert len(f.argtypes) == n, (name, len(f.argtypes), n)


@pytest.mark.skipif(shutil.which("nm") is None, reason="nm not available")
def test_no_undeclared_exports(lib):
    from hlbl_gb300.build import LIB

    out = subprocess.run(["nm", "-D", "--defined-only", LIB], capture_output=True, text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if re.search(r"\sT\s+hlbl_", ln)}
    assert exported == set(declared()), exported ^ set(declared())


def test_version_needs_no_device(lib):
    assert b"sm_103a" in lib.hlbl_version()


def test_device_calls_fail_loudly_without_a_gpu(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    i4 = C.c_int * 4
    st = lib.hlbl_ctx_create(C.byref(h), i4(4, 4, 4, 4), i4(4, 4, 4, 4), i4(0, 0, 0, 0), 0.4, 0)
    assert st != 0 and not h.value
    assert lib.hlbl_last_error().startswith(b"cuda")
    from hlbl_gb300._lib import HlblError, check

    with pytest.raises(HlblError):
        check(lib.hlbl_ctx_create(C.byref(h), i4(4, 4, 4, 4), i4(4, 4, 4, 4), i4(0, 0, 0, 0), 0.4, 0))


C_PROGRAM = r"""
#include "hlbl_gb300.h"
#include <stdio.h>
#include <string.h>
int main(void) {
  const char* v = hlbl_version();
  hlbl_ctx* ctx = 0;
  int g[4] = {4, 4, 4, 4}, pc[4] = {0, 0, 0, 0};
  int rc = hlbl_ctx_create(&ctx, g, g, pc, 0.4, 0);
  int ok = strstr(v, "sm_103a") != 0 && (rc == 0) == (ctx != 0);
  if (rc != 0) ok = ok && strlen(hlbl_last_error()) > 0;
  if (ctx) hlbl_ctx_destroy(ctx);
  printf("%s %d\n", v, rc);
  return ok ? 0 : 1;
}
"""


@pytest.mark.parametrize("lang", ["c", "c++"])
def test_header_compiles_links_and_runs_from_c_and_cxx(lang, lib, tmp_path):
    """include/hlbl_gb300.h is a plain C header (usable from the reference's
    C++ and from C shims): a program compiled with -Wall -Wextra links against
    the library and runs (without a GPU, context creation fails with a status
    and a message)."""
    from hlbl_gb300.build import LIB

    cc = shutil.which("gcc" if lang == "c" else "g++")
    if cc is None:
        pytest.skip(f"no {lang} compiler")
    src = tmp_path / ("t.c" if lang == "c" else "t.cpp")
    src.write_text(C_PROGRAM)
    exe = tmp_path / "t"
    libdir = os.path.dirname(LIB)
    std = "-std=c11" if lang == "c" else "-std=c++17"
    r = subprocess.run([cc, std, "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                        "-L", libdir, "-lhlbl_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
