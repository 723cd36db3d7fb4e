"""The C++ drop-in (hlbl_gb300/dropin): the reference's own src/driver.cpp,
src/contract.cpp, src/schedule.cpp, src/propagator_cache.cpp and
src/provider.cpp compile unchanged against the reference's headers and link
with the drop-in launchers (cu_dzu_dzsu, cu_4pt_contraction, compute_2p2_gpu)
and libhlbl_gb300.so, with no symbol of the reference's kernels left
undefined. CPU only (linking needs no GPU); skipped where neither a staged
copy of the reference's sources nor a checkout is present."""
import subprocess

import pytest

import dropin_build as D

pytestmark = pytest.mark.skipif(D.sources() is None, reason="no reference sources to compile")


def test_reference_driver_links_against_the_library():
    exe = D.build("gb300")
    und = subprocess.run(["nm", "-D", "--undefined-only", exe], capture_output=True, text=True).stdout
    for sym in ("hlbl_ctx_create", "hlbl_cu_dzu_dzsu", "hlbl_cu_4pt_contraction", "hlbl_compute_2p2"):
        assert sym in und, sym
    syms = subprocess.run(["nm", "-C", exe], capture_output=True, text=True).stdout
    # the launchers the reference's contract.cpp calls are defined by the drop-in
    for name in ("cu_dzu_dzsu(", "cu_4pt_contraction(", "compute_2p2_gpu(", "hlbl::run_chains(",
                 "hlbl::Contractor::kernel_sum("):
        lines = [ln for ln in syms.splitlines() if name in ln]
        assert lines and all(" U " not in ln for ln in lines), name
