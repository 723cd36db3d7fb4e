"""The library's KQED link path on CPU: built with a KQED install
(HLBL_KQED_DIR; here the stand-in install of tests/kqed_build.py) the library
compiles with relocatable device code, links KQED's device QED_Mkernel_L2 and
host initialise() from libKQED_cuda.a, and exports the same C ABI."""
import subprocess

import kqed_build as K


def test_library_links_with_a_kqed_install():
    lib = K.build_linked_library()
    defined = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    for sym in ("hlbl_ctx_set_qed_kernel", "hlbl_kernel_sum", "hlbl_kernel_sums_batched_f32",
                "hlbl_pieces_2p2", "initialise"):
        assert f" {sym}\n" in defined or defined.rstrip().endswith(f" {sym}"), sym
