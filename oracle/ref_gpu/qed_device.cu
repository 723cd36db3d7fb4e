// qed_device.cu -- TEST INFRASTRUCTURE. KQED's entry points for the GPU build
// of the reference's own kernels (oracle/ref_gpu): QED_Mkernel_L2 on the
// device, served by the project's test weights (include/hlbl_gb300_qed.h),
// and the host initialise()/free_QED_temps() the reference's callers use
// (bin/hlbl_hypercube.cpp:174-178). Never shipped.
#include "KQED.h"

extern "C" __device__ void QED_Mkernel_L2(const double Lambda, const double xv[4], const double yv[4],
                                          const struct QED_kernel_temps t, double kerv[6][4][4][4]) {
  if (t.dense) {
    hlbl_qed_dense_kernel(t.dense, xv, yv, kerv);
    return;
  }
  hlbl_qed_params p = t.p;
  p.lambda = Lambda;
  hlbl_qed_kernel(&p, xv, yv, kerv);
}

extern "C" int initialise(struct QED_kernel_temps* t) {
  hlbl_qed_params_init(&t->p, 0.4);
  t->dense = nullptr;
  return 0;
}

extern "C" int free_QED_temps(struct QED_kernel_temps*) { return 0; }
