/* GPU-build shim of KQED's header (oracle/ref_gpu): the reference's device
 * calls of QED_Mkernel_L2 (kernels/cuda_lattice.cu:266-275,
 * kernels/hlbl_kernels/kernels.cu) go to the project's test weights, defined
 * on the device in oracle/ref_gpu/qed_device.cu: the stand-in, or the dense
 * test weight when `dense` points at its table. Test infrastructure only. */
#ifndef HLBL_REF_GPU_KQED_H
#define HLBL_REF_GPU_KQED_H
#include <cuda_runtime.h>
#include "hlbl_gb300_qed.h"
#define KQED_ALIGN __attribute__((aligned(32)))
#ifdef __cplusplus
extern "C" {
#endif
struct QED_kernel_temps {
  hlbl_qed_params p;
  const double* dense; /* device table of the dense test weight, or NULL */
};
typedef struct QED_kernel_temps QED_kernel_temps;
int initialise(struct QED_kernel_temps* t);
int free_QED_temps(struct QED_kernel_temps* t);
__device__ void QED_Mkernel_L2(const double Lambda, const double xv[4], const double yv[4],
                               const struct QED_kernel_temps t, double kerv[6][4][4][4]);
#ifdef __cplusplus
}
#endif
#endif
