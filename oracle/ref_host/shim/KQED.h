/* Host-emulation shim of KQED's header (oracle/ref_host): the reference's
 * QED_Mkernel_L2 call is served by the project's stand-in weight
 * (include/hlbl_gb300_qed.h). Test infrastructure only. */
#ifndef HLBL_REF_HOST_KQED_H
#define HLBL_REF_HOST_KQED_H
#include "hlbl_gb300_qed.h"
#define KQED_ALIGN __attribute__((aligned(32)))
#ifdef __cplusplus
extern "C" {
#endif
struct QED_kernel_temps { hlbl_qed_params p; };
typedef struct QED_kernel_temps QED_kernel_temps;
int initialise(struct QED_kernel_temps* t);
int free_QED_temps(struct QED_kernel_temps* t);
void QED_Mkernel_L2(const double Lambda, const double xv[4], const double yv[4],
                    const struct QED_kernel_temps t, double kerv[6][4][4][4]);
#ifdef __cplusplus
}
#endif
#endif
