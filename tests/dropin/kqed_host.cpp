// kqed_host.cpp -- TEST INFRASTRUCTURE. KQED's host entry points for the
// drop-in build of run_chains_main (the library weights with its own QED
// kernel and does not read the temps). Never shipped.
#include "KQED.h"

extern "C" int initialise(struct QED_kernel_temps* t) {
  hlbl_qed_params_init(&t->p, 0.4);
  t->dense = nullptr;
  return 0;
}
extern "C" int free_QED_temps(struct QED_kernel_temps*) { return 0; }
