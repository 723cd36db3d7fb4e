/* The single-rank MPI shim of the host-emulation build, for the GPU build of
 * the reference (oracle/ref_gpu). Test infrastructure only. */
#pragma once
#include "../../ref_host/shim/mpi.h"
