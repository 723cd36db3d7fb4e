// hlbl_gb300_dropin.h -- shared by the drop-in launchers (cuda_lattice_gb300.cpp,
// kernels_2p2_gb300.cpp): the library context of a lattice and rank position
// on the current device, made on first use and kept for the process.
#pragma once

#include "hlbl_gb300.h"

hlbl_ctx* hlbl_dropin_context(const int global[4], const int local[4], const int pc[4]);
