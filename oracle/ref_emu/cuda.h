/* Stand-in for <cuda.h> when the reference kernels are compiled for the CPU
 * by oracle/build_ref.sh: the kernels need nothing from it. */
#pragma once
#include "mdt_cuda_emu.h"
