// Error reporting and device queries shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include "qutip_gb300.h"

namespace qg {
// Record a message for qg_last_error() on this thread and return code.
int set_error(int code, const char* msg);
// Check cudaGetLastError() after a launch; QG_OK or QG_ERR_CUDA.
int check_launch(const char* what);
// Multiprocessor count of the current device (cached per device).
int sm_count();
}  // namespace qg

// The dense kernel's fault flag, read and cleared (for qg_device_fault).
int dense_fault_take();
