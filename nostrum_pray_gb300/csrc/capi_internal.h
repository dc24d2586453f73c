// Error helpers shared by the C-ABI translation units.
#pragma once

#include <string>

#include <cuda_runtime.h>

#include "../../include/nostrum_pray.h"

namespace pray_gpu {

// Records msg as the calling thread's last error and returns st.
pray_status set_error(pray_status st, const std::string &msg);
// Maps a CUDA error to a status (allocation failures to PRAY_ERR_OUT_OF_MEMORY).
pray_status cuda_error(cudaError_t e, const char *what);

}  // namespace pray_gpu
