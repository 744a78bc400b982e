// Status strings and the per-thread record of the last CUDA error.
#include "common.cuh"

namespace fdtd {
static thread_local int g_last_cuda_error = 0;
void set_cuda_error(cudaError_t e) { g_last_cuda_error = (int)e; }
}  // namespace fdtd

extern "C" {

const char *fdtd_status_string(int status) {
    switch (status) {
        case FDTD_OK: return "ok";
        case FDTD_ERR_ARG: return "invalid argument (null pointer or bad value)";
        case FDTD_ERR_SHAPE: return "invalid extents or strides";
        case FDTD_ERR_ALIGN: return "pointer or stride alignment requirement violated";
        case FDTD_ERR_CUDA: return "CUDA error";
        case FDTD_ERR_TIMEOUT: return "bounded device wait expired";
        case FDTD_ERR_UNSUPPORTED: return "configuration not supported";
        case FDTD_ERR_CAPACITY: return "request exceeds a fixed capacity";
        default: return "unknown status";
    }
}

int fdtd_last_cuda_error(void) { return fdtd::g_last_cuda_error; }

}  // extern "C"
