// Status strings, the per-thread record of the last CUDA error, and the
// check words of the bounds-checked debug build.
#include <vector>

#include "common.cuh"

namespace fdtd {
static thread_local int g_last_cuda_error = 0;
void set_cuda_error(cudaError_t e) { g_last_cuda_error = (int)e; }
#ifdef FDTD_CHECK
static std::vector<int (*)(unsigned long long *)> &check_readers() {
    static std::vector<int (*)(unsigned long long *)> v;
    return v;
}
int check_register(int (*read)(unsigned long long *)) {
    check_readers().push_back(read);
    return 0;
}
#endif
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

int fdtd_debug_check(uint64_t *first_bad) {
    if (!first_bad) return FDTD_ERR_ARG;
    *first_bad = 0;
#ifdef FDTD_CHECK
    for (auto read : fdtd::check_readers()) {
        unsigned long long v = 0;
        FDTD_TRY(read(&v));
        if (v && !*first_bad) *first_bad = v;
    }
    return FDTD_OK;
#else
    return FDTD_ERR_UNSUPPORTED;
#endif
}

}  // extern "C"
