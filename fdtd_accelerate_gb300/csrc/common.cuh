// Shared helpers for the sm_103a kernels and the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include "fdtd_gb300.h"

namespace fdtd {

// Bounds-checked debug build (-DFDTD_CHECK, libfdtd_gb300_check.so): every
// global access wrapped in FDTD_IN compares its element index with the extent
// of its array.  A miss records (1 << 63 | source line << 40 | index) in the
// translation unit's check word, the first one only, and the access is skipped
// instead of faulting; fdtd_debug_check() reads and clears the words of every
// unit.  In the product build FDTD_IN is the constant true.
#ifdef FDTD_CHECK
static __device__ unsigned long long g_check_word;
__device__ __forceinline__ bool check_index(long long i, long long n, int line) {
    if (i >= 0 && i < n) return true;
    atomicCAS(&g_check_word, 0ull,
              (1ull << 63) | ((unsigned long long)(line & 0x7FFFFF) << 40) | ((unsigned long long)i & 0xFFFFFFFFFFull));
    return false;
}
#define FDTD_IN(i, n) ::fdtd::check_index((long long)(i), (long long)(n), __LINE__)
int check_register(int (*read)(unsigned long long *));  // abi.cu
static int check_read_unit(unsigned long long *w) {
    unsigned long long v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_check_word, sizeof(v));
    if (e == cudaSuccess && v) {
        const unsigned long long z = 0;
        e = cudaMemcpyToSymbol(g_check_word, &z, sizeof(z));
    }
    *w = v;
    return e == cudaSuccess ? FDTD_OK : FDTD_ERR_CUDA;
}
static const int g_check_registered = check_register(check_read_unit);
#else
#define FDTD_IN(i, n) true
#endif

// NVTX range around one step (or stage) of an entry point, for Nsight
// Systems timelines and `ncu --nvtx` filters.  Header-only NVTX v3: without
// an attached tool a push/pop pair is a call through a no-op pointer.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// Thread-local record of the last CUDA error seen by an entry point.
void set_cuda_error(cudaError_t e);

// Check a launch; map CUDA failures to FDTD_ERR_CUDA.
inline int check_launch() {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

#define FDTD_TRY(expr)                  \
    do {                                \
        int _st = (expr);               \
        if (_st != FDTD_OK) return _st; \
    } while (0)

struct Grid {
    int64_t nx, ny, nz, sx, sy;
};

inline int validate_grid(const fdtd_grid *g, Grid *out) {
    if (!g) return FDTD_ERR_ARG;
    if (g->nx < 1 || g->ny < 1 || g->nz < 1) return FDTD_ERR_SHAPE;
    if (g->sy < g->nz || g->sx < g->ny * g->sy) return FDTD_ERR_SHAPE;
    if (g->nx > 65535 || g->ny > 65535) return FDTD_ERR_SHAPE;  // grid.y/z launch limits
    *out = Grid{g->nx, g->ny, g->nz, g->sx, g->sy};
    return FDTD_OK;
}

template <typename... P>
inline bool all_nonnull(P... p) {
    return ((p != nullptr) && ...);
}

// TFSF helpers (tfsf.cu): validation, 1-D grid length, the fused-step table
// and the 1-D steps (which: 0 = E step of step t, 1 = H step, 2 = H step then
// the E step of step t).
int validate_tfsf(const Grid &g, const fdtd_tfsf *t);
int64_t tfsf_n1d(const fdtd_tfsf *t);
void tfsf_table(const fdtd_tfsf *t, float coef[2][6][2], int32_t ix[2][6][2], int32_t *vo);
int tfsf_launch_1d(const fdtd_tfsf *t, int which, int64_t step, cudaStream_t st);

// Drude box inside the grid, all nine arrays present.
inline int validate_drude(const Grid &g, const fdtd_drude *d) {
    if (!d) return FDTD_ERR_ARG;
    if (d->ni < 1 || d->nj < 1 || d->nk < 1 || d->i0 < 0 || d->j0 < 0 || d->k0 < 0) return FDTD_ERR_SHAPE;
    if (d->i0 + d->ni > g.nx || d->j0 + d->nj > g.ny || d->k0 + d->nk > g.nz) return FDTD_ERR_SHAPE;
    for (int q = 0; q < 3; q++)
        if (!all_nonnull(d->j[q], d->cja[q], d->cjb[q])) return FDTD_ERR_ARG;
    return FDTD_OK;
}

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Round-to-nearest arithmetic that the compiler may not contract into FMA:
// the kernels reproduce the rounding of the reference's NumPy expressions.
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }

// Drude ADE on one E value: e' = e - ce*J, J = cja*J + cjb*e'
// (kuFDTD/v0.2.0/dim3/cpu/core/drude_ade.c:71-78); returns e', sets jn.
__device__ __forceinline__ float drude_cell(float e, float ce, float j, float cja, float cjb, float &jn) {
    const float en = fsub(e, fmul(ce, j));
    jn = fadd(fmul(cja, j), fmul(cjb, en));
    return en;
}

// ((a - b) - c) + d : the grouping NumPy uses for `a - b - c + d`.
__device__ __forceinline__ float curl4(float a, float b, float c, float d) {
    return fadd(fsub(fsub(a, b), c), d);
}

// CPML slab index -> node index (front slab s < P at s+1, back slab at
// n-P-1+(s-P) for E nodes, n-P+(s-P) for H nodes).
__device__ __forceinline__ int64_t slab_node_e(int64_t s, int64_t P, int64_t n) {
    return s < P ? s + 1 : n - P - 1 + (s - P);
}
__device__ __forceinline__ int64_t slab_node_h(int64_t s, int64_t P, int64_t n) {
    return s < P ? s + 1 : n - P + (s - P);
}

}  // namespace fdtd
