// 4th-order spatial / symplectic-stage kernels (in place).
//
// One call is one stage of 4th_order-Symplectic/PyCUDA/100-base.py:124-141:
//   H -= cl * ch * (27 * (near difference) - (far difference))
//   E += dl * ce * (27 * (near difference) - (far difference))
// with the index ranges of the CUDA kernels at 100-base.py:17-43 and the
// operation grouping of 4th_order-Symplectic/Python-C/dielectric.c:35-89.
// Arrays are C order (nx, ny, nz); the stencil is written per axis, so the
// results equal the reference's Fortran-order arrays indexed [i, j, k].
#include "common.cuh"

namespace fdtd {

constexpr int kSympBlock = 128;

__global__ void __launch_bounds__(kSympBlock)
k_symp_h(Grid g, float cl, const float *__restrict__ ex, const float *__restrict__ ey,
         const float *__restrict__ ez, float *__restrict__ hx, float *__restrict__ hy, float *__restrict__ hz,
         const float *__restrict__ chx, const float *__restrict__ chy, const float *__restrict__ chz) {
    const int64_t k = (int64_t)blockIdx.x * kSympBlock + threadIdx.x;
    const int64_t j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    const int64_t c = i * g.sx + j * g.sy + k, X = g.sx, Y = g.sy;
    const bool jin = j > 1 && j < g.ny - 1, kin = k > 1 && k < g.nz - 1, iin = i > 1 && i < g.nx - 1;
    if (jin && kin) {
        float n = curl4(ez[c], ez[c - Y], ey[c], ey[c - 1]);
        float f = curl4(ez[c + Y], ez[c - 2 * Y], ey[c + 1], ey[c - 2]);
        hx[c] = fsub(hx[c], fmul(fmul(cl, chx[c]), fsub(fmul(27.0f, n), f)));
    }
    if (iin && kin) {
        float n = curl4(ex[c], ex[c - 1], ez[c], ez[c - X]);
        float f = curl4(ex[c + 1], ex[c - 2], ez[c + X], ez[c - 2 * X]);
        hy[c] = fsub(hy[c], fmul(fmul(cl, chy[c]), fsub(fmul(27.0f, n), f)));
    }
    if (iin && jin) {
        float n = curl4(ey[c], ey[c - X], ex[c], ex[c - Y]);
        float f = curl4(ey[c + X], ey[c - 2 * X], ex[c + Y], ex[c - 2 * Y]);
        hz[c] = fsub(hz[c], fmul(fmul(cl, chz[c]), fsub(fmul(27.0f, n), f)));
    }
}

__global__ void __launch_bounds__(kSympBlock)
k_symp_e(Grid g, float dl, float *__restrict__ ex, float *__restrict__ ey, float *__restrict__ ez,
         const float *__restrict__ hx, const float *__restrict__ hy, const float *__restrict__ hz,
         const float *__restrict__ cex, const float *__restrict__ cey, const float *__restrict__ cez) {
    const int64_t k = (int64_t)blockIdx.x * kSympBlock + threadIdx.x;
    const int64_t j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    const int64_t c = i * g.sx + j * g.sy + k, X = g.sx, Y = g.sy;
    const bool jin = j > 0 && j < g.ny - 2, kin = k > 0 && k < g.nz - 2, iin = i > 0 && i < g.nx - 2;
    if (jin && kin) {
        float n = curl4(hz[c + Y], hz[c], hy[c + 1], hy[c]);
        float f = curl4(hz[c + 2 * Y], hz[c - Y], hy[c + 2], hy[c - 1]);
        ex[c] = fadd(ex[c], fmul(fmul(dl, cex[c]), fsub(fmul(27.0f, n), f)));
    }
    if (iin && kin) {
        float n = curl4(hx[c + 1], hx[c], hz[c + X], hz[c]);
        float f = curl4(hx[c + 2], hx[c - 1], hz[c + 2 * X], hz[c - X]);
        ey[c] = fadd(ey[c], fmul(fmul(dl, cey[c]), fsub(fmul(27.0f, n), f)));
    }
    if (iin && jin) {
        float n = curl4(hy[c + X], hy[c], hx[c + Y], hx[c]);
        float f = curl4(hy[c + 2 * X], hy[c - X], hx[c + 2 * Y], hx[c - Y]);
        ez[c] = fadd(ez[c], fmul(fmul(dl, cez[c]), fsub(fmul(27.0f, n), f)));
    }
}

}  // namespace fdtd

using namespace fdtd;

extern "C" {

int fdtd_symplectic_h_f32(const fdtd_grid *gp, float cl, const float *ex, const float *ey, const float *ez,
                          float *hx, float *hy, float *hz, const float *chx, const float *chy, const float *chz,
                          void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!all_nonnull(ex, ey, ez, hx, hy, hz, chx, chy, chz)) return FDTD_ERR_ARG;
    dim3 grid((unsigned)((g.nz + kSympBlock - 1) / kSympBlock), (unsigned)g.ny, (unsigned)g.nx);
    k_symp_h<<<grid, kSympBlock, 0, as_stream(stream)>>>(g, cl, ex, ey, ez, hx, hy, hz, chx, chy, chz);
    return check_launch();
}

int fdtd_symplectic_e_f32(const fdtd_grid *gp, float dl, float *ex, float *ey, float *ez, const float *hx,
                          const float *hy, const float *hz, const float *cex, const float *cey, const float *cez,
                          void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!all_nonnull(ex, ey, ez, hx, hy, hz, cex, cey, cez)) return FDTD_ERR_ARG;
    dim3 grid((unsigned)((g.nz + kSympBlock - 1) / kSympBlock), (unsigned)g.ny, (unsigned)g.nx);
    k_symp_e<<<grid, kSympBlock, 0, as_stream(stream)>>>(g, dl, ex, ey, ez, hx, hy, hz, cex, cey, cez);
    return check_launch();
}

}  // extern "C"
