// FP64 form of the 2nd-order step (update_e, cpml_e, sources, update_h,
// cpml_h), one thread per cell, in place.  It evaluates the same expressions
// as the FP32 kernels in double precision with separately rounded operations,
// i.e. the reference's arithmetic (2nd_order-Yee/Numpy/fdtd3d.py:4-13,
// kuFDTD/before_CUDA/v0.3.0/boundary/core/cpml_core.c:238-263) run in FP64.
// Uses: accuracy checks against the FP32 path at full size, and central
// differences of an FP64 loss for the adjoint.  CPML tables and source
// amplitudes stay the FP32 values of the FP32 path, widened to double, so both
// paths discretise the same problem.  ch is the constant 0.5.
#include "common.cuh"

namespace fdtd {
namespace f64 {

constexpr int kB = 128;

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
// ((a - b) - c) + d
__device__ __forceinline__ double curl4d(double a, double b, double c, double d) {
    return dadd(dsub(dsub(a, b), c), d);
}

__global__ void __launch_bounds__(kB) k_update_e(Grid g, double *ex, double *ey, double *ez, const double *hx,
                                                 const double *hy, const double *hz, const double *cex,
                                                 const double *cey, const double *cez) {
    const int64_t k = (int64_t)blockIdx.x * kB + threadIdx.x;
    const int64_t j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    const int64_t c = i * g.sx + j * g.sy + k;
    if (j < g.ny - 1 && k < g.nz - 1) ex[c] = dadd(ex[c], dmul(cex[c], curl4d(hz[c + g.sy], hz[c], hy[c + 1], hy[c])));
    if (i < g.nx - 1 && k < g.nz - 1) ey[c] = dadd(ey[c], dmul(cey[c], curl4d(hx[c + 1], hx[c], hz[c + g.sx], hz[c])));
    if (i < g.nx - 1 && j < g.ny - 1) ez[c] = dadd(ez[c], dmul(cez[c], curl4d(hy[c + g.sx], hy[c], hx[c + g.sy], hx[c])));
}

__global__ void __launch_bounds__(kB) k_update_h(Grid g, const double *ex, const double *ey, const double *ez,
                                                 double *hx, double *hy, double *hz) {
    const int64_t k = (int64_t)blockIdx.x * kB + threadIdx.x;
    const int64_t j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    const int64_t c = i * g.sx + j * g.sy + k;
    if (j > 0 && k > 0) hx[c] = dsub(hx[c], dmul(0.5, curl4d(ez[c], ez[c - g.sy], ey[c], ey[c - 1])));
    if (i > 0 && k > 0) hy[c] = dsub(hy[c], dmul(0.5, curl4d(ex[c], ex[c - 1], ez[c], ez[c - g.sx])));
    if (i > 0 && j > 0) hz[c] = dsub(hz[c], dmul(0.5, curl4d(ey[c], ey[c - g.sx], ex[c], ex[c - g.sy])));
}

struct Axis {
    int P, front, back;
    const float *b, *a, *km1;  // FP32 tables, widened
    double *psi1, *psi2;
};

__device__ __forceinline__ double term(double &psi, double b, double a, double km1, double d) {
    psi = dadd(dmul(b, psi), dmul(a, d));
    return dadd(dmul(km1, d), psi);
}

// One CPML axis for E (EH = 0) or H (EH = 1), both psi arrays of the axis.
//   E: x (eyx: ey -= , ezx: ez +=), y (ezy: ez -=, exy: ex +=), z (exz: ex -=, eyz: ey +=)
//   H: x (hyx: hy +=, hzx: hz -=), y (hzy: hz +=, hxy: hx -=), z (hxz: hx +=, hyz: hy -=)
// f[0..5] = ex, ey, ez, hx, hy, hz; ce = cex, cey, cez (E only).
struct Ptrs {
    double *f[6];        // ex, ey, ez, hx, hy, hz
    const double *ce[3];
};

template <int AX, int EH>
__global__ void __launch_bounds__(kB) k_cpml(Grid g, Axis A, Ptrs ptr) {
    const int P = A.P;
    int64_t i, j, k, s, p;
    if (AX == 0) {
        k = (int64_t)blockIdx.x * kB + threadIdx.x; j = blockIdx.y; s = blockIdx.z;
        if (k >= g.nz) return;
        i = EH ? slab_node_h(s, P, g.nx) : slab_node_e(s, P, g.nx);
        p = (s * g.ny + j) * g.nz + k;
    } else if (AX == 1) {
        k = (int64_t)blockIdx.x * kB + threadIdx.x; s = blockIdx.y; i = blockIdx.z;
        if (k >= g.nz) return;
        j = EH ? slab_node_h(s, P, g.ny) : slab_node_e(s, P, g.ny);
        p = (i * 2 * P + s) * g.nz + k;
    } else {
        const int64_t t = (int64_t)blockIdx.x * kB + threadIdx.x;
        if (t >= g.nx * g.ny * 2 * P) return;
        s = t % (2 * P); j = (t / (2 * P)) % g.ny; i = t / (2 * P * g.ny);
        k = EH ? slab_node_h(s, P, g.nz) : slab_node_e(s, P, g.nz);
        p = t;
    }
    if (!(s < P ? A.front : A.back)) return;
    const int64_t c = i * g.sx + j * g.sy + k;
    const double b = A.b[s], a = A.a[s], km1 = A.km1[s];
    // (target, source, source stride, validity, sign) of psi1 and psi2
    const int64_t st = AX == 0 ? g.sx : AX == 1 ? g.sy : 1;
    int t1, s1, t2, s2;
    bool v1, v2;
    if (EH == 0) {
        t1 = AX == 0 ? 1 : AX == 1 ? 2 : 0;  s1 = AX == 0 ? 5 : AX == 1 ? 3 : 4;  // ey<-hz, ez<-hx, ex<-hy
        t2 = AX == 0 ? 2 : AX == 1 ? 0 : 1;  s2 = AX == 0 ? 4 : AX == 1 ? 5 : 3;  // ez<-hy, ex<-hz, ey<-hx
        v1 = AX == 0 ? k < g.nz - 1 : AX == 1 ? i < g.nx - 1 : j < g.ny - 1;
        v2 = AX == 0 ? j < g.ny - 1 : AX == 1 ? k < g.nz - 1 : i < g.nx - 1;
    } else {
        t1 = AX == 0 ? 4 : AX == 1 ? 5 : 3;  s1 = AX == 0 ? 2 : AX == 1 ? 0 : 1;  // hy<-ez, hz<-ex, hx<-ey
        t2 = AX == 0 ? 5 : AX == 1 ? 3 : 4;  s2 = AX == 0 ? 1 : AX == 1 ? 2 : 0;  // hz<-ey, hx<-ez, hy<-ex
        v1 = AX == 0 ? k > 0 : AX == 1 ? i > 0 : j > 0;
        v2 = AX == 0 ? j > 0 : AX == 1 ? k > 0 : i > 0;
    }
    if (v1) {
        const double *src = ptr.f[s1];
        const double d = EH == 0 ? dsub(src[c + st], src[c]) : dsub(src[c], src[c - st]);
        double psi = A.psi1[p];
        const double tt = term(psi, b, a, km1, d);
        A.psi1[p] = psi;
        double *f = ptr.f[t1];
        const double coef = EH == 0 ? ptr.ce[t1][c] : 0.5;
        f[c] = EH == 0 ? dsub(f[c], dmul(coef, tt)) : dadd(f[c], dmul(coef, tt));
    }
    if (v2) {
        const double *src = ptr.f[s2];
        const double d = EH == 0 ? dsub(src[c + st], src[c]) : dsub(src[c], src[c - st]);
        double psi = A.psi2[p];
        const double tt = term(psi, b, a, km1, d);
        A.psi2[p] = psi;
        double *f = ptr.f[t2];
        const double coef = EH == 0 ? ptr.ce[t2][c] : 0.5;
        f[c] = EH == 0 ? dadd(f[c], dmul(coef, tt)) : dsub(f[c], dmul(coef, tt));
    }
}

// sources in list order (one thread: repeated cells add in order)
__global__ void k_sources(Grid g, fdtd_sources src, int64_t t, double *ex, double *ey, double *ez) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (t < 0 || t >= src.namp) return;
    for (int s = 0; s < src.nsrc; s++) {
        const int64_t si = src.ijk[3 * s], sj = src.ijk[3 * s + 1], sk = src.ijk[3 * s + 2];
        if (si < 0 || si >= g.nx || sj < 0 || sj >= g.ny || sk < 0 || sk >= g.nz) continue;
        const int64_t c = si * g.sx + sj * g.sy + sk;
        double *f = src.comp[s] == 0 ? ex : (src.comp[s] == 1 ? ey : ez);
        f[c] = dadd(f[c], (double)src.amp[(int64_t)s * src.namp + t]);
    }
}

// out[p] = f[comp[p]][i, j, k] (NaN outside the grid)
__global__ void k_gather(Grid g, fdtd_points pts, const double *f0, const double *f1, const double *f2,
                         const double *f3, const double *f4, const double *f5, double *out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= pts.n) return;
    const int64_t i = pts.ijk[3 * p], j = pts.ijk[3 * p + 1], k = pts.ijk[3 * p + 2];
    const int q = pts.comp[p];
    if (i < 0 || i >= g.nx || j < 0 || j >= g.ny || k < 0 || k >= g.nz || q < 0 || q > 5) {
        out[p] = __longlong_as_double(0x7ff8000000000000ll);
        return;
    }
    const double *f = q == 0 ? f0 : q == 1 ? f1 : q == 2 ? f2 : q == 3 ? f3 : q == 4 ? f4 : f5;
    out[p] = f[i * g.sx + j * g.sy + k];
}

template <int AX, int EH>
static void launch_axis(const Grid &g, const Axis &A, const Ptrs &ptr, cudaStream_t st) {
    dim3 grid;
    if (AX == 0) grid = dim3((unsigned)((g.nz + kB - 1) / kB), (unsigned)g.ny, (unsigned)(2 * A.P));
    else if (AX == 1) grid = dim3((unsigned)((g.nz + kB - 1) / kB), (unsigned)(2 * A.P), (unsigned)g.nx);
    else grid = dim3((unsigned)((g.nx * g.ny * 2 * A.P + kB - 1) / kB));
    k_cpml<AX, EH><<<grid, kB, 0, st>>>(g, A, ptr);
}

}  // namespace f64
}  // namespace fdtd

using namespace fdtd;
using namespace fdtd::f64;

extern "C" {

int fdtd_step_unfused_f64(const fdtd_grid *gp, double *const f[6], const double *const ce[3], const fdtd_cpml *c,
                          double *const psi_e[6], double *const psi_h[6], const fdtd_sources *src, int64_t t,
                          void *stream) {
    NvtxRange nvtx_range("fdtd_step_unfused_f64");
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!f || !ce) return FDTD_ERR_ARG;
    if (!all_nonnull(f[0], f[1], f[2], f[3], f[4], f[5], ce[0], ce[1], ce[2])) return FDTD_ERR_ARG;
    const bool pml = c && (c->npml[0] > 0 || c->npml[1] > 0 || c->npml[2] > 0);
    Axis ax[3];
    const int64_t n[3] = {g.nx, g.ny, g.nz};
    for (int a = 0; a < 3; a++) {
        ax[a] = Axis{0, 0, 0, nullptr, nullptr, nullptr, nullptr, nullptr};
        if (!pml || c->npml[a] <= 0) continue;
        const int P = c->npml[a];
        if (n[a] < 2 * P + 2) return FDTD_ERR_SHAPE;
        if (a < 2 && 2 * P > 65535) return FDTD_ERR_SHAPE;
        if (!psi_e || !psi_h) return FDTD_ERR_ARG;
        if (!all_nonnull(c->b_e[a], c->a_e[a], c->km1_e[a], c->b_h[a], c->a_h[a], c->km1_h[a], psi_e[2 * a],
                         psi_e[2 * a + 1], psi_h[2 * a], psi_h[2 * a + 1]))
            return FDTD_ERR_ARG;
        ax[a].P = P;
        ax[a].front = (c->faces >> (2 * a)) & 1;
        ax[a].back = (c->faces >> (2 * a + 1)) & 1;
    }
    if (src) {
        if (src->nsrc < 0 || src->namp < 0) return FDTD_ERR_ARG;
        if (src->nsrc > 0 && !all_nonnull(src->ijk, src->comp, src->amp)) return FDTD_ERR_ARG;
    }
    cudaStream_t st = as_stream(stream);
    Ptrs ptr;
    for (int q = 0; q < 6; q++) ptr.f[q] = f[q];
    for (int q = 0; q < 3; q++) ptr.ce[q] = ce[q];
    const dim3 cells((unsigned)((g.nz + kB - 1) / kB), (unsigned)g.ny, (unsigned)g.nx);
    k_update_e<<<cells, kB, 0, st>>>(g, f[0], f[1], f[2], f[3], f[4], f[5], ce[0], ce[1], ce[2]);
    for (int a = 0; a < 3; a++) {
        if (!ax[a].P) continue;
        Axis A = ax[a];
        A.b = c->b_e[a]; A.a = c->a_e[a]; A.km1 = c->km1_e[a];
        A.psi1 = psi_e[2 * a]; A.psi2 = psi_e[2 * a + 1];
        if (a == 0) launch_axis<0, 0>(g, A, ptr, st);
        else if (a == 1) launch_axis<1, 0>(g, A, ptr, st);
        else launch_axis<2, 0>(g, A, ptr, st);
    }
    if (src && src->nsrc > 0) k_sources<<<1, 32, 0, st>>>(g, *src, t, f[0], f[1], f[2]);
    k_update_h<<<cells, kB, 0, st>>>(g, f[0], f[1], f[2], f[3], f[4], f[5]);
    for (int a = 0; a < 3; a++) {
        if (!ax[a].P) continue;
        Axis A = ax[a];
        A.b = c->b_h[a]; A.a = c->a_h[a]; A.km1 = c->km1_h[a];
        A.psi1 = psi_h[2 * a]; A.psi2 = psi_h[2 * a + 1];
        if (a == 0) launch_axis<0, 1>(g, A, ptr, st);
        else if (a == 1) launch_axis<1, 1>(g, A, ptr, st);
        else launch_axis<2, 1>(g, A, ptr, st);
    }
    return check_launch();
}

int fdtd_add_sources_f64(const fdtd_grid *gp, const fdtd_sources *src, int64_t t, double *ex, double *ey,
                         double *ez, void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!src || src->nsrc < 0 || src->namp < 0) return FDTD_ERR_ARG;
    if (src->nsrc == 0) return FDTD_OK;
    if (!all_nonnull(src->ijk, src->comp, src->amp, ex, ey, ez)) return FDTD_ERR_ARG;
    k_sources<<<1, 32, 0, as_stream(stream)>>>(g, *src, t, ex, ey, ez);
    return check_launch();
}

int fdtd_gather_points_f64(const fdtd_grid *gp, const fdtd_points *pts, const double *const f[6], double *out,
                           void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!pts || pts->n < 0) return FDTD_ERR_ARG;
    if (pts->n == 0) return FDTD_OK;
    if (!all_nonnull(pts->ijk, pts->comp) || !f || !out) return FDTD_ERR_ARG;
    k_gather<<<(pts->n + 127) / 128, 128, 0, as_stream(stream)>>>(g, *pts, f[0], f[1], f[2], f[3], f[4], f[5], out);
    return check_launch();
}

}  // extern "C"
