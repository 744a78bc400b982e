// FP64 form of one 4th-order symplectic stage with its stage-wise CPML: the
// arithmetic of k_symp_stage (symplectic.cu; the stencil and index ranges of
// 4th_order-Symplectic/PyCUDA/100-base.py:17-43, the grouping of
// Python-C/dielectric.c:35-89) evaluated in double precision with separately
// rounded operations, one thread per cell, 64-bit offsets.  CPML tables stay
// the FP32 values of the FP32 path, widened; the caller passes coefficient
// arrays, stage coefficient and uniform ch as the FP32 values widened, so the
// FP32 and FP64 runs discretise the same problem and their difference is the
// FP32 rounding.  Used for the accuracy of the 4th-order workload against
// FP64 at full size.
#include "common.cuh"

namespace fdtd {
namespace s64 {

constexpr int kB = 128;

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double curl4d(double a, double b, double c, double d) {
    return dadd(dsub(dsub(a, b), c), d);
}

struct Stage64 {
    double coef;           // cl (H) or dl (E)
    double cscalar;        // uniform coefficient (H without ch arrays)
    double clch;           // coef * cscalar (H, uniform ch)
    const double *c[3];    // coefficient arrays of the updated components (NULL: uniform)
    int32_t P[3];
    int32_t front[3], back[3];
    const float *b[3], *a[3], *km1[3];  // FP32 tables of the stage, widened
    double *psi[6];
};

template <bool E, bool CARR>
__global__ void __launch_bounds__(kB)
k_symp_stage64(Grid g, Stage64 A, double *__restrict__ ex, double *__restrict__ ey, double *__restrict__ ez,
               double *__restrict__ hx, double *__restrict__ hy, double *__restrict__ hz) {
    const int64_t k = (int64_t)blockIdx.x * kB + threadIdx.x;
    const int64_t j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    const int64_t c = i * g.sx + j * g.sy + k, X = g.sx, Y = g.sy;
    const int64_t n3[3] = {g.nx, g.ny, g.nz}, x3[3] = {i, j, k}, st3[3] = {X, Y, 1};
    int64_t sl[3];
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
        const int64_t P = A.P[ax], n = n3[ax], x = x3[ax];
        int64_t s = -1;
        if (P > 0) {
            if (A.front[ax] && x >= 1 && x <= P) s = x - 1;
            const int64_t b0 = E ? n - P - 1 : n - P, b1 = E ? n - 2 : n - 1;
            if (A.back[ax] && x >= b0 && x <= b1) s = P + x - b0;
        }
        sl[ax] = s;
    }
    const double c27 = 27.0;
    auto deriv = [&](const double *F, int ax) {
        const int64_t st = st3[ax];
        return E ? dsub(dmul(c27, dsub(F[c + st], F[c])), dsub(F[c + 2 * st], F[c - st]))
                 : dsub(dmul(c27, dsub(F[c], F[c - st])), dsub(F[c + st], F[c - 2 * st]));
    };
    auto term = [&](int ax, int w, double d, double cv) {
        const int64_t s = sl[ax], twoP = 2 * (int64_t)A.P[ax];
        const int64_t q = ax == 0 ? (s * g.ny + j) * g.nz + k
                                  : (ax == 1 ? (i * twoP + s) * g.nz + k : (i * g.ny + j) * twoP + s);
        double *ps = A.psi[2 * ax + w];
        const double psi = dadd(dmul((double)A.b[ax][s], ps[q]), dmul((double)A.a[ax][s], d));
        ps[q] = psi;
        return dmul(dmul(A.coef, cv), dadd(dmul((double)A.km1[ax][s], d), psi));
    };
    if (E) {
        const bool jin = j > 0 && j < g.ny - 2, kin = k > 0 && k < g.nz - 2, iin = i > 0 && i < g.nx - 2;
        if (jin && kin) {
            const double n = curl4d(hz[c + Y], hz[c], hy[c + 1], hy[c]);
            const double f = curl4d(hz[c + 2 * Y], hz[c - Y], hy[c + 2], hy[c - 1]);
            const double cv = A.c[0][c];
            double v = dadd(ex[c], dmul(dmul(A.coef, cv), dsub(dmul(c27, n), f)));
            if (sl[1] >= 0) v = dadd(v, term(1, 1, deriv(hz, 1), cv));
            if (sl[2] >= 0) v = dsub(v, term(2, 0, deriv(hy, 2), cv));
            ex[c] = v;
        }
        if (iin && kin) {
            const double n = curl4d(hx[c + 1], hx[c], hz[c + X], hz[c]);
            const double f = curl4d(hx[c + 2], hx[c - 1], hz[c + 2 * X], hz[c - X]);
            const double cv = A.c[1][c];
            double v = dadd(ey[c], dmul(dmul(A.coef, cv), dsub(dmul(c27, n), f)));
            if (sl[0] >= 0) v = dsub(v, term(0, 0, deriv(hz, 0), cv));
            if (sl[2] >= 0) v = dadd(v, term(2, 1, deriv(hx, 2), cv));
            ey[c] = v;
        }
        if (iin && jin) {
            const double n = curl4d(hy[c + X], hy[c], hx[c + Y], hx[c]);
            const double f = curl4d(hy[c + 2 * X], hy[c - X], hx[c + 2 * Y], hx[c - Y]);
            const double cv = A.c[2][c];
            double v = dadd(ez[c], dmul(dmul(A.coef, cv), dsub(dmul(c27, n), f)));
            if (sl[0] >= 0) v = dadd(v, term(0, 1, deriv(hy, 0), cv));
            if (sl[1] >= 0) v = dsub(v, term(1, 0, deriv(hx, 1), cv));
            ez[c] = v;
        }
    } else {
        const bool jin = j > 1 && j < g.ny - 1, kin = k > 1 && k < g.nz - 1, iin = i > 1 && i < g.nx - 1;
        auto stage = [&](double h, double cv, double d27) {
            return dsub(h, dmul(CARR ? dmul(A.coef, cv) : A.clch, d27));
        };
        if (jin && kin) {
            const double n = curl4d(ez[c], ez[c - Y], ey[c], ey[c - 1]);
            const double f = curl4d(ez[c + Y], ez[c - 2 * Y], ey[c + 1], ey[c - 2]);
            const double cv = CARR ? A.c[0][c] : A.cscalar;
            double v = stage(hx[c], cv, dsub(dmul(c27, n), f));
            if (sl[1] >= 0) v = dsub(v, term(1, 1, deriv(ez, 1), cv));
            if (sl[2] >= 0) v = dadd(v, term(2, 0, deriv(ey, 2), cv));
            hx[c] = v;
        }
        if (iin && kin) {
            const double n = curl4d(ex[c], ex[c - 1], ez[c], ez[c - X]);
            const double f = curl4d(ex[c + 1], ex[c - 2], ez[c + X], ez[c - 2 * X]);
            const double cv = CARR ? A.c[1][c] : A.cscalar;
            double v = stage(hy[c], cv, dsub(dmul(c27, n), f));
            if (sl[0] >= 0) v = dadd(v, term(0, 0, deriv(ez, 0), cv));
            if (sl[2] >= 0) v = dsub(v, term(2, 1, deriv(ex, 2), cv));
            hy[c] = v;
        }
        if (iin && jin) {
            const double n = curl4d(ey[c], ey[c - X], ex[c], ex[c - Y]);
            const double f = curl4d(ey[c + X], ey[c - 2 * X], ex[c + Y], ex[c - 2 * Y]);
            const double cv = CARR ? A.c[2][c] : A.cscalar;
            double v = stage(hz[c], cv, dsub(dmul(c27, n), f));
            if (sl[0] >= 0) v = dsub(v, term(0, 1, deriv(ey, 0), cv));
            if (sl[1] >= 0) v = dadd(v, term(1, 0, deriv(ex, 1), cv));
            hz[c] = v;
        }
    }
}

}  // namespace s64
}  // namespace fdtd

using namespace fdtd;
using namespace fdtd::s64;

extern "C" {

int fdtd_symplectic_stage_f64(const fdtd_grid *gp, const fdtd_cpml *cp, int32_t e_or_h, double coef,
                              double ch_scalar, double *const f[6], const double *const cf[3],
                              double *const psi[6], void *stream) {
    NvtxRange nvtx_range("fdtd_symplectic_stage_f64");
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!f || (e_or_h != 0 && e_or_h != 1)) return FDTD_ERR_ARG;
    for (int q = 0; q < 6; q++)
        if (!f[q]) return FDTD_ERR_ARG;
    const bool E = e_or_h == 1;
    const bool carr = cf && cf[0] && cf[1] && cf[2];
    if (cf && !carr && (cf[0] || cf[1] || cf[2])) return FDTD_ERR_ARG;
    if (E && !carr) return FDTD_ERR_ARG;
    Stage64 A{};
    A.coef = coef;
    A.cscalar = ch_scalar;
    A.clch = coef * ch_scalar;  // the FP64 oracle's cl * ch
    for (int q = 0; q < 3; q++) A.c[q] = carr ? cf[q] : nullptr;
    if (cp) {
        if (!psi) return FDTD_ERR_ARG;
        const int64_t n3[3] = {g.nx, g.ny, g.nz};
        for (int ax = 0; ax < 3; ax++) {
            const int P = cp->npml[ax];
            if (P < 0) return FDTD_ERR_ARG;
            A.front[ax] = (cp->faces >> (2 * ax)) & 1;
            A.back[ax] = (cp->faces >> (2 * ax + 1)) & 1;
            if (P == 0 || !(A.front[ax] || A.back[ax])) continue;
            if (n3[ax] < 2 * (int64_t)P + 2) return FDTD_ERR_SHAPE;
            A.P[ax] = P;
            A.b[ax] = E ? cp->b_e[ax] : cp->b_h[ax];
            A.a[ax] = E ? cp->a_e[ax] : cp->a_h[ax];
            A.km1[ax] = E ? cp->km1_e[ax] : cp->km1_h[ax];
            A.psi[2 * ax] = psi[2 * ax];
            A.psi[2 * ax + 1] = psi[2 * ax + 1];
            if (!all_nonnull(A.b[ax], A.a[ax], A.km1[ax], A.psi[2 * ax], A.psi[2 * ax + 1])) return FDTD_ERR_ARG;
        }
    }
    const dim3 grid((unsigned)((g.nz + kB - 1) / kB), (unsigned)g.ny, (unsigned)g.nx);
    cudaStream_t st = as_stream(stream);
    if (E) k_symp_stage64<true, true><<<grid, kB, 0, st>>>(g, A, f[0], f[1], f[2], f[3], f[4], f[5]);
    else if (carr) k_symp_stage64<false, true><<<grid, kB, 0, st>>>(g, A, f[0], f[1], f[2], f[3], f[4], f[5]);
    else k_symp_stage64<false, false><<<grid, kB, 0, st>>>(g, A, f[0], f[1], f[2], f[3], f[4], f[5]);
    return check_launch();
}

}  // extern "C"
