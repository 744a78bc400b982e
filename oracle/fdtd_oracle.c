/*
 * CPU oracle for the Yee time step -- TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C, the arithmetic of the reference's CPU
 * implementations of the FDTD hot path so that the CUDA kernels of this
 * package can be checked against it.  It is built twice: with REAL=float
 * (bit-level parity target for the FP32 CUDA kernels) and REAL=double (the
 * FP64 accuracy oracle).  Only tests/, the smoke check and the CPU-baseline
 * leg of the benchmark may load it; no product code path calls it.
 *
 * Compile with -ffp-contract=off: every product and sum is rounded on its
 * own, exactly as NumPy evaluates the reference's array expressions.
 *
 * Array convention (identical to the reference's NumPy arrays): C order,
 * logical shape (nx, ny, nz), z fastest; g[3] = x stride, g[4] = y stride in
 * elements (z stride 1), so padded (pitched) storage is allowed.
 *
 * References (paths inside the wbkifun/fdtd_accelerate project):
 *   update_e / update_h      2nd_order-Yee/Numpy/fdtd3d.py:4-13
 *                            (operation grouping ((a-b)-c)+d as NumPy
 *                            evaluates it left to right)
 *   coefficient arrays ch    KEMP/v0.7_pml/fdtd3d/naive/core.py:37-47
 *   periodic planes          2nd_order-Yee/Numpy/fdtd3d.py:16-37
 *   CPML psi recursion       kuFDTD/v0.2.0/dim3/cpu/core/cpml_non_kappa.c:14-429
 *                            (slab index ranges, psi = b*psi + a*dF)
 *   kappa correction term    kuFDTD/before_CUDA/v0.3.0/boundary/core/cpml_core.c:238-263
 *                            (F += -/+ c*((1/kappa-1)*dF + psi), ds = 1)
 *   soft source              2nd_order-Yee/CUDA/fdtd3d_201_250x250x320cell_15npml_100000tstep.cu:352-363
 *                            and KEMP/v0.7_pml/fdtd3d/naive/incident_direct.py:52-70
 *   Drude ADE (E pass)       kuFDTD/v0.2.0/dim3/cpu/core/drude_ade.c:48-93
 *                            (e' = e - ce*J; J = cja*J + cjb*e', per
 *                            component, on a sub-box of the E arrays)
 *   4th-order stages         4th_order-Symplectic/PyCUDA/100-base.py:10-44
 *                            (index ranges of the CUDA kernels; grouping of
 *                            4th_order-Symplectic/Python-C/dielectric.c:35-89)
 */
#include <stdint.h>
#include <stddef.h>

#ifndef REAL
#define REAL float
#endif
#ifndef SFX
#define SFX _f32
#endif
#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(orc_, CAT(name, SFX))

#define GRID                                                                   \
    const int64_t nx = g[0], ny = g[1], nz = g[2], sx = g[3], sy = g[4];     \
    (void)nx; (void)ny; (void)nz; (void)sx; (void)sy

/* ------------------------------------------------------------------------ */
/* a2: E update, fdtd3d.py:10-13                                             */
/* ------------------------------------------------------------------------ */
void FN(update_e)(const int64_t *g, REAL *ex, REAL *ey, REAL *ez,
                  const REAL *hx, const REAL *hy, const REAL *hz,
                  const REAL *cex, const REAL *cey, const REAL *cez)
{
    GRID;
#pragma omp parallel for collapse(2) schedule(static)
    for (int64_t i = 0; i < nx; i++)
        for (int64_t j = 0; j < ny; j++)
            for (int64_t k = 0; k < nz; k++) {
                const int64_t c = i * sx + j * sy + k;
                if (j < ny - 1 && k < nz - 1) {
                    REAL s = ((hz[c + sy] - hz[c]) - hy[c + 1]) + hy[c];
                    ex[c] = ex[c] + cex[c] * s;
                }
                if (i < nx - 1 && k < nz - 1) {
                    REAL s = ((hx[c + 1] - hx[c]) - hz[c + sx]) + hz[c];
                    ey[c] = ey[c] + cey[c] * s;
                }
                if (i < nx - 1 && j < ny - 1) {
                    REAL s = ((hy[c + sx] - hy[c]) - hx[c + sy]) + hx[c];
                    ez[c] = ez[c] + cez[c] * s;
                }
            }
}

/* ------------------------------------------------------------------------ */
/* a1: H update, fdtd3d.py:4-7; ch arrays optional (NULL -> 0.5)             */
/* ------------------------------------------------------------------------ */
void FN(update_h)(const int64_t *g, const REAL *ex, const REAL *ey, const REAL *ez,
                  REAL *hx, REAL *hy, REAL *hz,
                  const REAL *chx, const REAL *chy, const REAL *chz)
{
    GRID;
    const REAL half = (REAL)0.5;
#pragma omp parallel for collapse(2) schedule(static)
    for (int64_t i = 0; i < nx; i++)
        for (int64_t j = 0; j < ny; j++)
            for (int64_t k = 0; k < nz; k++) {
                const int64_t c = i * sx + j * sy + k;
                if (j > 0 && k > 0) {
                    REAL s = ((ez[c] - ez[c - sy]) - ey[c]) + ey[c - 1];
                    hx[c] = hx[c] - (chx ? chx[c] : half) * s;
                }
                if (i > 0 && k > 0) {
                    REAL s = ((ex[c] - ex[c - 1]) - ez[c]) + ez[c - sx];
                    hy[c] = hy[c] - (chy ? chy[c] : half) * s;
                }
                if (i > 0 && j > 0) {
                    REAL s = ((ey[c] - ey[c - sx]) - ex[c]) + ex[c - sy];
                    hz[c] = hz[c] - (chz ? chz[c] : half) * s;
                }
            }
}

/* ------------------------------------------------------------------------ */
/* a12: periodic planes, fdtd3d.py:16-37 (axes bit 0=x, 1=y, 2=z)            */
/* ------------------------------------------------------------------------ */
void FN(pbc_h)(const int64_t *g, int axes, REAL *hx, REAL *hy, REAL *hz)
{
    GRID;
    if (axes & 1)
        for (int64_t j = 0; j < ny; j++)
            for (int64_t k = 0; k < nz; k++) {
                const int64_t d = j * sy + k, s = (nx - 1) * sx + d;
                hy[d] = hy[s];
                hz[d] = hz[s];
            }
    if (axes & 2)
        for (int64_t i = 0; i < nx; i++)
            for (int64_t k = 0; k < nz; k++) {
                const int64_t d = i * sx + k, s = d + (ny - 1) * sy;
                hz[d] = hz[s];
                hx[d] = hx[s];
            }
    if (axes & 4)
        for (int64_t i = 0; i < nx; i++)
            for (int64_t j = 0; j < ny; j++) {
                const int64_t d = i * sx + j * sy, s = d + nz - 1;
                hx[d] = hx[s];
                hy[d] = hy[s];
            }
}

void FN(pbc_e)(const int64_t *g, int axes, REAL *ex, REAL *ey, REAL *ez)
{
    GRID;
    if (axes & 1)
        for (int64_t j = 0; j < ny; j++)
            for (int64_t k = 0; k < nz; k++) {
                const int64_t s = j * sy + k, d = (nx - 1) * sx + s;
                ey[d] = ey[s];
                ez[d] = ez[s];
            }
    if (axes & 2)
        for (int64_t i = 0; i < nx; i++)
            for (int64_t k = 0; k < nz; k++) {
                const int64_t s = i * sx + k, d = s + (ny - 1) * sy;
                ez[d] = ez[s];
                ex[d] = ex[s];
            }
    if (axes & 4)
        for (int64_t i = 0; i < nx; i++)
            for (int64_t j = 0; j < ny; j++) {
                const int64_t s = i * sx + j * sy, d = s + nz - 1;
                ex[d] = ex[s];
                ey[d] = ey[s];
            }
}

/* ------------------------------------------------------------------------ */
/* a5/a6: CPML with kappa.                                                   */
/*                                                                          */
/* Slab index s in [0, 2P): s < P is the front slab, node index s+1; s >= P  */
/* is the back slab, node index n-P-1+(s-P) for E nodes and n-P+(s-P) for H */
/* nodes (the ranges of cpml_non_kappa.c:59-60,127-128).  Tables b, a, km1  */
/* (= 1/kappa - 1) have 2P entries per axis.  psi layouts:                  */
/*   x slab (2P, ny, nz), y slab (nx, 2P, nz), z slab (nx, ny, 2P), dense.  */
/* A face is skipped when its bit in `faces` is clear (bit 2a front,        */
/* 2a+1 back).  Updates happen only where the main update touches the      */
/* component, so psi stays zero on the PEC planes.                          */
/* ------------------------------------------------------------------------ */
static inline int64_t slab_node_e(int64_t s, int64_t P, int64_t n) { return s < P ? s + 1 : n - P - 1 + (s - P); }
static inline int64_t slab_node_h(int64_t s, int64_t P, int64_t n) { return s < P ? s + 1 : n - P + (s - P); }
static inline int face_on(int faces, int axis, int64_t s, int64_t P) { return (faces >> (2 * axis + (s < P ? 0 : 1))) & 1; }

/* psi[axis][0/1]: x:(eyx, ezx) y:(ezy, exy) z:(exz, eyz) */
void FN(cpml_e)(const int64_t *g, const int32_t *npml, int faces,
                const REAL *const *b, const REAL *const *a, const REAL *const *km1,
                REAL *ex, REAL *ey, REAL *ez,
                const REAL *hx, const REAL *hy, const REAL *hz,
                const REAL *cex, const REAL *cey, const REAL *cez,
                REAL *const *psi)
{
    GRID;
    /* x axis: ey -= cey*(...dHz/dx...), ez += cez*(...dHy/dx...) */
    if (npml[0] > 0) {
        const int64_t P = npml[0];
        REAL *p1 = psi[0], *p2 = psi[1];
#pragma omp parallel for collapse(2) schedule(static)
        for (int64_t s = 0; s < 2 * P; s++)
            for (int64_t j = 0; j < ny; j++) {
                if (!face_on(faces, 0, s, P)) continue;
                const int64_t i = slab_node_e(s, P, nx);
                const REAL bb = b[0][s], aa = a[0][s], kk = km1[0][s];
                for (int64_t k = 0; k < nz; k++) {
                    const int64_t c = i * sx + j * sy + k, p = (s * ny + j) * nz + k;
                    if (k < nz - 1) {
                        REAL d = hz[c + sx] - hz[c];
                        p1[p] = bb * p1[p] + aa * d;
                        ey[c] = ey[c] - cey[c] * (kk * d + p1[p]);
                    }
                    if (j < ny - 1) {
                        REAL d = hy[c + sx] - hy[c];
                        p2[p] = bb * p2[p] + aa * d;
                        ez[c] = ez[c] + cez[c] * (kk * d + p2[p]);
                    }
                }
            }
    }
    /* y axis: ez -= cez*(...dHx/dy...), ex += cex*(...dHz/dy...) */
    if (npml[1] > 0) {
        const int64_t P = npml[1];
        REAL *p1 = psi[2], *p2 = psi[3];
#pragma omp parallel for collapse(2) schedule(static)
        for (int64_t i = 0; i < nx; i++)
            for (int64_t s = 0; s < 2 * P; s++) {
                if (!face_on(faces, 1, s, P)) continue;
                const int64_t j = slab_node_e(s, P, ny);
                const REAL bb = b[1][s], aa = a[1][s], kk = km1[1][s];
                for (int64_t k = 0; k < nz; k++) {
                    const int64_t c = i * sx + j * sy + k, p = (i * 2 * P + s) * nz + k;
                    if (i < nx - 1) {
                        REAL d = hx[c + sy] - hx[c];
                        p1[p] = bb * p1[p] + aa * d;
                        ez[c] = ez[c] - cez[c] * (kk * d + p1[p]);
                    }
                    if (k < nz - 1) {
                        REAL d = hz[c + sy] - hz[c];
                        p2[p] = bb * p2[p] + aa * d;
                        ex[c] = ex[c] + cex[c] * (kk * d + p2[p]);
                    }
                }
            }
    }
    /* z axis: ex -= cex*(...dHy/dz...), ey += cey*(...dHx/dz...) */
    if (npml[2] > 0) {
        const int64_t P = npml[2];
        REAL *p1 = psi[4], *p2 = psi[5];
#pragma omp parallel for collapse(2) schedule(static)
        for (int64_t i = 0; i < nx; i++)
            for (int64_t j = 0; j < ny; j++)
                for (int64_t s = 0; s < 2 * P; s++) {
                    if (!face_on(faces, 2, s, P)) continue;
                    const int64_t k = slab_node_e(s, P, nz);
                    const REAL bb = b[2][s], aa = a[2][s], kk = km1[2][s];
                    const int64_t c = i * sx + j * sy + k, p = (i * ny + j) * 2 * P + s;
                    if (j < ny - 1) {
                        REAL d = hy[c + 1] - hy[c];
                        p1[p] = bb * p1[p] + aa * d;
                        ex[c] = ex[c] - cex[c] * (kk * d + p1[p]);
                    }
                    if (i < nx - 1) {
                        REAL d = hx[c + 1] - hx[c];
                        p2[p] = bb * p2[p] + aa * d;
                        ey[c] = ey[c] + cey[c] * (kk * d + p2[p]);
                    }
                }
    }
}

/* psi[axis][0/1]: x:(hyx, hzx) y:(hzy, hxy) z:(hxz, hyz); ch NULL -> 0.5 */
void FN(cpml_h)(const int64_t *g, const int32_t *npml, int faces,
                const REAL *const *b, const REAL *const *a, const REAL *const *km1,
                const REAL *ex, const REAL *ey, const REAL *ez,
                REAL *hx, REAL *hy, REAL *hz,
                const REAL *chx, const REAL *chy, const REAL *chz,
                REAL *const *psi)
{
    GRID;
    const REAL half = (REAL)0.5;
    if (npml[0] > 0) {
        const int64_t P = npml[0];
        REAL *p1 = psi[0], *p2 = psi[1];
#pragma omp parallel for collapse(2) schedule(static)
        for (int64_t s = 0; s < 2 * P; s++)
            for (int64_t j = 0; j < ny; j++) {
                if (!face_on(faces, 0, s, P)) continue;
                const int64_t i = slab_node_h(s, P, nx);
                const REAL bb = b[0][s], aa = a[0][s], kk = km1[0][s];
                for (int64_t k = 0; k < nz; k++) {
                    const int64_t c = i * sx + j * sy + k, p = (s * ny + j) * nz + k;
                    if (k > 0) {
                        REAL d = ez[c] - ez[c - sx];
                        p1[p] = bb * p1[p] + aa * d;
                        hy[c] = hy[c] + (chy ? chy[c] : half) * (kk * d + p1[p]);
                    }
                    if (j > 0) {
                        REAL d = ey[c] - ey[c - sx];
                        p2[p] = bb * p2[p] + aa * d;
                        hz[c] = hz[c] - (chz ? chz[c] : half) * (kk * d + p2[p]);
                    }
                }
            }
    }
    if (npml[1] > 0) {
        const int64_t P = npml[1];
        REAL *p1 = psi[2], *p2 = psi[3];
#pragma omp parallel for collapse(2) schedule(static)
        for (int64_t i = 0; i < nx; i++)
            for (int64_t s = 0; s < 2 * P; s++) {
                if (!face_on(faces, 1, s, P)) continue;
                const int64_t j = slab_node_h(s, P, ny);
                const REAL bb = b[1][s], aa = a[1][s], kk = km1[1][s];
                for (int64_t k = 0; k < nz; k++) {
                    const int64_t c = i * sx + j * sy + k, p = (i * 2 * P + s) * nz + k;
                    if (i > 0) {
                        REAL d = ex[c] - ex[c - sy];
                        p1[p] = bb * p1[p] + aa * d;
                        hz[c] = hz[c] + (chz ? chz[c] : half) * (kk * d + p1[p]);
                    }
                    if (k > 0) {
                        REAL d = ez[c] - ez[c - sy];
                        p2[p] = bb * p2[p] + aa * d;
                        hx[c] = hx[c] - (chx ? chx[c] : half) * (kk * d + p2[p]);
                    }
                }
            }
    }
    if (npml[2] > 0) {
        const int64_t P = npml[2];
        REAL *p1 = psi[4], *p2 = psi[5];
#pragma omp parallel for collapse(2) schedule(static)
        for (int64_t i = 0; i < nx; i++)
            for (int64_t j = 0; j < ny; j++)
                for (int64_t s = 0; s < 2 * P; s++) {
                    if (!face_on(faces, 2, s, P)) continue;
                    const int64_t k = slab_node_h(s, P, nz);
                    const REAL bb = b[2][s], aa = a[2][s], kk = km1[2][s];
                    const int64_t c = i * sx + j * sy + k, p = (i * ny + j) * 2 * P + s;
                    if (j > 0) {
                        REAL d = ey[c] - ey[c - 1];
                        p1[p] = bb * p1[p] + aa * d;
                        hx[c] = hx[c] + (chx ? chx[c] : half) * (kk * d + p1[p]);
                    }
                    if (i > 0) {
                        REAL d = ex[c] - ex[c - 1];
                        p2[p] = bb * p2[p] + aa * d;
                        hy[c] = hy[c] - (chy ? chy[c] : half) * (kk * d + p2[p]);
                    }
                }
    }
}

/* ------------------------------------------------------------------------ */
/* a7: soft source, F[offset] += amp, in list order                          */
/* ------------------------------------------------------------------------ */
void FN(add_points)(REAL *f, const int64_t *offsets, const REAL *amp, int64_t n)
{
    for (int64_t p = 0; p < n; p++) f[offsets[p]] = f[offsets[p]] + amp[p];
}

/* ------------------------------------------------------------------------ */
/* a10: 4th-order symplectic stages (C order; index ranges of the CUDA     */
/* kernels in 100-base.py:17-43).  c = stage coefficient, ch/ce arrays.     */
/* ------------------------------------------------------------------------ */
void FN(symp_h)(const int64_t *g, REAL cl, const REAL *ex, const REAL *ey, const REAL *ez,
                REAL *hx, REAL *hy, REAL *hz,
                const REAL *chx, const REAL *chy, const REAL *chz)
{
    GRID;
    const REAL c27 = (REAL)27;
#pragma omp parallel for collapse(2) schedule(static)
    for (int64_t i = 0; i < nx; i++)
        for (int64_t j = 0; j < ny; j++)
            for (int64_t k = 0; k < nz; k++) {
                const int64_t c = i * sx + j * sy + k;
                if (j > 1 && j < ny - 1 && k > 1 && k < nz - 1) {
                    REAL n = ((ez[c] - ez[c - sy]) - ey[c]) + ey[c - 1];
                    REAL f = ((ez[c + sy] - ez[c - 2 * sy]) - ey[c + 1]) + ey[c - 2];
                    hx[c] = hx[c] - (cl * chx[c]) * (c27 * n - f);
                }
                if (i > 1 && i < nx - 1 && k > 1 && k < nz - 1) {
                    REAL n = ((ex[c] - ex[c - 1]) - ez[c]) + ez[c - sx];
                    REAL f = ((ex[c + 1] - ex[c - 2]) - ez[c + sx]) + ez[c - 2 * sx];
                    hy[c] = hy[c] - (cl * chy[c]) * (c27 * n - f);
                }
                if (i > 1 && i < nx - 1 && j > 1 && j < ny - 1) {
                    REAL n = ((ey[c] - ey[c - sx]) - ex[c]) + ex[c - sy];
                    REAL f = ((ey[c + sx] - ey[c - 2 * sx]) - ex[c + sy]) + ex[c - 2 * sy];
                    hz[c] = hz[c] - (cl * chz[c]) * (c27 * n - f);
                }
            }
}

void FN(symp_e)(const int64_t *g, REAL dl, REAL *ex, REAL *ey, REAL *ez,
                const REAL *hx, const REAL *hy, const REAL *hz,
                const REAL *cex, const REAL *cey, const REAL *cez)
{
    GRID;
    const REAL c27 = (REAL)27;
#pragma omp parallel for collapse(2) schedule(static)
    for (int64_t i = 0; i < nx; i++)
        for (int64_t j = 0; j < ny; j++)
            for (int64_t k = 0; k < nz; k++) {
                const int64_t c = i * sx + j * sy + k;
                if (j > 0 && j < ny - 2 && k > 0 && k < nz - 2) {
                    REAL n = ((hz[c + sy] - hz[c]) - hy[c + 1]) + hy[c];
                    REAL f = ((hz[c + 2 * sy] - hz[c - sy]) - hy[c + 2]) + hy[c - 1];
                    ex[c] = ex[c] + (dl * cex[c]) * (c27 * n - f);
                }
                if (i > 0 && i < nx - 2 && k > 0 && k < nz - 2) {
                    REAL n = ((hx[c + 1] - hx[c]) - hz[c + sx]) + hz[c];
                    REAL f = ((hx[c + 2] - hx[c - 1]) - hz[c + 2 * sx]) + hz[c - sx];
                    ey[c] = ey[c] + (dl * cey[c]) * (c27 * n - f);
                }
                if (i > 0 && i < nx - 2 && j > 0 && j < ny - 2) {
                    REAL n = ((hy[c + sx] - hy[c]) - hx[c + sy]) + hx[c];
                    REAL f = ((hy[c + 2 * sx] - hy[c - sx]) - hx[c + 2 * sy]) + hx[c - sy];
                    ez[c] = ez[c] + (dl * cez[c]) * (c27 * n - f);
                }
            }
}

/* ------------------------------------------------------------------------ */
/* 4th-order CPML (builder-defined: the reference has none).  Same slab     */
/* geometry and psi layout as the 2nd-order CPML; the derivative along the  */
/* slab axis is the 4th-order combination d = 27*(near) - (far) of the      */
/* stage stencil; per stage: psi = b*psi + a*d and                          */
/* F -/+= (c*coef)*(km1*d + psi), only where the stage updates F.            */
/* E nodes use d = 27*(F[i+1]-F[i]) - (F[i+2]-F[i-1]);                      */
/* H nodes use d = 27*(F[i]-F[i-1]) - (F[i+1]-F[i-2]).                      */
/* ------------------------------------------------------------------------ */
static inline REAL d4e(const REAL *F, int64_t c, int64_t st)
{
    return (REAL)27 * (F[c + st] - F[c]) - (F[c + 2 * st] - F[c - st]);
}
static inline REAL d4h(const REAL *F, int64_t c, int64_t st)
{
    return (REAL)27 * (F[c] - F[c - st]) - (F[c + st] - F[c - 2 * st]);
}

/* coef: E stage coefficient dl; ce arrays. psi[6] as cpml_e. */
void FN(symp_cpml_e)(const int64_t *g, const int32_t *npml, int faces, REAL dl,
                     const REAL *const *b, const REAL *const *a, const REAL *const *km1,
                     REAL *ex, REAL *ey, REAL *ez,
                     const REAL *hx, const REAL *hy, const REAL *hz,
                     const REAL *cex, const REAL *cey, const REAL *cez,
                     REAL *const *psi)
{
    GRID;
    for (int ax = 0; ax < 3; ax++) {
        const int64_t P = npml[ax];
        if (P <= 0) continue;
        const int64_t n_ax = ax == 0 ? nx : (ax == 1 ? ny : nz);
        const int64_t st_ax = ax == 0 ? sx : (ax == 1 ? sy : 1);
        REAL *p1 = psi[2 * ax], *p2 = psi[2 * ax + 1];
#pragma omp parallel for collapse(2) schedule(static)
        for (int64_t i = 0; i < nx; i++)
            for (int64_t j = 0; j < ny; j++)
                for (int64_t k = 0; k < nz; k++) {
                    const int64_t idx = ax == 0 ? i : (ax == 1 ? j : k);
                    int64_t s;
                    if ((faces >> (2 * ax)) & 1 && idx >= 1 && idx <= P) s = idx - 1;
                    else if ((faces >> (2 * ax + 1)) & 1 && idx >= n_ax - P - 1 && idx <= n_ax - 2)
                        s = P + idx - (n_ax - P - 1);
                    else continue;
                    const int64_t c = i * sx + j * sy + k;
                    const int64_t q = ax == 0 ? (s * ny + j) * nz + k
                                    : ax == 1 ? (i * 2 * P + s) * nz + k
                                              : (i * ny + j) * 2 * P + s;
                    const REAL bb = b[ax][s], aa = a[ax][s], kk = km1[ax][s];
                    /* update ranges: ex j,k in [1,n-3]; ey i,k; ez i,j */
                    const int ok_i = i >= 1 && i <= nx - 3, ok_j = j >= 1 && j <= ny - 3,
                              ok_k = k >= 1 && k <= nz - 3;
                    REAL *f1, *f2;
                    const REAL *g1, *g2, *c1, *c2;
                    int ok1, ok2;
                    REAL s1, s2;
                    if (ax == 0) { f1 = ey; g1 = hz; c1 = cey; ok1 = ok_i && ok_k; s1 = -1;
                                   f2 = ez; g2 = hy; c2 = cez; ok2 = ok_i && ok_j; s2 = +1; }
                    else if (ax == 1) { f1 = ez; g1 = hx; c1 = cez; ok1 = ok_i && ok_j; s1 = -1;
                                        f2 = ex; g2 = hz; c2 = cex; ok2 = ok_j && ok_k; s2 = +1; }
                    else { f1 = ex; g1 = hy; c1 = cex; ok1 = ok_j && ok_k; s1 = -1;
                           f2 = ey; g2 = hx; c2 = cey; ok2 = ok_i && ok_k; s2 = +1; }
                    if (ok1) {
                        REAL d = d4e(g1, c, st_ax);
                        p1[q] = bb * p1[q] + aa * d;
                        REAL t = (dl * c1[c]) * (kk * d + p1[q]);
                        f1[c] = s1 > 0 ? f1[c] + t : f1[c] - t;
                    }
                    if (ok2) {
                        REAL d = d4e(g2, c, st_ax);
                        p2[q] = bb * p2[q] + aa * d;
                        REAL t = (dl * c2[c]) * (kk * d + p2[q]);
                        f2[c] = s2 > 0 ? f2[c] + t : f2[c] - t;
                    }
                }
    }
}

/* coef: H stage coefficient cl; ch arrays or NULL -> ch_scalar. psi[6] as cpml_h. */
void FN(symp_cpml_h)(const int64_t *g, const int32_t *npml, int faces, REAL cl, REAL ch_scalar,
                     const REAL *const *b, const REAL *const *a, const REAL *const *km1,
                     const REAL *ex, const REAL *ey, const REAL *ez,
                     REAL *hx, REAL *hy, REAL *hz,
                     const REAL *chx, const REAL *chy, const REAL *chz,
                     REAL *const *psi)
{
    GRID;
    for (int ax = 0; ax < 3; ax++) {
        const int64_t P = npml[ax];
        if (P <= 0) continue;
        const int64_t n_ax = ax == 0 ? nx : (ax == 1 ? ny : nz);
        const int64_t st_ax = ax == 0 ? sx : (ax == 1 ? sy : 1);
        REAL *p1 = psi[2 * ax], *p2 = psi[2 * ax + 1];
#pragma omp parallel for collapse(2) schedule(static)
        for (int64_t i = 0; i < nx; i++)
            for (int64_t j = 0; j < ny; j++)
                for (int64_t k = 0; k < nz; k++) {
                    const int64_t idx = ax == 0 ? i : (ax == 1 ? j : k);
                    int64_t s;
                    if ((faces >> (2 * ax)) & 1 && idx >= 1 && idx <= P) s = idx - 1;
                    else if ((faces >> (2 * ax + 1)) & 1 && idx >= n_ax - P && idx <= n_ax - 1)
                        s = P + idx - (n_ax - P);
                    else continue;
                    const int64_t c = i * sx + j * sy + k;
                    const int64_t q = ax == 0 ? (s * ny + j) * nz + k
                                    : ax == 1 ? (i * 2 * P + s) * nz + k
                                              : (i * ny + j) * 2 * P + s;
                    const REAL bb = b[ax][s], aa = a[ax][s], kk = km1[ax][s];
                    /* update ranges: hx j,k in [2,n-2]; hy i,k; hz i,j */
                    const int ok_i = i >= 2 && i <= nx - 2, ok_j = j >= 2 && j <= ny - 2,
                              ok_k = k >= 2 && k <= nz - 2;
                    REAL *f1, *f2;
                    const REAL *g1, *g2, *c1, *c2;
                    int ok1, ok2;
                    REAL s1, s2;
                    if (ax == 0) { f1 = hy; g1 = ez; c1 = chy; ok1 = ok_i && ok_k; s1 = +1;
                                   f2 = hz; g2 = ey; c2 = chz; ok2 = ok_i && ok_j; s2 = -1; }
                    else if (ax == 1) { f1 = hz; g1 = ex; c1 = chz; ok1 = ok_i && ok_j; s1 = +1;
                                        f2 = hx; g2 = ez; c2 = chx; ok2 = ok_j && ok_k; s2 = -1; }
                    else { f1 = hx; g1 = ey; c1 = chx; ok1 = ok_j && ok_k; s1 = +1;
                           f2 = hy; g2 = ex; c2 = chy; ok2 = ok_i && ok_k; s2 = -1; }
                    if (ok1) {
                        REAL d = d4h(g1, c, st_ax);
                        p1[q] = bb * p1[q] + aa * d;
                        REAL t = (cl * (c1 ? c1[c] : ch_scalar)) * (kk * d + p1[q]);
                        f1[c] = s1 > 0 ? f1[c] + t : f1[c] - t;
                    }
                    if (ok2) {
                        REAL d = d4h(g2, c, st_ax);
                        p2[q] = bb * p2[q] + aa * d;
                        REAL t = (cl * (c2 ? c2[c] : ch_scalar)) * (kk * d + p2[q]);
                        f2[c] = s2 > 0 ? f2[c] + t : f2[c] - t;
                    }
                }
    }
}

/* 4th-order H stage with a scalar ch (ch arrays NULL): same arithmetic as symp_h */
void FN(symp_h_scalar)(const int64_t *g, REAL cl, REAL ch, const REAL *ex, const REAL *ey, const REAL *ez,
                       REAL *hx, REAL *hy, REAL *hz)
{
    GRID;
    const REAL c27 = (REAL)27;
    const REAL cc = cl * ch;
#pragma omp parallel for collapse(2) schedule(static)
    for (int64_t i = 0; i < nx; i++)
        for (int64_t j = 0; j < ny; j++)
            for (int64_t k = 0; k < nz; k++) {
                const int64_t c = i * sx + j * sy + k;
                if (j > 1 && j < ny - 1 && k > 1 && k < nz - 1) {
                    REAL n = ((ez[c] - ez[c - sy]) - ey[c]) + ey[c - 1];
                    REAL f = ((ez[c + sy] - ez[c - 2 * sy]) - ey[c + 1]) + ey[c - 2];
                    hx[c] = hx[c] - cc * (c27 * n - f);
                }
                if (i > 1 && i < nx - 1 && k > 1 && k < nz - 1) {
                    REAL n = ((ex[c] - ex[c - 1]) - ez[c]) + ez[c - sx];
                    REAL f = ((ex[c + 1] - ex[c - 2]) - ez[c + sx]) + ez[c - 2 * sx];
                    hy[c] = hy[c] - cc * (c27 * n - f);
                }
                if (i > 1 && i < nx - 1 && j > 1 && j < ny - 1) {
                    REAL n = ((ey[c] - ey[c - sx]) - ex[c]) + ex[c - sy];
                    REAL f = ((ey[c + sx] - ey[c - 2 * sx]) - ex[c + sy]) + ex[c - 2 * sy];
                    hz[c] = hz[c] - cc * (c27 * n - f);
                }
            }
}

/* ------------------------------------------------------------------------ */
/* Drude ADE, kuFDTD/v0.2.0/dim3/cpu/core/drude_ade.c:48-93: on the sub-box   */
/* of ni x nj x nk cells starting at (i0, j0, k0) of the E arrays; J, cja,   */
/* cjb are dense (ni, nj, nk) arrays.  Per cell and component:               */
/*   e' = e - ce*J;  e = e';  J = cja*J + cjb*e'                              */
/* ------------------------------------------------------------------------ */
void FN(drude_e)(const int64_t *g, const int64_t *box, REAL *ex, REAL *ey, REAL *ez,
                 const REAL *cex, const REAL *cey, const REAL *cez,
                 REAL *jx, REAL *jy, REAL *jz, const REAL *cjax, const REAL *cjay, const REAL *cjaz,
                 const REAL *cjbx, const REAL *cjby, const REAL *cjbz)
{
    GRID;
    const int64_t i0 = box[0], j0 = box[1], k0 = box[2], ni = box[3], nj = box[4], nk = box[5];
    REAL *E[3] = {ex, ey, ez}, *J[3] = {jx, jy, jz};
    const REAL *CE[3] = {cex, cey, cez}, *CA[3] = {cjax, cjay, cjaz}, *CB[3] = {cjbx, cjby, cjbz};
#pragma omp parallel for collapse(2) schedule(static)
    for (int64_t i = 0; i < ni; i++)
        for (int64_t j = 0; j < nj; j++)
            for (int64_t k = 0; k < nk; k++) {
                const int64_t ji = (i * nj + j) * nk + k;
                const int64_t ei = (i0 + i) * sx + (j0 + j) * sy + (k0 + k);
                for (int q = 0; q < 3; q++) {
                    const REAL f = J[q][ji];
                    const REAL t = CE[q][ei] * f;
                    const REAL e = E[q][ei] - t;
                    E[q][ei] = e;
                    const REAL a = CA[q][ji] * f;
                    const REAL b = CB[q][ji] * e;
                    J[q][ji] = a + b;
                }
            }
}
