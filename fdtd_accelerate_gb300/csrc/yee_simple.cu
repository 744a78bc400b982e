// In-place, reference-shaped kernels: one thread per cell, z-coalesced.
//
// Semantics (index ranges, operation grouping) follow
//   2nd_order-Yee/Numpy/fdtd3d.py:4-37                   (E, H, periodic planes)
//   kuFDTD/v0.2.0/dim3/cpu/core/cpml_non_kappa.c:14-429  (psi recursion, slab ranges)
//   kuFDTD/before_CUDA/v0.3.0/boundary/core/cpml_core.c:238-263 (kappa term)
// Arithmetic uses explicit round-to-nearest intrinsics so results equal the
// FP32 NumPy/C evaluation bit for bit.
#include "common.cuh"

namespace fdtd {

constexpr int kBlockZ = 128;

__global__ void __launch_bounds__(kBlockZ)
k_update_e(Grid g, float *__restrict__ ex, float *__restrict__ ey, float *__restrict__ ez,
           const float *__restrict__ hx, const float *__restrict__ hy, const float *__restrict__ hz,
           const float *__restrict__ cex, const float *__restrict__ cey, const float *__restrict__ cez) {
    const int64_t k = (int64_t)blockIdx.x * kBlockZ + threadIdx.x;
    const int64_t j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    const int64_t c = i * g.sx + j * g.sy + k;
    if (j < g.ny - 1 && k < g.nz - 1)
        ex[c] = fadd(ex[c], fmul(cex[c], curl4(hz[c + g.sy], hz[c], hy[c + 1], hy[c])));
    if (i < g.nx - 1 && k < g.nz - 1)
        ey[c] = fadd(ey[c], fmul(cey[c], curl4(hx[c + 1], hx[c], hz[c + g.sx], hz[c])));
    if (i < g.nx - 1 && j < g.ny - 1)
        ez[c] = fadd(ez[c], fmul(cez[c], curl4(hy[c + g.sx], hy[c], hx[c + g.sy], hx[c])));
}

__global__ void __launch_bounds__(kBlockZ)
k_update_h(Grid g, const float *__restrict__ ex, const float *__restrict__ ey, const float *__restrict__ ez,
           float *__restrict__ hx, float *__restrict__ hy, float *__restrict__ hz,
           const float *__restrict__ chx, const float *__restrict__ chy, const float *__restrict__ chz) {
    const int64_t k = (int64_t)blockIdx.x * kBlockZ + threadIdx.x;
    const int64_t j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    const int64_t c = i * g.sx + j * g.sy + k;
    if (j > 0 && k > 0)
        hx[c] = fsub(hx[c], fmul(chx ? chx[c] : 0.5f, curl4(ez[c], ez[c - g.sy], ey[c], ey[c - 1])));
    if (i > 0 && k > 0)
        hy[c] = fsub(hy[c], fmul(chy ? chy[c] : 0.5f, curl4(ex[c], ex[c - 1], ez[c], ez[c - g.sx])));
    if (i > 0 && j > 0)
        hz[c] = fsub(hz[c], fmul(chz ? chz[c] : 0.5f, curl4(ey[c], ey[c - g.sx], ex[c], ex[c - g.sy])));
}

// Periodic planes, fdtd3d.py:16-37.  grid: (ceil(m/128), n_other, 1)
__global__ void k_pbc_plane(Grid g, int axis, int e_or_h, float *f1, float *f2) {
    const int64_t a = (int64_t)blockIdx.x * kBlockZ + threadIdx.x;
    const int64_t b = blockIdx.y;
    int64_t lo, hi;  // offsets of the first and last plane cell
    if (axis == 0) {  // plane (j=b, k=a)
        if (a >= g.nz || b >= g.ny) return;
        lo = b * g.sy + a;
        hi = lo + (g.nx - 1) * g.sx;
    } else if (axis == 1) {  // plane (i=b, k=a)
        if (a >= g.nz || b >= g.nx) return;
        lo = b * g.sx + a;
        hi = lo + (g.ny - 1) * g.sy;
    } else {  // plane (i=b, j=a)
        if (a >= g.ny || b >= g.nx) return;
        lo = b * g.sx + a * g.sy;
        hi = lo + g.nz - 1;
    }
    if (e_or_h == 0) {  // E: last plane <- first plane
        f1[hi] = f1[lo];
        f2[hi] = f2[lo];
    } else {            // H: first plane <- last plane
        f1[lo] = f1[hi];
        f2[lo] = f2[hi];
    }
}

struct CpmlAxis {
    int64_t P;
    int front, back;
    const float *b, *a, *km1;
    float *psi1, *psi2;
};

__device__ __forceinline__ float cpml_term(float &psi, float b, float a, float km1, float d) {
    psi = fadd(fmul(b, psi), fmul(a, d));
    return fadd(fmul(km1, d), psi);
}

// E, x axis: ey -= cey*(...dHz/dx...), ez += cez*(...dHy/dx...)
__global__ void k_cpml_e_x(Grid g, CpmlAxis A, float *ey, float *ez, const float *hy, const float *hz,
                           const float *cey, const float *cez) {
    const int64_t k = (int64_t)blockIdx.x * kBlockZ + threadIdx.x;
    const int64_t j = blockIdx.y, s = blockIdx.z;
    if (k >= g.nz) return;
    if (!(s < A.P ? A.front : A.back)) return;
    const int64_t i = slab_node_e(s, A.P, g.nx);
    const int64_t c = i * g.sx + j * g.sy + k, p = (s * g.ny + j) * g.nz + k;
    const float b = A.b[s], a = A.a[s], km1 = A.km1[s];
    if (k < g.nz - 1) {
        float psi = A.psi1[p];
        float t = cpml_term(psi, b, a, km1, fsub(hz[c + g.sx], hz[c]));
        A.psi1[p] = psi;
        ey[c] = fsub(ey[c], fmul(cey[c], t));
    }
    if (j < g.ny - 1) {
        float psi = A.psi2[p];
        float t = cpml_term(psi, b, a, km1, fsub(hy[c + g.sx], hy[c]));
        A.psi2[p] = psi;
        ez[c] = fadd(ez[c], fmul(cez[c], t));
    }
}

// E, y axis: ez -= cez*(...dHx/dy...), ex += cex*(...dHz/dy...)
__global__ void k_cpml_e_y(Grid g, CpmlAxis A, float *ez, float *ex, const float *hx, const float *hz,
                           const float *cez, const float *cex) {
    const int64_t k = (int64_t)blockIdx.x * kBlockZ + threadIdx.x;
    const int64_t s = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    if (!(s < A.P ? A.front : A.back)) return;
    const int64_t j = slab_node_e(s, A.P, g.ny);
    const int64_t c = i * g.sx + j * g.sy + k, p = (i * 2 * A.P + s) * g.nz + k;
    const float b = A.b[s], a = A.a[s], km1 = A.km1[s];
    if (i < g.nx - 1) {
        float psi = A.psi1[p];
        float t = cpml_term(psi, b, a, km1, fsub(hx[c + g.sy], hx[c]));
        A.psi1[p] = psi;
        ez[c] = fsub(ez[c], fmul(cez[c], t));
    }
    if (k < g.nz - 1) {
        float psi = A.psi2[p];
        float t = cpml_term(psi, b, a, km1, fsub(hz[c + g.sy], hz[c]));
        A.psi2[p] = psi;
        ex[c] = fadd(ex[c], fmul(cex[c], t));
    }
}

// E, z axis: ex -= cex*(...dHy/dz...), ey += cey*(...dHx/dz...)
__global__ void k_cpml_e_z(Grid g, CpmlAxis A, float *ex, float *ey, const float *hx, const float *hy,
                           const float *cex, const float *cey) {
    const int64_t t = (int64_t)blockIdx.x * kBlockZ + threadIdx.x;
    const int64_t twoP = 2 * A.P;
    if (t >= g.nx * g.ny * twoP) return;
    const int64_t s = t % twoP, j = (t / twoP) % g.ny, i = t / (twoP * g.ny);
    if (!(s < A.P ? A.front : A.back)) return;
    const int64_t k = slab_node_e(s, A.P, g.nz);
    const int64_t c = i * g.sx + j * g.sy + k, p = t;
    const float b = A.b[s], a = A.a[s], km1 = A.km1[s];
    if (j < g.ny - 1) {
        float psi = A.psi1[p];
        float tt = cpml_term(psi, b, a, km1, fsub(hy[c + 1], hy[c]));
        A.psi1[p] = psi;
        ex[c] = fsub(ex[c], fmul(cex[c], tt));
    }
    if (i < g.nx - 1) {
        float psi = A.psi2[p];
        float tt = cpml_term(psi, b, a, km1, fsub(hx[c + 1], hx[c]));
        A.psi2[p] = psi;
        ey[c] = fadd(ey[c], fmul(cey[c], tt));
    }
}

// H, x axis: hy += ch*(...dEz/dx...), hz -= ch*(...dEy/dx...)
__global__ void k_cpml_h_x(Grid g, CpmlAxis A, float *hy, float *hz, const float *ey, const float *ez,
                           const float *chy, const float *chz) {
    const int64_t k = (int64_t)blockIdx.x * kBlockZ + threadIdx.x;
    const int64_t j = blockIdx.y, s = blockIdx.z;
    if (k >= g.nz) return;
    if (!(s < A.P ? A.front : A.back)) return;
    const int64_t i = slab_node_h(s, A.P, g.nx);
    const int64_t c = i * g.sx + j * g.sy + k, p = (s * g.ny + j) * g.nz + k;
    const float b = A.b[s], a = A.a[s], km1 = A.km1[s];
    if (k > 0) {
        float psi = A.psi1[p];
        float t = cpml_term(psi, b, a, km1, fsub(ez[c], ez[c - g.sx]));
        A.psi1[p] = psi;
        hy[c] = fadd(hy[c], fmul(chy ? chy[c] : 0.5f, t));
    }
    if (j > 0) {
        float psi = A.psi2[p];
        float t = cpml_term(psi, b, a, km1, fsub(ey[c], ey[c - g.sx]));
        A.psi2[p] = psi;
        hz[c] = fsub(hz[c], fmul(chz ? chz[c] : 0.5f, t));
    }
}

// H, y axis: hz += ch*(...dEx/dy...), hx -= ch*(...dEz/dy...)
__global__ void k_cpml_h_y(Grid g, CpmlAxis A, float *hz, float *hx, const float *ex, const float *ez,
                           const float *chz, const float *chx) {
    const int64_t k = (int64_t)blockIdx.x * kBlockZ + threadIdx.x;
    const int64_t s = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    if (!(s < A.P ? A.front : A.back)) return;
    const int64_t j = slab_node_h(s, A.P, g.ny);
    const int64_t c = i * g.sx + j * g.sy + k, p = (i * 2 * A.P + s) * g.nz + k;
    const float b = A.b[s], a = A.a[s], km1 = A.km1[s];
    if (i > 0) {
        float psi = A.psi1[p];
        float t = cpml_term(psi, b, a, km1, fsub(ex[c], ex[c - g.sy]));
        A.psi1[p] = psi;
        hz[c] = fadd(hz[c], fmul(chz ? chz[c] : 0.5f, t));
    }
    if (k > 0) {
        float psi = A.psi2[p];
        float t = cpml_term(psi, b, a, km1, fsub(ez[c], ez[c - g.sy]));
        A.psi2[p] = psi;
        hx[c] = fsub(hx[c], fmul(chx ? chx[c] : 0.5f, t));
    }
}

// H, z axis: hx += ch*(...dEy/dz...), hy -= ch*(...dEx/dz...)
__global__ void k_cpml_h_z(Grid g, CpmlAxis A, float *hx, float *hy, const float *ex, const float *ey,
                           const float *chx, const float *chy) {
    const int64_t t = (int64_t)blockIdx.x * kBlockZ + threadIdx.x;
    const int64_t twoP = 2 * A.P;
    if (t >= g.nx * g.ny * twoP) return;
    const int64_t s = t % twoP, j = (t / twoP) % g.ny, i = t / (twoP * g.ny);
    if (!(s < A.P ? A.front : A.back)) return;
    const int64_t k = slab_node_h(s, A.P, g.nz);
    const int64_t c = i * g.sx + j * g.sy + k, p = t;
    const float b = A.b[s], a = A.a[s], km1 = A.km1[s];
    if (j > 0) {
        float psi = A.psi1[p];
        float tt = cpml_term(psi, b, a, km1, fsub(ey[c], ey[c - 1]));
        A.psi1[p] = psi;
        hx[c] = fadd(hx[c], fmul(chx ? chx[c] : 0.5f, tt));
    }
    if (i > 0) {
        float psi = A.psi2[p];
        float tt = cpml_term(psi, b, a, km1, fsub(ex[c], ex[c - 1]));
        A.psi2[p] = psi;
        hy[c] = fsub(hy[c], fmul(chy ? chy[c] : 0.5f, tt));
    }
}

// Soft sources, sequential in list order (duplicates accumulate in order).
// Drude ADE on the box of d, one thread per box cell (z fastest).
__global__ void __launch_bounds__(kBlockZ)
k_drude_e(Grid g, fdtd_drude d, float *ex, float *ey, float *ez, const float *cex, const float *cey,
          const float *cez) {
    const int64_t t = (int64_t)blockIdx.x * kBlockZ + threadIdx.x;
    if (t >= d.ni * d.nj * d.nk) return;
    const int64_t k = t % d.nk, j = (t / d.nk) % d.nj, i = t / (d.nk * d.nj);
    const int64_t c = (d.i0 + i) * g.sx + (d.j0 + j) * g.sy + d.k0 + k;
    float *E[3] = {ex, ey, ez};
    const float *CE[3] = {cex, cey, cez};
#pragma unroll
    for (int q = 0; q < 3; q++) {
        float jn;
        E[q][c] = drude_cell(E[q][c], CE[q][c], d.j[q][t], d.cja[q][t], d.cjb[q][t], jn);
        d.j[q][t] = jn;
    }
}

__global__ void k_sources(Grid g, fdtd_sources src, int64_t t, float *ex, float *ey, float *ez) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (t < 0 || t >= src.namp) return;
    for (int s = 0; s < src.nsrc; s++) {
        const int64_t si = src.ijk[3 * s], sj = src.ijk[3 * s + 1], sk = src.ijk[3 * s + 2];
        if (si < 0 || si >= g.nx || sj < 0 || sj >= g.ny || sk < 0 || sk >= g.nz) continue;
        const int64_t c = si * g.sx + sj * g.sy + sk;
        float *f = src.comp[s] == 0 ? ex : (src.comp[s] == 1 ? ey : ez);
        f[c] = fadd(f[c], src.amp[(int64_t)s * src.namp + t]);
    }
}

static dim3 cell_grid(const Grid &g) {
    return dim3((unsigned)((g.nz + kBlockZ - 1) / kBlockZ), (unsigned)g.ny, (unsigned)g.nx);
}

static int validate_cpml(const Grid &g, const fdtd_cpml *c, const fdtd_psi *psi, bool e) {
    if (!c || !psi) return FDTD_ERR_ARG;
    const int64_t n[3] = {g.nx, g.ny, g.nz};
    for (int a = 0; a < 3; a++) {
        const int64_t P = c->npml[a];
        if (P < 0) return FDTD_ERR_ARG;
        if (P == 0) continue;
        if (n[a] < 2 * P + 2) return FDTD_ERR_SHAPE;
        if (a < 2 && 2 * P > 65535) return FDTD_ERR_SHAPE;
        const float *const *tb = e ? c->b_e : c->b_h;
        const float *const *ta = e ? c->a_e : c->a_h;
        const float *const *tk = e ? c->km1_e : c->km1_h;
        float *const *ps = e ? psi->e : psi->h;
        if (!all_nonnull(tb[a], ta[a], tk[a], ps[2 * a], ps[2 * a + 1])) return FDTD_ERR_ARG;
    }
    return FDTD_OK;
}

static CpmlAxis make_axis(const fdtd_cpml *c, const fdtd_psi *psi, int a, bool e) {
    CpmlAxis A;
    A.P = c->npml[a];
    A.front = (c->faces >> (2 * a)) & 1;
    A.back = (c->faces >> (2 * a + 1)) & 1;
    A.b = e ? c->b_e[a] : c->b_h[a];
    A.a = e ? c->a_e[a] : c->a_h[a];
    A.km1 = e ? c->km1_e[a] : c->km1_h[a];
    A.psi1 = e ? psi->e[2 * a] : psi->h[2 * a];
    A.psi2 = e ? psi->e[2 * a + 1] : psi->h[2 * a + 1];
    return A;
}

static int launch_cpml_e(const Grid &g, const fdtd_cpml *c, const fdtd_psi *psi, float *ex, float *ey,
                         float *ez, const float *hx, const float *hy, const float *hz, const float *cex,
                         const float *cey, const float *cez, cudaStream_t st) {
    if (c->npml[0] > 0) {
        CpmlAxis A = make_axis(c, psi, 0, true);
        dim3 grid((unsigned)((g.nz + kBlockZ - 1) / kBlockZ), (unsigned)g.ny, (unsigned)(2 * A.P));
        k_cpml_e_x<<<grid, kBlockZ, 0, st>>>(g, A, ey, ez, hy, hz, cey, cez);
    }
    if (c->npml[1] > 0) {
        CpmlAxis A = make_axis(c, psi, 1, true);
        dim3 grid((unsigned)((g.nz + kBlockZ - 1) / kBlockZ), (unsigned)(2 * A.P), (unsigned)g.nx);
        k_cpml_e_y<<<grid, kBlockZ, 0, st>>>(g, A, ez, ex, hx, hz, cez, cex);
    }
    if (c->npml[2] > 0) {
        CpmlAxis A = make_axis(c, psi, 2, true);
        const int64_t n = g.nx * g.ny * 2 * A.P;
        k_cpml_e_z<<<(unsigned)((n + kBlockZ - 1) / kBlockZ), kBlockZ, 0, st>>>(g, A, ex, ey, hx, hy, cex, cey);
    }
    return check_launch();
}

static int launch_cpml_h(const Grid &g, const fdtd_cpml *c, const fdtd_psi *psi, const float *ex,
                         const float *ey, const float *ez, float *hx, float *hy, float *hz, const float *chx,
                         const float *chy, const float *chz, cudaStream_t st) {
    if (c->npml[0] > 0) {
        CpmlAxis A = make_axis(c, psi, 0, false);
        dim3 grid((unsigned)((g.nz + kBlockZ - 1) / kBlockZ), (unsigned)g.ny, (unsigned)(2 * A.P));
        k_cpml_h_x<<<grid, kBlockZ, 0, st>>>(g, A, hy, hz, ey, ez, chy, chz);
    }
    if (c->npml[1] > 0) {
        CpmlAxis A = make_axis(c, psi, 1, false);
        dim3 grid((unsigned)((g.nz + kBlockZ - 1) / kBlockZ), (unsigned)(2 * A.P), (unsigned)g.nx);
        k_cpml_h_y<<<grid, kBlockZ, 0, st>>>(g, A, hz, hx, ex, ez, chz, chx);
    }
    if (c->npml[2] > 0) {
        CpmlAxis A = make_axis(c, psi, 2, false);
        const int64_t n = g.nx * g.ny * 2 * A.P;
        k_cpml_h_z<<<(unsigned)((n + kBlockZ - 1) / kBlockZ), kBlockZ, 0, st>>>(g, A, hx, hy, ex, ey, chx, chy);
    }
    return check_launch();
}

static int validate_sources(const Grid &g, const fdtd_sources *s) {
    if (!s) return FDTD_ERR_ARG;
    if (s->nsrc < 0 || s->namp < 0) return FDTD_ERR_ARG;
    if (s->nsrc > 0 && !all_nonnull(s->ijk, s->comp, s->amp)) return FDTD_ERR_ARG;
    return FDTD_OK;
}

}  // namespace fdtd

using namespace fdtd;

extern "C" {

int fdtd_update_e_f32(const fdtd_grid *gp, float *ex, float *ey, float *ez, const float *hx, const float *hy,
                      const float *hz, const float *cex, const float *cey, const float *cez, void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!all_nonnull(ex, ey, ez, hx, hy, hz, cex, cey, cez)) return FDTD_ERR_ARG;
    k_update_e<<<cell_grid(g), kBlockZ, 0, as_stream(stream)>>>(g, ex, ey, ez, hx, hy, hz, cex, cey, cez);
    return check_launch();
}

int fdtd_update_h_f32(const fdtd_grid *gp, const float *ex, const float *ey, const float *ez, float *hx,
                      float *hy, float *hz, const float *chx, const float *chy, const float *chz, void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!all_nonnull(ex, ey, ez, hx, hy, hz)) return FDTD_ERR_ARG;
    k_update_h<<<cell_grid(g), kBlockZ, 0, as_stream(stream)>>>(g, ex, ey, ez, hx, hy, hz, chx, chy, chz);
    return check_launch();
}

static int pbc_common(const fdtd_grid *gp, int32_t axes, float *f0, float *f1, float *f2, int e_or_h,
                      void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!all_nonnull(f0, f1, f2)) return FDTD_ERR_ARG;
    if (axes & ~7) return FDTD_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    // E: x -> (ey, ez), y -> (ez, ex), z -> (ex, ey); H likewise with h.
    if (axes & 1)
        k_pbc_plane<<<dim3((unsigned)((g.nz + kBlockZ - 1) / kBlockZ), (unsigned)g.ny), kBlockZ, 0, st>>>(
            g, 0, e_or_h, f1, f2);
    if (axes & 2)
        k_pbc_plane<<<dim3((unsigned)((g.nz + kBlockZ - 1) / kBlockZ), (unsigned)g.nx), kBlockZ, 0, st>>>(
            g, 1, e_or_h, f2, f0);
    if (axes & 4)
        k_pbc_plane<<<dim3((unsigned)((g.ny + kBlockZ - 1) / kBlockZ), (unsigned)g.nx), kBlockZ, 0, st>>>(
            g, 2, e_or_h, f0, f1);
    return check_launch();
}

int fdtd_update_pbc_e_f32(const fdtd_grid *g, int32_t axes, float *ex, float *ey, float *ez, void *stream) {
    return pbc_common(g, axes, ex, ey, ez, 0, stream);
}

int fdtd_update_pbc_h_f32(const fdtd_grid *g, int32_t axes, float *hx, float *hy, float *hz, void *stream) {
    return pbc_common(g, axes, hx, hy, hz, 1, stream);
}

int fdtd_cpml_e_f32(const fdtd_grid *gp, const fdtd_cpml *c, float *ex, float *ey, float *ez, const float *hx,
                    const float *hy, const float *hz, const float *cex, const float *cey, const float *cez,
                    const fdtd_psi *psi, void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!all_nonnull(ex, ey, ez, hx, hy, hz, cex, cey, cez)) return FDTD_ERR_ARG;
    FDTD_TRY(validate_cpml(g, c, psi, true));
    return launch_cpml_e(g, c, psi, ex, ey, ez, hx, hy, hz, cex, cey, cez, as_stream(stream));
}

int fdtd_cpml_h_f32(const fdtd_grid *gp, const fdtd_cpml *c, const float *ex, const float *ey, const float *ez,
                    float *hx, float *hy, float *hz, const float *chx, const float *chy, const float *chz,
                    const fdtd_psi *psi, void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!all_nonnull(ex, ey, ez, hx, hy, hz)) return FDTD_ERR_ARG;
    FDTD_TRY(validate_cpml(g, c, psi, false));
    return launch_cpml_h(g, c, psi, ex, ey, ez, hx, hy, hz, chx, chy, chz, as_stream(stream));
}

int fdtd_add_sources_f32(const fdtd_grid *gp, const fdtd_sources *src, int64_t t, float *ex, float *ey,
                         float *ez, void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!all_nonnull(ex, ey, ez)) return FDTD_ERR_ARG;
    FDTD_TRY(validate_sources(g, src));
    if (src->nsrc == 0) return FDTD_OK;
    k_sources<<<1, 32, 0, as_stream(stream)>>>(g, *src, t, ex, ey, ez);
    return check_launch();
}

int fdtd_drude_update_e_f32(const fdtd_grid *gp, const fdtd_drude *d, float *ex, float *ey, float *ez,
                            const float *cex, const float *cey, const float *cez, void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!all_nonnull(ex, ey, ez, cex, cey, cez)) return FDTD_ERR_ARG;
    FDTD_TRY(validate_drude(g, d));
    const int64_t n = d->ni * d->nj * d->nk;
    k_drude_e<<<(unsigned)((n + kBlockZ - 1) / kBlockZ), kBlockZ, 0, as_stream(stream)>>>(g, *d, ex, ey, ez, cex,
                                                                                         cey, cez);
    return check_launch();
}

int fdtd_step_unfused_f32(const fdtd_grid *gp, float *const f[6], const float *const ce[3],
                          const float *const ch[3], const fdtd_cpml *c, const fdtd_psi *psi,
                          const fdtd_sources *src, int64_t t, void *stream) {
    NvtxRange nvtx_range("fdtd_step_unfused");
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!f || !ce) return FDTD_ERR_ARG;
    if (!all_nonnull(f[0], f[1], f[2], f[3], f[4], f[5], ce[0], ce[1], ce[2])) return FDTD_ERR_ARG;
    const float *chx = ch ? ch[0] : nullptr, *chy = ch ? ch[1] : nullptr, *chz = ch ? ch[2] : nullptr;
    const bool pml = c && (c->npml[0] > 0 || c->npml[1] > 0 || c->npml[2] > 0);
    if (pml) {
        FDTD_TRY(validate_cpml(g, c, psi, true));
        FDTD_TRY(validate_cpml(g, c, psi, false));
    }
    if (src) FDTD_TRY(validate_sources(g, src));
    cudaStream_t st = as_stream(stream);
    k_update_e<<<cell_grid(g), kBlockZ, 0, st>>>(g, f[0], f[1], f[2], f[3], f[4], f[5], ce[0], ce[1], ce[2]);
    FDTD_TRY(check_launch());
    if (pml) FDTD_TRY(launch_cpml_e(g, c, psi, f[0], f[1], f[2], f[3], f[4], f[5], ce[0], ce[1], ce[2], st));
    if (src && src->nsrc > 0) {
        k_sources<<<1, 32, 0, st>>>(g, *src, t, f[0], f[1], f[2]);
        FDTD_TRY(check_launch());
    }
    k_update_h<<<cell_grid(g), kBlockZ, 0, st>>>(g, f[0], f[1], f[2], f[3], f[4], f[5], chx, chy, chz);
    FDTD_TRY(check_launch());
    if (pml) FDTD_TRY(launch_cpml_h(g, c, psi, f[0], f[1], f[2], f[3], f[4], f[5], chx, chy, chz, st));
    return FDTD_OK;
}

}  // extern "C"
