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

// H stage with a uniform ch (the 4th-order workload's ch = S/24): same
// arithmetic as k_symp_h with (cl * ch) formed once.
__global__ void __launch_bounds__(kSympBlock)
k_symp_h_scalar(Grid g, float clch, const float *__restrict__ ex, const float *__restrict__ ey,
                const float *__restrict__ ez, float *__restrict__ hx, float *__restrict__ hy, float *__restrict__ hz) {
    const int64_t k = (int64_t)blockIdx.x * kSympBlock + threadIdx.x;
    const int64_t j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    const int64_t c = i * g.sx + j * g.sy + k, X = g.sx, Y = g.sy;
    const bool jin = j > 1 && j < g.ny - 1, kin = k > 1 && k < g.nz - 1, iin = i > 1 && i < g.nx - 1;
    if (jin && kin) {
        float n = curl4(ez[c], ez[c - Y], ey[c], ey[c - 1]);
        float f = curl4(ez[c + Y], ez[c - 2 * Y], ey[c + 1], ey[c - 2]);
        hx[c] = fsub(hx[c], fmul(clch, fsub(fmul(27.0f, n), f)));
    }
    if (iin && kin) {
        float n = curl4(ex[c], ex[c - 1], ez[c], ez[c - X]);
        float f = curl4(ex[c + 1], ex[c - 2], ez[c + X], ez[c - 2 * X]);
        hy[c] = fsub(hy[c], fmul(clch, fsub(fmul(27.0f, n), f)));
    }
    if (iin && jin) {
        float n = curl4(ey[c], ey[c - X], ex[c], ex[c - Y]);
        float f = curl4(ey[c + X], ey[c - 2 * X], ex[c + Y], ex[c - 2 * Y]);
        hz[c] = fsub(hz[c], fmul(clch, fsub(fmul(27.0f, n), f)));
    }
}

// 4th-order CPML (no reference counterpart: the reference's 4th-order code
// has no absorbing boundary).  Same slab geometry as the 2nd-order CPML; the
// derivative along the slab axis is the stage stencil's
//   E nodes: d = 27*(F[i+1]-F[i]) - (F[i+2]-F[i-1])
//   H nodes: d = 27*(F[i]-F[i-1]) - (F[i+1]-F[i-2])
// psi = b*psi + a*d with the stage's b, a; F -/+= (coef*c)*(km1*d + psi)
// only where the stage updates F.
struct SympCpmlArgs {
    int64_t P;
    int front, back;
    const float *b, *a, *km1;
    float *psi1, *psi2;
    float *f1, *f2;         // updated components
    const float *g1, *g2;   // differentiated components
    const float *c1, *c2;   // coefficient arrays (NULL -> scalar)
    float coef, cscalar;    // stage coefficient, uniform coefficient
};

template <int AX, bool E>
__global__ void k_symp_cpml(Grid g, SympCpmlArgs A) {
    int64_t i, j, k, s;
    const int64_t twoP = 2 * A.P;
    if (AX == 0) {
        k = (int64_t)blockIdx.x * kSympBlock + threadIdx.x;
        j = blockIdx.y;
        s = blockIdx.z;
        if (k >= g.nz) return;
    } else if (AX == 1) {
        k = (int64_t)blockIdx.x * kSympBlock + threadIdx.x;
        s = blockIdx.y;
        i = blockIdx.z;
        if (k >= g.nz) return;
    } else {
        const int64_t t = (int64_t)blockIdx.x * kSympBlock + threadIdx.x;
        if (t >= g.nx * g.ny * twoP) return;
        s = t % twoP;
        j = (t / twoP) % g.ny;
        i = t / (twoP * g.ny);
    }
    if (!(s < A.P ? A.front : A.back)) return;
    const int64_t n_ax = AX == 0 ? g.nx : (AX == 1 ? g.ny : g.nz);
    const int64_t node = E ? slab_node_e(s, A.P, n_ax) : slab_node_h(s, A.P, n_ax);
    if (AX == 0) i = node;
    else if (AX == 1) j = node;
    else k = node;
    const int64_t st = AX == 0 ? g.sx : (AX == 1 ? g.sy : 1);
    const int64_t c = i * g.sx + j * g.sy + k;
    const int64_t q = AX == 0 ? (s * g.ny + j) * g.nz + k : (AX == 1 ? (i * twoP + s) * g.nz + k : (i * g.ny + j) * twoP + s);
    // update ranges of the stage: E in [1, n-3], H in [2, n-2] along the two
    // axes the component differentiates
    auto in_e = [&](int64_t x, int64_t n) { return x >= 1 && x <= n - 3; };
    auto in_h = [&](int64_t x, int64_t n) { return x >= 2 && x <= n - 2; };
    bool ok_i, ok_j, ok_k;
    if (E) { ok_i = in_e(i, g.nx); ok_j = in_e(j, g.ny); ok_k = in_e(k, g.nz); }
    else { ok_i = in_h(i, g.nx); ok_j = in_h(j, g.ny); ok_k = in_h(k, g.nz); }
    // component 1 (sign -1 for E, +1 for H) and component 2 (opposite sign)
    bool ok1, ok2;
    if (AX == 0) { ok1 = ok_i && ok_k; ok2 = ok_i && ok_j; }
    else if (AX == 1) { ok1 = ok_i && ok_j; ok2 = ok_j && ok_k; }
    else { ok1 = ok_j && ok_k; ok2 = ok_i && ok_k; }
    const float b = A.b[s], a = A.a[s], km1 = A.km1[s];
    auto deriv = [&](const float *F) {
        return E ? fsub(fmul(27.0f, fsub(F[c + st], F[c])), fsub(F[c + 2 * st], F[c - st]))
                 : fsub(fmul(27.0f, fsub(F[c], F[c - st])), fsub(F[c + st], F[c - 2 * st]));
    };
    if (ok1) {
        const float d = deriv(A.g1);
        const float psi = fadd(fmul(b, A.psi1[q]), fmul(a, d));
        A.psi1[q] = psi;
        const float t = fmul(fmul(A.coef, A.c1 ? A.c1[c] : A.cscalar), fadd(fmul(km1, d), psi));
        A.f1[c] = E ? fsub(A.f1[c], t) : fadd(A.f1[c], t);
    }
    if (ok2) {
        const float d = deriv(A.g2);
        const float psi = fadd(fmul(b, A.psi2[q]), fmul(a, d));
        A.psi2[q] = psi;
        const float t = fmul(fmul(A.coef, A.c2 ? A.c2[c] : A.cscalar), fadd(fmul(km1, d), psi));
        A.f2[c] = E ? fadd(A.f2[c], t) : fsub(A.f2[c], t);
    }
}

template <bool E>
static int launch_symp_cpml(const Grid &g, const fdtd_cpml *cp, const fdtd_psi *psi, float coef, float cscalar,
                            float *const F[3], const float *const G[3], const float *const Cf[3], cudaStream_t st) {
    for (int ax = 0; ax < 3; ax++) {
        const int64_t P = cp->npml[ax];
        if (P <= 0) continue;
        const int64_t n_ax = ax == 0 ? g.nx : (ax == 1 ? g.ny : g.nz);
        if (n_ax < 2 * P + 2) return FDTD_ERR_SHAPE;
        SympCpmlArgs A;
        A.P = P;
        A.front = (cp->faces >> (2 * ax)) & 1;
        A.back = (cp->faces >> (2 * ax + 1)) & 1;
        A.b = E ? cp->b_e[ax] : cp->b_h[ax];
        A.a = E ? cp->a_e[ax] : cp->a_h[ax];
        A.km1 = E ? cp->km1_e[ax] : cp->km1_h[ax];
        A.psi1 = E ? psi->e[2 * ax] : psi->h[2 * ax];
        A.psi2 = E ? psi->e[2 * ax + 1] : psi->h[2 * ax + 1];
        if (!all_nonnull(A.b, A.a, A.km1, A.psi1, A.psi2)) return FDTD_ERR_ARG;
        // (updated, differentiated) pairs: E: x (ey,hz),(ez,hy); y (ez,hx),(ex,hz); z (ex,hy),(ey,hx)
        //                                  H: x (hy,ez),(hz,ey); y (hz,ex),(hx,ez); z (hx,ey),(hy,ex)
        static const int u1[3] = {1, 2, 0}, u2[3] = {2, 0, 1};
        static const int ge1[3] = {2, 0, 1}, ge2[3] = {1, 2, 0};
        A.f1 = F[u1[ax]];
        A.f2 = F[u2[ax]];
        A.g1 = G[ge1[ax]];
        A.g2 = G[ge2[ax]];
        A.c1 = Cf ? Cf[u1[ax]] : nullptr;
        A.c2 = Cf ? Cf[u2[ax]] : nullptr;
        A.coef = coef;
        A.cscalar = cscalar;
        if (ax == 0) {
            dim3 grid((unsigned)((g.nz + kSympBlock - 1) / kSympBlock), (unsigned)g.ny, (unsigned)(2 * P));
            k_symp_cpml<0, E><<<grid, kSympBlock, 0, st>>>(g, A);
        } else if (ax == 1) {
            dim3 grid((unsigned)((g.nz + kSympBlock - 1) / kSympBlock), (unsigned)(2 * P), (unsigned)g.nx);
            k_symp_cpml<1, E><<<grid, kSympBlock, 0, st>>>(g, A);
        } else {
            const int64_t n = g.nx * g.ny * 2 * P;
            k_symp_cpml<2, E><<<(unsigned)((n + kSympBlock - 1) / kSympBlock), kSympBlock, 0, st>>>(g, A);
        }
        FDTD_TRY(check_launch());
    }
    return FDTD_OK;
}

// ---------------------------------------------------------------------------
// One stage with its CPML corrections in one pass.  Each cell takes the stage
// update (the arithmetic of k_symp_h / k_symp_h_scalar / k_symp_e), then, on
// the slabs of the enabled faces, the corrections k_symp_cpml applies, in its
// launch order (x, then y, then z) and with its arithmetic.  The two orders
// agree because a stage reads only the other field: every correction of a
// cell depends on the differentiated field and the cell's own value.
// Per component, (axis: sign, differentiated field, psi):
//   E: ex  y: +hz exy, z: -hy exz    H: hx  y: -ez hxy, z: +ey hxz
//      ey  x: -hz eyx, z: +hx eyz       hy  x: +ez hyx, z: -ex hyz
//      ez  x: +hy ezx, y: -hx ezy       hz  x: -ey hzx, y: +ex hzy
// ---------------------------------------------------------------------------
struct SympStage {
    float coef;            // cl (H) or dl (E)
    float cscalar;         // uniform coefficient (H without ch arrays)
    float clch;            // cl * ch as one product (H, uniform ch)
    const float *c[3];     // coefficient arrays of the updated components (NULL: uniform)
    int32_t P[3];          // slab thickness per axis (0: none)
    int32_t front[3], back[3];
    const float *b[3], *a[3], *km1[3];
    float *psi[6];         // per axis a: psi[2a] (first pair), psi[2a+1] (second pair)
};

// Grid with 32-bit extents and strides: the stage kernel indexes fields of
// fewer than 2^31 elements (the host checks), so its offsets stay 32-bit
// (64-bit index arithmetic made up a large part of its instructions).
struct Grid32 {
    int32_t nx, ny, nz;
    uint32_t sx, sy;
};

// One thread per cell, 128-thread blocks along z.
template <bool E, bool CARR>
__global__ void __launch_bounds__(kSympBlock)
k_symp_stage(Grid32 g, SympStage A, float *__restrict__ ex, float *__restrict__ ey, float *__restrict__ ez,
             float *__restrict__ hx, float *__restrict__ hy, float *__restrict__ hz) {
    const int k = blockIdx.x * kSympBlock + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    const uint32_t c = (uint32_t)i * g.sx + (uint32_t)j * g.sy + k, X = g.sx, Y = g.sy;
    const int n3[3] = {g.nx, g.ny, g.nz}, x3[3] = {i, j, k};
    const uint32_t st3[3] = {X, Y, 1u};
    // slab index of this cell along each axis (E or H nodes of the stage), -1 outside
    int sl[3];
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
        const int P = A.P[ax], n = n3[ax], x = x3[ax];
        int s = -1;
        if (P > 0) {
            if (A.front[ax] && x >= 1 && x <= P) s = x - 1;
            const int b0 = E ? n - P - 1 : n - P, b1 = E ? n - 2 : n - 1;
            if (A.back[ax] && x >= b0 && x <= b1) s = P + x - b0;
        }
        sl[ax] = s;
    }
    // derivative along ax of F at this cell (E nodes: forward, H nodes: backward stencil)
    auto deriv = [&](const float *F, int ax) {
        const uint32_t st = st3[ax];
        return E ? fsub(fmul(27.0f, fsub(F[c + st], F[c])), fsub(F[c + 2 * st], F[c - st]))
                 : fsub(fmul(27.0f, fsub(F[c], F[c - st])), fsub(F[c + st], F[c - 2 * st]));
    };
    // psi update of pair w (0, 1) of axis ax; returns (coef * cv) * (km1 * d + psi)
    auto term = [&](int ax, int w, float d, float cv) {
        const int s = sl[ax];
        const uint32_t twoP = 2u * A.P[ax];
        const uint32_t q = ax == 0 ? ((uint32_t)s * g.ny + j) * g.nz + k
                                   : (ax == 1 ? ((uint32_t)i * twoP + s) * g.nz + k : ((uint32_t)i * g.ny + j) * twoP + s);
        float *ps = A.psi[2 * ax + w];
        const float psi = fadd(fmul(A.b[ax][s], ps[q]), fmul(A.a[ax][s], d));
        ps[q] = psi;
        return fmul(fmul(A.coef, cv), fadd(fmul(A.km1[ax][s], d), psi));
    };
    if (E) {
        const bool jin = j > 0 && j < g.ny - 2, kin = k > 0 && k < g.nz - 2, iin = i > 0 && i < g.nx - 2;
        if (jin && kin) {
            float n = curl4(hz[c + Y], hz[c], hy[c + 1], hy[c]);
            float f = curl4(hz[c + 2 * Y], hz[c - Y], hy[c + 2], hy[c - 1]);
            const float cv = A.c[0][c];
            float v = fadd(ex[c], fmul(fmul(A.coef, cv), fsub(fmul(27.0f, n), f)));
            if (sl[1] >= 0) v = fadd(v, term(1, 1, deriv(hz, 1), cv));
            if (sl[2] >= 0) v = fsub(v, term(2, 0, deriv(hy, 2), cv));
            ex[c] = v;
        }
        if (iin && kin) {
            float n = curl4(hx[c + 1], hx[c], hz[c + X], hz[c]);
            float f = curl4(hx[c + 2], hx[c - 1], hz[c + 2 * X], hz[c - X]);
            const float cv = A.c[1][c];
            float v = fadd(ey[c], fmul(fmul(A.coef, cv), fsub(fmul(27.0f, n), f)));
            if (sl[0] >= 0) v = fsub(v, term(0, 0, deriv(hz, 0), cv));
            if (sl[2] >= 0) v = fadd(v, term(2, 1, deriv(hx, 2), cv));
            ey[c] = v;
        }
        if (iin && jin) {
            float n = curl4(hy[c + X], hy[c], hx[c + Y], hx[c]);
            float f = curl4(hy[c + 2 * X], hy[c - X], hx[c + 2 * Y], hx[c - Y]);
            const float cv = A.c[2][c];
            float v = fadd(ez[c], fmul(fmul(A.coef, cv), fsub(fmul(27.0f, n), f)));
            if (sl[0] >= 0) v = fadd(v, term(0, 1, deriv(hy, 0), cv));
            if (sl[1] >= 0) v = fsub(v, term(1, 0, deriv(hx, 1), cv));
            ez[c] = v;
        }
    } else {
        const bool jin = j > 1 && j < g.ny - 1, kin = k > 1 && k < g.nz - 1, iin = i > 1 && i < g.nx - 1;
        // stage factor: (cl * ch[c]) per cell, or cl * ch formed once on the host
        auto stage = [&](float h, float cv, float d27) {
            return fsub(h, fmul(CARR ? fmul(A.coef, cv) : A.clch, d27));
        };
        if (jin && kin) {
            float n = curl4(ez[c], ez[c - Y], ey[c], ey[c - 1]);
            float f = curl4(ez[c + Y], ez[c - 2 * Y], ey[c + 1], ey[c - 2]);
            const float cv = CARR ? A.c[0][c] : A.cscalar;
            float v = stage(hx[c], cv, fsub(fmul(27.0f, n), f));
            if (sl[1] >= 0) v = fsub(v, term(1, 1, deriv(ez, 1), cv));
            if (sl[2] >= 0) v = fadd(v, term(2, 0, deriv(ey, 2), cv));
            hx[c] = v;
        }
        if (iin && kin) {
            float n = curl4(ex[c], ex[c - 1], ez[c], ez[c - X]);
            float f = curl4(ex[c + 1], ex[c - 2], ez[c + X], ez[c - 2 * X]);
            const float cv = CARR ? A.c[1][c] : A.cscalar;
            float v = stage(hy[c], cv, fsub(fmul(27.0f, n), f));
            if (sl[0] >= 0) v = fadd(v, term(0, 0, deriv(ez, 0), cv));
            if (sl[2] >= 0) v = fsub(v, term(2, 1, deriv(ex, 2), cv));
            hy[c] = v;
        }
        if (iin && jin) {
            float n = curl4(ey[c], ey[c - X], ex[c], ex[c - Y]);
            float f = curl4(ey[c + X], ey[c - 2 * X], ex[c + Y], ex[c - 2 * Y]);
            const float cv = CARR ? A.c[2][c] : A.cscalar;
            float v = stage(hz[c], cv, fsub(fmul(27.0f, n), f));
            if (sl[0] >= 0) v = fsub(v, term(0, 1, deriv(ey, 0), cv));
            if (sl[1] >= 0) v = fadd(v, term(1, 0, deriv(ex, 1), cv));
            hz[c] = v;
        }
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

int fdtd_symplectic_h_scalar_f32(const fdtd_grid *gp, float cl, float ch, const float *ex, const float *ey,
                                 const float *ez, float *hx, float *hy, float *hz, void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!all_nonnull(ex, ey, ez, hx, hy, hz)) return FDTD_ERR_ARG;
    dim3 grid((unsigned)((g.nz + kSympBlock - 1) / kSympBlock), (unsigned)g.ny, (unsigned)g.nx);
    const float clch = cl * ch;  // one IEEE single-precision product, as the reference's (cl*ch[c])
    k_symp_h_scalar<<<grid, kSympBlock, 0, as_stream(stream)>>>(g, clch, ex, ey, ez, hx, hy, hz);
    return check_launch();
}

int fdtd_symplectic_cpml_e_f32(const fdtd_grid *gp, const fdtd_cpml *c, float dl, float *ex, float *ey, float *ez,
                               const float *hx, const float *hy, const float *hz, const float *cex,
                               const float *cey, const float *cez, const fdtd_psi *psi, void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!c || !psi || !all_nonnull(ex, ey, ez, hx, hy, hz, cex, cey, cez)) return FDTD_ERR_ARG;
    float *const F[3] = {ex, ey, ez};
    const float *const G[3] = {hx, hy, hz};
    const float *const Cf[3] = {cex, cey, cez};
    return launch_symp_cpml<true>(g, c, psi, dl, 0.f, F, G, Cf, as_stream(stream));
}

int fdtd_symplectic_cpml_h_f32(const fdtd_grid *gp, const fdtd_cpml *c, float cl, float ch, const float *ex,
                               const float *ey, const float *ez, float *hx, float *hy, float *hz, const float *chx,
                               const float *chy, const float *chz, const fdtd_psi *psi, void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!c || !psi || !all_nonnull(ex, ey, ez, hx, hy, hz)) return FDTD_ERR_ARG;
    float *const F[3] = {hx, hy, hz};
    const float *const G[3] = {ex, ey, ez};
    const float *const Cf[3] = {chx, chy, chz};
    return launch_symp_cpml<false>(g, c, psi, cl, ch, F, G, chx ? Cf : nullptr, as_stream(stream));
}

int fdtd_symplectic_stage_f32(const fdtd_grid *gp, const fdtd_cpml *cp, int32_t e_or_h, float coef,
                              float ch_scalar, float *const f[6], const float *const cf[3], const fdtd_psi *psi,
                              void *stream) {
    NvtxRange nvtx_range("fdtd_symplectic_stage");
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!f || (e_or_h != 0 && e_or_h != 1)) return FDTD_ERR_ARG;
    for (int q = 0; q < 6; q++)
        if (!f[q]) return FDTD_ERR_ARG;
    const bool E = e_or_h == 1;
    const bool carr = cf && cf[0] && cf[1] && cf[2];
    if (cf && !carr && (cf[0] || cf[1] || cf[2])) return FDTD_ERR_ARG;  // all three or none
    if (E && !carr) return FDTD_ERR_ARG;                                 // E stages take ce arrays
    SympStage A{};
    A.coef = coef;
    A.cscalar = ch_scalar;
    A.clch = coef * ch_scalar;  // one IEEE single-precision product, as fdtd_symplectic_h_scalar_f32
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
            A.psi[2 * ax] = E ? psi->e[2 * ax] : psi->h[2 * ax];
            A.psi[2 * ax + 1] = E ? psi->e[2 * ax + 1] : psi->h[2 * ax + 1];
            if (!all_nonnull(A.b[ax], A.a[ax], A.km1[ax], A.psi[2 * ax], A.psi[2 * ax + 1])) return FDTD_ERR_ARG;
        }
    }
    // 32-bit offsets: every field and psi array has fewer than 2^31 elements
    if (g.nx * g.sx >= ((int64_t)1 << 31)) return FDTD_ERR_UNSUPPORTED;
    const Grid32 g32{(int32_t)g.nx, (int32_t)g.ny, (int32_t)g.nz, (uint32_t)g.sx, (uint32_t)g.sy};
    const dim3 grid((unsigned)((g.nz + kSympBlock - 1) / kSympBlock), (unsigned)g.ny, (unsigned)g.nx);
    cudaStream_t st = as_stream(stream);
    if (E) k_symp_stage<true, true><<<grid, kSympBlock, 0, st>>>(g32, A, f[0], f[1], f[2], f[3], f[4], f[5]);
    else if (carr) k_symp_stage<false, true><<<grid, kSympBlock, 0, st>>>(g32, A, f[0], f[1], f[2], f[3], f[4], f[5]);
    else k_symp_stage<false, false><<<grid, kSympBlock, 0, st>>>(g32, A, f[0], f[1], f[2], f[3], f[4], f[5]);
    return check_launch();
}

}  // extern "C"
