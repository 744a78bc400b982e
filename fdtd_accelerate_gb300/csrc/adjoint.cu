// Reverse-time (adjoint) kernels of the 2nd-order Yee step with CPML.
//
// The forward step (update_e, cpml_e, sources, update_h, cpml_h; the order of
// 2nd_order-Yee/CUDA/fdtd3d_201_250x250x320cell_15npml_100000tstep.cu:718-742
// with the kappa CPML of kuFDTD/before_CUDA/v0.3.0/boundary/core/cpml_core.c)
// is linear in the state (E, H, psi_e, psi_h) for fixed CE.  One adjoint step
// applies the transpose of that map to the adjoint state (lE, lH, lpsi_e,
// lpsi_h) and adds this step's share of dL/dCE:
//
//   reverse H part  lE += -0.5 curl_f(lH)                   (E-update form)
//                   + transpose of cpml_h (psi_h recursion, scatter of d)
//   reverse E part  nu = CE * lE
//                   lH += curl_b(nu)                        (H-update form)
//                   + transpose of cpml_e
//   gradient        dL/dCE += lE * G,  G = curl_f(H_prev) + sum sigma (km1 d + psi_e')
//
// where H_prev is the forward H entering the step and psi_e' the forward E-psi
// after its update in the step (G is the E increment divided by CE).
// Fields outside a component's update region never change in the forward
// step, so their adjoints feed nothing: every gather below reads the other
// family through its update mask, and only cells inside a mask are written.
// No atomics: each output element is produced by one thread, so the result
// does not depend on scheduling.
#include <cuda.h>

#include "common.cuh"

#include <mutex>

namespace fdtd {
namespace adj {

constexpr int kB = 128;

struct Args {
    Grid g;
    int P[3], front[3], back[3];
    float *lf[6];                 // lex, ley, lez, lhx, lhy, lhz
    float *lpe[6], *lph[6];       // adjoint psi (layouts of fdtd_psi)
    float *we[6], *wh[6];         // adjoint of the psi-driving differences (scratch)
    float *gce[3];                // dL/dCE accumulators
    const float *hp[3];           // forward H entering the step
    const float *pe[6];           // forward E-psi after its update in the step
    const float *ce[3];
    const float *be[3], *ae[3], *ke[3];
    const float *bh[3], *ah[3], *kh[3];
    // gbox = 1: dL/dCE accumulated only on cells [gb0, gb1) (a design region);
    // the adjoint fields are the same either way
    int32_t gbox;
    int64_t gb0[3], gb1[3];
};

// dense psi indices: x (2P, ny, nz), y (nx, 2P, nz), z (nx, ny, 2P)
__device__ __forceinline__ int64_t px(const Grid &g, int64_t s, int64_t j, int64_t k) { return (s * g.ny + j) * g.nz + k; }
__device__ __forceinline__ int64_t py(const Grid &g, int P, int64_t i, int64_t s, int64_t k) {
    return (i * 2 * P + s) * g.nz + k;
}
__device__ __forceinline__ int64_t pz(const Grid &g, int P, int64_t i, int64_t j, int64_t s) {
    return (i * g.ny + j) * 2 * P + s;
}

// node index -> slab index (or -1) on an enabled face; inverse of slab_node_e/h
__device__ __forceinline__ int slab_of_e(int64_t x, int P, int64_t n, int front, int back) {
    if (P == 0) return -1;
    if (front && x >= 1 && x <= P) return (int)(x - 1);
    if (back && x >= n - P - 1 && x <= n - 2) return (int)(P + x - (n - P - 1));
    return -1;
}
__device__ __forceinline__ int slab_of_h(int64_t x, int P, int64_t n, int front, int back) {
    if (P == 0) return -1;
    if (front && x >= 1 && x <= P) return (int)(x - 1);
    if (back && x >= n - P && x <= n - 1) return (int)(P + x - (n - P));
    return -1;
}

// update masks (2nd_order-Yee/Numpy/fdtd3d.py:4-13)
__device__ __forceinline__ bool em(const Grid &g, int q, int64_t i, int64_t j, int64_t k) {
    return q == 0 ? (j < g.ny - 1 && k < g.nz - 1) : q == 1 ? (i < g.nx - 1 && k < g.nz - 1) : (i < g.nx - 1 && j < g.ny - 1);
}
__device__ __forceinline__ bool hm(int q, int64_t i, int64_t j, int64_t k) {
    return q == 0 ? (j > 0 && k > 0) : q == 1 ? (i > 0 && k > 0) : (i > 0 && j > 0);
}

// ---------------------------------------------------------------------------
// 1. transpose of cpml_h on one axis: lpsi_h <- b*mu, w_h <- adjoint of d
//    (mu = lpsi + sigma*0.5*lH_target).  Invalid elements get w = 0.
//    psi order per axis: x (hyx, hzx), y (hzy, hxy), z (hxz, hyz); sigma (+, -)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void adj_psi(float &lpsi, float &w, float lt, float coef, int sigma, float b, float a,
                                        float km1) {
    const float h = fmul(coef, lt);
    const float mu = sigma > 0 ? fadd(lpsi, h) : fsub(lpsi, h);
    lpsi = fmul(b, mu);
    const float t = fmul(km1, h);
    w = fadd(sigma > 0 ? t : -t, fmul(a, mu));
}

template <int AX>
__global__ void __launch_bounds__(kB) k_adj_hpsi(Args A) {
    const Grid &g = A.g;
    const int P = A.P[AX];
    int64_t i, j, k, s, p;
    if (AX == 0) {
        k = (int64_t)blockIdx.x * kB + threadIdx.x; j = blockIdx.y; s = blockIdx.z;
        if (k >= g.nz) return;
        i = slab_node_h(s, P, g.nx);
        p = px(g, s, j, k);
    } else if (AX == 1) {
        k = (int64_t)blockIdx.x * kB + threadIdx.x; s = blockIdx.y; i = blockIdx.z;
        if (k >= g.nz) return;
        j = slab_node_h(s, P, g.ny);
        p = py(g, P, i, s, k);
    } else {  // blockIdx.y = i; u = j * 2P + s within the plane
        const uint32_t u = blockIdx.x * kB + threadIdx.x, w = 2u * (uint32_t)P;
        if (u >= (uint32_t)g.ny * w) return;
        i = blockIdx.y;
        j = u / w;
        s = u - (uint32_t)j * w;
        k = slab_node_h(s, P, g.nz);
        p = i * g.ny * w + u;
    }
    if (!(s < P ? A.front[AX] : A.back[AX])) return;
    const int64_t c = i * g.sx + j * g.sy + k;
    const float b = A.bh[AX][s], a = A.ah[AX][s], km1 = A.kh[AX][s];
    // (target H component, validity) of psi1 / psi2 on this axis
    const int t1 = AX == 0 ? 1 : AX == 1 ? 2 : 0;   // hy, hz, hx
    const int t2 = AX == 0 ? 2 : AX == 1 ? 0 : 1;   // hz, hx, hy
    const bool v1 = AX == 0 ? k > 0 : AX == 1 ? i > 0 : j > 0;
    const bool v2 = AX == 0 ? j > 0 : AX == 1 ? k > 0 : i > 0;
    float *lp1 = A.lph[2 * AX], *lp2 = A.lph[2 * AX + 1];
    float *w1 = A.wh[2 * AX], *w2 = A.wh[2 * AX + 1];
    if (v1) {
        float l = lp1[p], w;
        adj_psi(l, w, A.lf[3 + t1][c], 0.5f, +1, b, a, km1);
        lp1[p] = l;
        w1[p] = w;
    } else {
        w1[p] = 0.f;
    }
    if (v2) {
        float l = lp2[p], w;
        adj_psi(l, w, A.lf[3 + t2][c], 0.5f, -1, b, a, km1);
        lp2[p] = l;
        w2[p] = w;
    } else {
        w2[p] = 0.f;
    }
}

// ---------------------------------------------------------------------------
// 2. reverse H part on E cells + gradient.  One thread per cell.  Every load
//    comes first, then the arithmetic, then the stores: a store could alias a
//    later load as far as the compiler knows, and loads placed after stores
//    would wait for them instead of overlapping.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kB) k_adj_e(Args A) {
    const Grid &g = A.g;
    const int64_t k = (int64_t)blockIdx.x * kB + threadIdx.x;
    const int64_t j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    const int64_t c = i * g.sx + j * g.sy + k, X = g.sx, Y = g.sy;
    const bool e0 = em(g, 0, i, j, k), e1 = em(g, 1, i, j, k), e2 = em(g, 2, i, j, k);
    // slab indices of this cell's nodes (H-node form for the w_h gather,
    // E-node form for the gradient's psi terms)
    const int sxh0 = slab_of_h(i, A.P[0], g.nx, A.front[0], A.back[0]);
    const int sxh1 = slab_of_h(i + 1, A.P[0], g.nx, A.front[0], A.back[0]);
    const int syh0 = slab_of_h(j, A.P[1], g.ny, A.front[1], A.back[1]);
    const int syh1 = slab_of_h(j + 1, A.P[1], g.ny, A.front[1], A.back[1]);
    const int szh0 = slab_of_h(k, A.P[2], g.nz, A.front[2], A.back[2]);
    const int szh1 = slab_of_h(k + 1, A.P[2], g.nz, A.front[2], A.back[2]);
    const int sxe = slab_of_e(i, A.P[0], g.nx, A.front[0], A.back[0]);
    const int sye = slab_of_e(j, A.P[1], g.ny, A.front[1], A.back[1]);
    const int sze = slab_of_e(k, A.P[2], g.nz, A.front[2], A.back[2]);
    const int Py = A.P[1], Pz = A.P[2];
    const bool gin = !A.gbox || (i >= A.gb0[0] && i < A.gb1[0] && j >= A.gb0[1] && j < A.gb1[1] &&
                                 k >= A.gb0[2] && k < A.gb1[2]);

    // ---- loads
    auto L = [&](const float *f, bool m, int64_t o) { return m ? __ldg(f + c + o) : 0.f; };
    auto W = [&](int q, bool m, int64_t p) { return m ? __ldg(A.wh[q] + p) : 0.f; };
    const float *lhx = A.lf[3], *lhy = A.lf[4], *lhz = A.lf[5];
    // adjoint H through the H update masks: the cell, and the +1 neighbours
    // each E component differentiates (their loads only where it is updated)
    const float hz0 = L(lhz, i > 0 && j > 0, 0), hy0 = L(lhy, i > 0 && k > 0, 0), hx0 = L(lhx, j > 0 && k > 0, 0);
    const float hzj = L(lhz, e0 && i > 0, Y), hyk = L(lhy, e0 && i > 0, 1);  // ex
    const float hxk = L(lhx, e1 && j > 0, 1), hzi = L(lhz, e1 && j > 0, X);  // ey
    const float hyi = L(lhy, e2 && k > 0, X), hxj = L(lhx, e2 && k > 0, Y);  // ez
    // w_h of the slab nodes at this index (+) and one above (-), per component
    // ex: hzy (y, psi 0 of h) and hyz (z, psi 1); ey: hzx (x, psi 1) and hxz
    // (z, psi 0); ez: hyx (x, psi 0) and hxy (y, psi 1)
    const float wx0 = W(2, e0 && syh0 >= 0, py(g, Py, i, syh0, k)), wx1 = W(2, e0 && syh1 >= 0, py(g, Py, i, syh1, k));
    const float wx2 = W(5, e0 && szh0 >= 0, pz(g, Pz, i, j, szh0)), wx3 = W(5, e0 && szh1 >= 0, pz(g, Pz, i, j, szh1));
    const float wy0 = W(1, e1 && sxh0 >= 0, px(g, sxh0, j, k)), wy1 = W(1, e1 && sxh1 >= 0, px(g, sxh1, j, k));
    const float wy2 = W(4, e1 && szh0 >= 0, pz(g, Pz, i, j, szh0)), wy3 = W(4, e1 && szh1 >= 0, pz(g, Pz, i, j, szh1));
    const float wz0 = W(0, e2 && sxh0 >= 0, px(g, sxh0, j, k)), wz1 = W(0, e2 && sxh1 >= 0, px(g, sxh1, j, k));
    const float wz2 = W(3, e2 && syh0 >= 0, py(g, Py, i, syh0, k)), wz3 = W(3, e2 && syh1 >= 0, py(g, Py, i, syh1, k));
    const float le0 = e0 ? A.lf[0][c] : 0.f, le1 = e1 ? A.lf[1][c] : 0.f, le2 = e2 ? A.lf[2][c] : 0.f;
    // gradient: forward H entering the step (unmasked), forward E-psi, accumulators
    float Hz0 = 0.f, Hzj = 0.f, Hzi = 0.f, Hy0 = 0.f, Hyk = 0.f, Hyi = 0.f, Hx0 = 0.f, Hxk = 0.f, Hxj = 0.f;
    float pe3 = 0.f, pe4 = 0.f, pe0 = 0.f, pe5 = 0.f, pe1 = 0.f, pe2 = 0.f, g0 = 0.f, g1 = 0.f, g2 = 0.f;
    if (gin) {
        const float *hx = A.hp[0], *hy = A.hp[1], *hz = A.hp[2];
        Hz0 = __ldg(hz + c);
        Hy0 = __ldg(hy + c);
        Hx0 = __ldg(hx + c);
        if (e0) {
            Hzj = __ldg(hz + c + Y);
            Hyk = __ldg(hy + c + 1);
            if (sye >= 0) pe3 = __ldg(A.pe[3] + py(g, Py, i, sye, k));
            if (sze >= 0) pe4 = __ldg(A.pe[4] + pz(g, Pz, i, j, sze));
            g0 = A.gce[0][c];
        }
        if (e1) {
            Hxk = __ldg(hx + c + 1);
            Hzi = __ldg(hz + c + X);
            if (sxe >= 0) pe0 = __ldg(A.pe[0] + px(g, sxe, j, k));
            if (sze >= 0) pe5 = __ldg(A.pe[5] + pz(g, Pz, i, j, sze));
            g1 = A.gce[1][c];
        }
        if (e2) {
            Hyi = __ldg(hy + c + X);
            Hxj = __ldg(hx + c + Y);
            if (sxe >= 0) pe1 = __ldg(A.pe[1] + px(g, sxe, j, k));
            if (sye >= 0) pe2 = __ldg(A.pe[2] + py(g, Py, i, sye, k));
            g2 = A.gce[2][c];
        }
    }

    // ---- arithmetic and stores
    if (e0) {  // ex
        float d = fmul(-0.5f, curl4(hzj, hz0, hyk, hy0));
        if (syh0 >= 0) d = fadd(d, wx0);
        if (syh1 >= 0) d = fsub(d, wx1);
        if (szh0 >= 0) d = fadd(d, wx2);
        if (szh1 >= 0) d = fsub(d, wx3);
        const float l = fadd(le0, d);
        A.lf[0][c] = l;
        if (gin) {
            // G = curl_f(H) + (exy: +) + (exz: -)
            float G = curl4(Hzj, Hz0, Hyk, Hy0);
            if (sye >= 0) G = fadd(G, fadd(fmul(__ldg(A.ke[1] + sye), fsub(Hzj, Hz0)), pe3));
            if (sze >= 0) G = fsub(G, fadd(fmul(__ldg(A.ke[2] + sze), fsub(Hyk, Hy0)), pe4));
            A.gce[0][c] = fadd(g0, fmul(l, G));
        }
    }
    if (e1) {  // ey
        float d = fmul(-0.5f, curl4(hxk, hx0, hzi, hz0));
        if (sxh0 >= 0) d = fadd(d, wy0);
        if (sxh1 >= 0) d = fsub(d, wy1);
        if (szh0 >= 0) d = fadd(d, wy2);
        if (szh1 >= 0) d = fsub(d, wy3);
        const float l = fadd(le1, d);
        A.lf[1][c] = l;
        if (gin) {
            // G = curl_f(H) + (eyx: -) + (eyz: +)
            float G = curl4(Hxk, Hx0, Hzi, Hz0);
            if (sxe >= 0) G = fsub(G, fadd(fmul(__ldg(A.ke[0] + sxe), fsub(Hzi, Hz0)), pe0));
            if (sze >= 0) G = fadd(G, fadd(fmul(__ldg(A.ke[2] + sze), fsub(Hxk, Hx0)), pe5));
            A.gce[1][c] = fadd(g1, fmul(l, G));
        }
    }
    if (e2) {  // ez
        float d = fmul(-0.5f, curl4(hyi, hy0, hxj, hx0));
        if (sxh0 >= 0) d = fadd(d, wz0);
        if (sxh1 >= 0) d = fsub(d, wz1);
        if (syh0 >= 0) d = fadd(d, wz2);
        if (syh1 >= 0) d = fsub(d, wz3);
        const float l = fadd(le2, d);
        A.lf[2][c] = l;
        if (gin) {
            // G = curl_f(H) + (ezx: +) + (ezy: -)
            float G = curl4(Hyi, Hy0, Hxj, Hx0);
            if (sxe >= 0) G = fadd(G, fadd(fmul(__ldg(A.ke[0] + sxe), fsub(Hyi, Hy0)), pe1));
            if (sye >= 0) G = fsub(G, fadd(fmul(__ldg(A.ke[1] + sye), fsub(Hxj, Hx0)), pe2));
            A.gce[2][c] = fadd(g2, fmul(l, G));
        }
    }
}

// ---------------------------------------------------------------------------
// 3. transpose of cpml_e on one axis: nu = CE*lE_target, mu = lpsi + sigma*nu,
//    lpsi_e <- b*mu, w_e <- sigma*km1*nu + a*mu.
//    psi order per axis: x (eyx -, ezx +), y (ezy -, exy +), z (exz -, eyz +)
// ---------------------------------------------------------------------------
template <int AX>
__global__ void __launch_bounds__(kB) k_adj_epsi(Args A) {
    const Grid &g = A.g;
    const int P = A.P[AX];
    int64_t i, j, k, s, p;
    if (AX == 0) {
        k = (int64_t)blockIdx.x * kB + threadIdx.x; j = blockIdx.y; s = blockIdx.z;
        if (k >= g.nz) return;
        i = slab_node_e(s, P, g.nx);
        p = px(g, s, j, k);
    } else if (AX == 1) {
        k = (int64_t)blockIdx.x * kB + threadIdx.x; s = blockIdx.y; i = blockIdx.z;
        if (k >= g.nz) return;
        j = slab_node_e(s, P, g.ny);
        p = py(g, P, i, s, k);
    } else {  // blockIdx.y = i; u = j * 2P + s within the plane
        const uint32_t u = blockIdx.x * kB + threadIdx.x, w = 2u * (uint32_t)P;
        if (u >= (uint32_t)g.ny * w) return;
        i = blockIdx.y;
        j = u / w;
        s = u - (uint32_t)j * w;
        k = slab_node_e(s, P, g.nz);
        p = i * g.ny * w + u;
    }
    if (!(s < P ? A.front[AX] : A.back[AX])) return;
    const int64_t c = i * g.sx + j * g.sy + k;
    const float b = A.be[AX][s], a = A.ae[AX][s], km1 = A.ke[AX][s];
    const int t1 = AX == 0 ? 1 : AX == 1 ? 2 : 0;   // ey, ez, ex
    const int t2 = AX == 0 ? 2 : AX == 1 ? 0 : 1;   // ez, ex, ey
    const bool v1 = AX == 0 ? k < g.nz - 1 : AX == 1 ? i < g.nx - 1 : j < g.ny - 1;
    const bool v2 = AX == 0 ? j < g.ny - 1 : AX == 1 ? k < g.nz - 1 : i < g.nx - 1;
    float *lp1 = A.lpe[2 * AX], *lp2 = A.lpe[2 * AX + 1];
    float *w1 = A.we[2 * AX], *w2 = A.we[2 * AX + 1];
    if (v1) {
        float l = lp1[p], w;
        adj_psi(l, w, A.lf[t1][c], A.ce[t1][c], -1, b, a, km1);
        lp1[p] = l;
        w1[p] = w;
    } else {
        w1[p] = 0.f;
    }
    if (v2) {
        float l = lp2[p], w;
        adj_psi(l, w, A.lf[t2][c], A.ce[t2][c], +1, b, a, km1);
        lp2[p] = l;
        w2[p] = w;
    } else {
        w2[p] = 0.f;
    }
}

// ---------------------------------------------------------------------------
// 4. reverse E part on H cells: lH += curl_b(CE*lE) + scatter of w_e.  Loads
//    first, as in k_adj_e.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kB) k_adj_h(Args A) {
    const Grid &g = A.g;
    const int64_t k = (int64_t)blockIdx.x * kB + threadIdx.x;
    const int64_t j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    const int64_t c = i * g.sx + j * g.sy + k, X = g.sx, Y = g.sy;
    const bool h0 = hm(0, i, j, k), h1 = hm(1, i, j, k), h2 = hm(2, i, j, k);
    const int Px = A.P[0], Py = A.P[1], Pz = A.P[2];
    // E-node slabs at this index and one below (H cell h: +w at node h-1, -w at node h)
    const int sx0 = slab_of_e(i - 1, Px, g.nx, A.front[0], A.back[0]);
    const int sx1 = slab_of_e(i, Px, g.nx, A.front[0], A.back[0]);
    const int sy0 = slab_of_e(j - 1, Py, g.ny, A.front[1], A.back[1]);
    const int sy1 = slab_of_e(j, Py, g.ny, A.front[1], A.back[1]);
    const int sz0 = slab_of_e(k - 1, Pz, g.nz, A.front[2], A.back[2]);
    const int sz1 = slab_of_e(k, Pz, g.nz, A.front[2], A.back[2]);

    // ---- loads
    // nu = CE * lE of component q at offset o, zero outside q's update mask
    // (m: the mask at that cell; the load only where it is needed)
    auto NU = [&](int q, bool need, bool m, int64_t o) {
        return need && m ? fmul(__ldg(A.ce[q] + c + o), __ldg(A.lf[q] + c + o)) : 0.f;
    };
    auto W = [&](int q, bool m, int64_t p) { return m ? __ldg(A.we[q] + p) : 0.f; };
    const float n0 = NU(0, h1 || h2, em(g, 0, i, j, k), 0), n1 = NU(1, h0 || h2, em(g, 1, i, j, k), 0),
                n2 = NU(2, h0 || h1, em(g, 2, i, j, k), 0);
    const float n2j = NU(2, h0, em(g, 2, i, j - 1, k), -Y), n1k = NU(1, h0, em(g, 1, i, j, k - 1), -1);  // hx
    const float n0k = NU(0, h1, em(g, 0, i, j, k - 1), -1), n2i = NU(2, h1, em(g, 2, i - 1, j, k), -X);  // hy
    const float n1i = NU(1, h2, em(g, 1, i - 1, j, k), -X), n0j = NU(0, h2, em(g, 0, i, j - 1, k), -Y);  // hz
    // w_e of the slab nodes one below (+) and at this index (-), per component
    // hx: ezy (y, psi 0 of e) and eyz (z, psi 1); hy: ezx (x, psi 1) and exz
    // (z, psi 0); hz: eyx (x, psi 0) and exy (y, psi 1)
    const float wx0 = W(2, h0 && sy0 >= 0, py(g, Py, i, sy0, k)), wx1 = W(2, h0 && sy1 >= 0, py(g, Py, i, sy1, k));
    const float wx2 = W(5, h0 && sz0 >= 0, pz(g, Pz, i, j, sz0)), wx3 = W(5, h0 && sz1 >= 0, pz(g, Pz, i, j, sz1));
    const float wy0 = W(1, h1 && sx0 >= 0, px(g, sx0, j, k)), wy1 = W(1, h1 && sx1 >= 0, px(g, sx1, j, k));
    const float wy2 = W(4, h1 && sz0 >= 0, pz(g, Pz, i, j, sz0)), wy3 = W(4, h1 && sz1 >= 0, pz(g, Pz, i, j, sz1));
    const float wz0 = W(0, h2 && sx0 >= 0, px(g, sx0, j, k)), wz1 = W(0, h2 && sx1 >= 0, px(g, sx1, j, k));
    const float wz2 = W(3, h2 && sy0 >= 0, py(g, Py, i, sy0, k)), wz3 = W(3, h2 && sy1 >= 0, py(g, Py, i, sy1, k));
    const float lh0 = h0 ? A.lf[3][c] : 0.f, lh1 = h1 ? A.lf[4][c] : 0.f, lh2 = h2 ? A.lf[5][c] : 0.f;

    // ---- arithmetic and stores
    if (h0) {  // hx
        float d = curl4(n2, n2j, n1, n1k);
        if (sy0 >= 0) d = fadd(d, wx0);
        if (sy1 >= 0) d = fsub(d, wx1);
        if (sz0 >= 0) d = fadd(d, wx2);
        if (sz1 >= 0) d = fsub(d, wx3);
        A.lf[3][c] = fadd(lh0, d);
    }
    if (h1) {  // hy
        float d = curl4(n0, n0k, n2, n2i);
        if (sx0 >= 0) d = fadd(d, wy0);
        if (sx1 >= 0) d = fsub(d, wy1);
        if (sz0 >= 0) d = fadd(d, wy2);
        if (sz1 >= 0) d = fsub(d, wy3);
        A.lf[4][c] = fadd(lh1, d);
    }
    if (h2) {  // hz
        float d = curl4(n1, n1i, n0, n0j);
        if (sx0 >= 0) d = fadd(d, wz0);
        if (sx1 >= 0) d = fsub(d, wz1);
        if (sy0 >= 0) d = fadd(d, wz2);
        if (sy1 >= 0) d = fsub(d, wz3);
        A.lf[5][c] = fadd(lh2, d);
    }
}

// ---------------------------------------------------------------------------
// point lists: gather (monitors) and add (adjoint injection), list order
// ---------------------------------------------------------------------------
// cell offset of point p, or -1 when the point or its component is out of range
__device__ __forceinline__ int64_t point_offset(const Grid &g, const fdtd_points &pts, int p) {
    const int64_t i = pts.ijk[3 * p], j = pts.ijk[3 * p + 1], k = pts.ijk[3 * p + 2];
    const int q = pts.comp[p];
    if (i < 0 || i >= g.nx || j < 0 || j >= g.ny || k < 0 || k >= g.nz || q < 0 || q > 5) return -1;
    return i * g.sx + j * g.sy + k;
}

// out-of-range points read as NaN
__global__ void k_gather_points(Grid g, fdtd_points pts, fdtd_fields6 f, float *out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= pts.n) return;
    const int64_t c = point_offset(g, pts, p);
    out[p] = c >= 0 ? f.f[pts.comp[p]][c] : __int_as_float(0x7fc00000);
}

// Adds vals[p] to the cell of every point p, as a walk of the list in order
// would (out-of-range points are skipped).  Lists of up to kAddThreads
// points: one thread per point, one block.  A point whose cell and component
// an earlier point also names is skipped by its thread; the thread of the
// first such point adds the values of all of them in list order.
constexpr int kAddThreads = 1024;
__global__ void k_add_points(Grid g, fdtd_points pts, fdtd_fields6 f, const float *vals) {
    const int p = threadIdx.x;
    if (blockIdx.x != 0 || p >= pts.n) return;
    const int64_t c = point_offset(g, pts, p);
    if (c < 0) return;
    const int q = pts.comp[p];
    for (int r = 0; r < p; r++)
        if (pts.comp[r] == q && point_offset(g, pts, r) == c) return;
    float *fp = f.f[q] + c;
    float v = *fp;
    for (int r = p; r < pts.n; r++)
        if (pts.comp[r] == q && point_offset(g, pts, r) == c) v = fadd(v, vals[r]);
    *fp = v;
}
// longer lists: one thread walks the list
__global__ void k_add_points_walk(Grid g, fdtd_points pts, fdtd_fields6 f, const float *vals) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int p = 0; p < pts.n; p++) {
        const int64_t c = point_offset(g, pts, p);
        if (c < 0) continue;
        float *fp = f.f[pts.comp[p]] + c;
        *fp = fadd(*fp, vals[p]);
    }
}
static void add_points(const Grid &g, const fdtd_points &pts, const fdtd_fields6 &f, const float *vals,
                       cudaStream_t st) {
    if (pts.n <= kAddThreads)
        k_add_points<<<1, (pts.n + 31) / 32 * 32, 0, st>>>(g, pts, f, vals);
    else
        k_add_points_walk<<<1, 32, 0, st>>>(g, pts, f, vals);
}

static dim3 cells(const Grid &g) {
    return dim3((unsigned)((g.nz + kB - 1) / kB), (unsigned)g.ny, (unsigned)g.nx);
}

template <int AX>
static void launch_slab(const Grid &g, int P, bool e, const Args &A, cudaStream_t st) {
    dim3 grid;
    if (AX == 0) grid = dim3((unsigned)((g.nz + kB - 1) / kB), (unsigned)g.ny, (unsigned)(2 * P));
    else if (AX == 1) grid = dim3((unsigned)((g.nz + kB - 1) / kB), (unsigned)(2 * P), (unsigned)g.nx);
    else grid = dim3((unsigned)((g.ny * 2 * P + kB - 1) / kB), (unsigned)g.nx);
    if (e) k_adj_epsi<AX><<<grid, kB, 0, st>>>(A);
    else k_adj_hpsi<AX><<<grid, kB, 0, st>>>(A);
}

static int validate_points(const Grid &g, const fdtd_points *pts) {
    if (!pts || pts->n < 0) return FDTD_ERR_ARG;
    if (pts->n > 0 && !all_nonnull(pts->ijk, pts->comp)) return FDTD_ERR_ARG;
    (void)g;
    return FDTD_OK;
}

}  // namespace adj
}  // namespace fdtd

using namespace fdtd;
using namespace fdtd::adj;

extern "C" {

}  // extern "C"

// one reverse step; box (i0, j0, k0, ni, nj, nk) limits the dL/dCE
// accumulation, NULL: every cell
static int adjoint_step(const fdtd_grid *gp, const fdtd_cpml *cp, const fdtd_adjoint_state *s,
                        const float *const h_prev[3], const float *const psi_e_cur[6], const float *const ce[3],
                        const fdtd_points *mon, const float *mon_grad, const int64_t *box, void *stream) {
    NvtxRange nvtx_range("fdtd_adjoint_step");
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!s || !h_prev || !ce) return FDTD_ERR_ARG;
    for (int q = 0; q < 6; q++)
        if (!s->lf[q]) return FDTD_ERR_ARG;
    for (int q = 0; q < 3; q++)
        if (!all_nonnull(s->grad_ce[q], h_prev[q], ce[q])) return FDTD_ERR_ARG;
    Args A{};
    A.g = g;
    const int64_t n[3] = {g.nx, g.ny, g.nz};
    for (int a = 0; a < 3; a++) {
        const int P = cp ? cp->npml[a] : 0;
        if (P < 0) return FDTD_ERR_ARG;
        A.P[a] = P;
        A.front[a] = cp ? (cp->faces >> (2 * a)) & 1 : 0;
        A.back[a] = cp ? (cp->faces >> (2 * a + 1)) & 1 : 0;
        if (P == 0) continue;
        if (n[a] < 2 * P + 2) return FDTD_ERR_SHAPE;
        if (a < 2 && 2 * P > 65535) return FDTD_ERR_SHAPE;
        if (!psi_e_cur) return FDTD_ERR_ARG;
        if (!all_nonnull(cp->b_e[a], cp->a_e[a], cp->km1_e[a], cp->b_h[a], cp->a_h[a], cp->km1_h[a]))
            return FDTD_ERR_ARG;
        for (int q = 2 * a; q < 2 * a + 2; q++)
            if (!all_nonnull(s->lpsi_e[q], s->lpsi_h[q], s->w_e[q], s->w_h[q], psi_e_cur[q])) return FDTD_ERR_ARG;
        A.be[a] = cp->b_e[a]; A.ae[a] = cp->a_e[a]; A.ke[a] = cp->km1_e[a];
        A.bh[a] = cp->b_h[a]; A.ah[a] = cp->a_h[a]; A.kh[a] = cp->km1_h[a];
    }
    for (int q = 0; q < 6; q++) {
        A.lf[q] = s->lf[q];
        A.lpe[q] = s->lpsi_e[q];
        A.lph[q] = s->lpsi_h[q];
        A.we[q] = s->w_e[q];
        A.wh[q] = s->w_h[q];
        A.pe[q] = psi_e_cur ? psi_e_cur[q] : nullptr;
    }
    for (int q = 0; q < 3; q++) {
        A.gce[q] = s->grad_ce[q];
        A.hp[q] = h_prev[q];
        A.ce[q] = ce[q];
    }
    if (box) {
        const int64_t n3[3] = {g.nx, g.ny, g.nz};
        for (int a = 0; a < 3; a++) {
            if (box[a] < 0 || box[3 + a] < 0 || box[a] + box[3 + a] > n3[a]) return FDTD_ERR_SHAPE;
            A.gb0[a] = box[a];
            A.gb1[a] = box[a] + box[3 + a];
        }
        A.gbox = 1;
    }
    cudaStream_t st = as_stream(stream);
    if (mon && mon->n > 0) {
        FDTD_TRY(validate_points(g, mon));
        if (!mon_grad) return FDTD_ERR_ARG;
        fdtd_fields6 lf;
        for (int q = 0; q < 6; q++) lf.f[q] = s->lf[q];
        add_points(g, *mon, lf, mon_grad, st);
    }
    if (A.P[0]) launch_slab<0>(g, A.P[0], false, A, st);
    if (A.P[1]) launch_slab<1>(g, A.P[1], false, A, st);
    if (A.P[2]) launch_slab<2>(g, A.P[2], false, A, st);
    k_adj_e<<<cells(g), kB, 0, st>>>(A);
    if (A.P[0]) launch_slab<0>(g, A.P[0], true, A, st);
    if (A.P[1]) launch_slab<1>(g, A.P[1], true, A, st);
    if (A.P[2]) launch_slab<2>(g, A.P[2], true, A, st);
    k_adj_h<<<cells(g), kB, 0, st>>>(A);
    return check_launch();
}

extern "C" {

int fdtd_adjoint_step_f32(const fdtd_grid *gp, const fdtd_cpml *cp, const fdtd_adjoint_state *s,
                          const float *const h_prev[3], const float *const psi_e_cur[6], const float *const ce[3],
                          const fdtd_points *mon, const float *mon_grad, void *stream) {
    return adjoint_step(gp, cp, s, h_prev, psi_e_cur, ce, mon, mon_grad, nullptr, stream);
}

int fdtd_adjoint_step_region_f32(const fdtd_grid *gp, const fdtd_cpml *cp, const fdtd_adjoint_state *s,
                                 const float *const h_prev[3], const float *const psi_e_cur[6],
                                 const float *const ce[3], const fdtd_points *mon, const float *mon_grad,
                                 const int64_t grad_box[6], void *stream) {
    if (!grad_box) return FDTD_ERR_ARG;
    return adjoint_step(gp, cp, s, h_prev, psi_e_cur, ce, mon, mon_grad, grad_box, stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free adjoint step.
//
// fdtd_adjoint_step_f32 needs scratch for the w_e / w_h arrays (the adjoint
// of the psi-driving differences, psi-shaped, written and read within one
// call).  Some callers cannot provide it: a host binding with no device
// allocator of its own (a plain C, cgo or JNI caller of this library), or a
// loop that must not call cudaMalloc, which synchronises the device and is
// not allowed while a stream is being captured.  This entry point takes the
// scratch from a fixed device array compiled into the library instead.
//
//  * Maximum: kNoAllocScratchFloats floats (4 Mi floats = 16 MiB) for the
//    12 w arrays, i.e. 4 * (2Px*ny*nz + nx*2Py*nz + nx*ny*2Pz) floats plus
//    alignment; larger CPML layers are refused with FDTD_ERR_CAPACITY.
//  * Set-up: the first call in a CUDA context looks up the array's device
//    address (cudaGetSymbolAddress, with that context's device current) and
//    caches it under the context's unique id; make that first call before
//    any stream capture.  A context created anew (after cudaDeviceReset, for
//    instance) loads the module again and gets a fresh lookup.
//  * Nothing in the scratch has to start at zero: every element the kernels
//    read is written earlier in the same call (disabled faces are neither
//    written nor read).
//  * One scratch per device: calls that overlap in time (different streams
//    or host threads on one device) race on it.
// ---------------------------------------------------------------------------
namespace fdtd {
namespace adj {

constexpr size_t kNoAllocScratchFloats = size_t(4) << 20;
constexpr int kMaxContexts = 64;

static __device__ __align__(256) float g_noalloc_scratch[kNoAllocScratchFloats];

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

// Unique id of the calling thread's current context (0 when none is current).
static int current_context_id(unsigned long long *id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    if (!get_current || !get_id) {
        void *a = nullptr, *b = nullptr;
        cudaDriverEntryPointQueryResult qa, qb;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) != cudaSuccess ||
            qa != cudaDriverEntryPointSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) != cudaSuccess ||
            qb != cudaDriverEntryPointSuccess)
            return FDTD_ERR_CUDA;
        get_current = reinterpret_cast<CtxGetCurrentFn>(a);
        get_id = reinterpret_cast<CtxGetIdFn>(b);
    }
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return FDTD_ERR_CUDA;
    return get_id(ctx, id) == CUDA_SUCCESS ? FDTD_OK : FDTD_ERR_CUDA;
}

static std::mutex g_noalloc_mu;
static unsigned long long g_noalloc_ctx[kMaxContexts];
static float *g_noalloc_ptr[kMaxContexts];
static int g_noalloc_n = 0;

static int noalloc_scratch(float **out) {
    unsigned long long id = 0;
    cudaError_t e;
    if (current_context_id(&id) != FDTD_OK) {
        // no context current on this thread yet: the symbol lookup initialises
        // the current device's primary context and makes it current
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) { set_cuda_error(e); return FDTD_ERR_CUDA; }
        FDTD_TRY(current_context_id(&id));
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    for (int q = 0; q < g_noalloc_n; q++)
        if (g_noalloc_ctx[q] == id) {
            *out = g_noalloc_ptr[q];
            return FDTD_OK;
        }
    if (g_noalloc_n == kMaxContexts) return FDTD_ERR_UNSUPPORTED;
    void *ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) { set_cuda_error(e); return FDTD_ERR_CUDA; }
    g_noalloc_ctx[g_noalloc_n] = id;
    g_noalloc_ptr[g_noalloc_n] = static_cast<float *>(ptr);
    g_noalloc_n++;
    *out = static_cast<float *>(ptr);
    return FDTD_OK;
}

}  // namespace adj
}  // namespace fdtd

extern "C" {

int fdtd_adjoint_step_noalloc_f32(const fdtd_grid *gp, const fdtd_cpml *cp, const fdtd_adjoint_state *s,
                                  const float *const h_prev[3], const float *const psi_e_cur[6],
                                  const float *const ce[3], const fdtd_points *mon, const float *mon_grad,
                                  void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!s) return FDTD_ERR_ARG;
    // psi-shaped w arrays of each axis, 256-byte aligned inside the scratch
    size_t sz[3] = {0, 0, 0};
    if (cp) {
        for (int a = 0; a < 3; a++)
            if (cp->npml[a] < 0) return FDTD_ERR_ARG;
        sz[0] = (size_t)2 * cp->npml[0] * g.ny * g.nz;
        sz[1] = (size_t)g.nx * 2 * cp->npml[1] * g.nz;
        sz[2] = (size_t)g.nx * g.ny * 2 * cp->npml[2];
    }
    auto al = [](size_t n) { return (n + 63) / 64 * 64; };
    const size_t need = 4 * (al(sz[0]) + al(sz[1]) + al(sz[2]));
    if (need > kNoAllocScratchFloats) return FDTD_ERR_CAPACITY;
    float *base = nullptr;
    FDTD_TRY(noalloc_scratch(&base));
    fdtd_adjoint_state t = *s;
    size_t off = 0;
    for (int a = 0; a < 3; a++) {
        float **slots[4] = {&t.w_e[2 * a], &t.w_e[2 * a + 1], &t.w_h[2 * a], &t.w_h[2 * a + 1]};
        for (float **w : slots) {
            *w = sz[a] ? base + off : nullptr;
            off += al(sz[a]);
        }
    }
    return fdtd_adjoint_step_f32(gp, cp, &t, h_prev, psi_e_cur, ce, mon, mon_grad, stream);
}

int fdtd_gather_points_f32(const fdtd_grid *gp, const fdtd_points *pts, const float *const f[6], float *out,
                           void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    FDTD_TRY(validate_points(g, pts));
    if (pts->n == 0) return FDTD_OK;
    if (!f || !out) return FDTD_ERR_ARG;
    fdtd_fields6 ff;
    for (int q = 0; q < 6; q++) ff.f[q] = const_cast<float *>(f[q]);
    k_gather_points<<<(pts->n + 127) / 128, 128, 0, as_stream(stream)>>>(g, *pts, ff, out);
    return check_launch();
}

int fdtd_add_points_f32(const fdtd_grid *gp, const fdtd_points *pts, float *const f[6], const float *vals,
                        void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    FDTD_TRY(validate_points(g, pts));
    if (pts->n == 0) return FDTD_OK;
    if (!f || !vals) return FDTD_ERR_ARG;
    fdtd_fields6 ff;
    for (int q = 0; q < 6; q++) ff.f[q] = f[q];
    add_points(g, *pts, ff, vals, as_stream(stream));
    return check_launch();
}

}  // extern "C"
