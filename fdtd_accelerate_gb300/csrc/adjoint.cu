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

#include <algorithm>
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

// transpose of one psi recursion at one slab element: mu = lpsi + sigma *
// coef * lt (lt the adjoint of the component the psi corrects), lpsi <- b*mu,
// w <- sigma*km1*coef*lt + a*mu (the adjoint of the psi-driving difference)
__device__ __forceinline__ void adj_psi(float &lpsi, float &w, float lt, float coef, int sigma, float b, float a,
                                        float km1) {
    const float h = fmul(coef, lt);
    const float mu = sigma > 0 ? fadd(lpsi, h) : fsub(lpsi, h);
    lpsi = fmul(b, mu);
    const float t = fmul(km1, h);
    w = fadd(sigma > 0 ? t : -t, fmul(a, mu));
}

// ---------------------------------------------------------------------------
// 1. and 3. The psi transposes of one family, all three axes in one launch
//    (E false: transpose of cpml_h, lpsi_h <- b*mu, w_h <- adjoint of d with
//    mu = lpsi + sigma*0.5*lH_target; E true: transpose of cpml_e, nu =
//    CE*lE_target, mu = lpsi + sigma*nu, lpsi_e <- b*mu, w_e <- sigma*km1*nu +
//    a*mu).  Invalid elements get w = 0.  Blocks [nb[a-1], nb[a]) take axis a,
//    kB consecutive elements of its dense psi array each; indices in I.
//    psi order per axis: x (y, z targets), y (z, x), z (x, y); H sigma (+, -),
//    E sigma (-, +).
// ---------------------------------------------------------------------------
struct PsiBlocks {
    int32_t nb[3];  // cumulative block counts of the x, y and z slabs
};
template <bool E, typename I>
__global__ void __launch_bounds__(kB) k_adj_psi3(Args A, PsiBlocks R) {
    const int b = blockIdx.x;
    const int ax = b < R.nb[0] ? 0 : (b < R.nb[1] ? 1 : 2);
    const I nx = A.g.nx, ny = A.g.ny, nz = A.g.nz;
    const int P = A.P[ax];
    const I tp = 2 * P;
    const I t = (I)(b - (ax ? R.nb[ax - 1] : 0)) * kB + threadIdx.x;  // element of the dense psi array
    I i, j, k;
    int s;
    auto node = [&](int sl, I n) { return (I)(E ? slab_node_e(sl, P, n) : slab_node_h(sl, P, n)); };
    if (ax == 0) {  // (2P, ny, nz)
        if (t >= tp * ny * nz) return;
        k = t % nz;
        const I r = t / nz;
        j = r % ny;
        s = (int)(r / ny);
        i = node(s, nx);
    } else if (ax == 1) {  // (nx, 2P, nz)
        if (t >= nx * tp * nz) return;
        k = t % nz;
        const I r = t / nz;
        s = (int)(r % tp);
        i = r / tp;
        j = node(s, ny);
    } else {  // (nx, ny, 2P)
        if (t >= nx * ny * tp) return;
        s = (int)(t % tp);
        const I r = t / tp;
        j = r % ny;
        i = r / ny;
        k = node(s, nz);
    }
    if (!(s < P ? A.front[ax] : A.back[ax])) return;
    const I c = i * (I)A.g.sx + j * (I)A.g.sy + k;
    const float bcoef = E ? A.be[ax][s] : A.bh[ax][s], a = E ? A.ae[ax][s] : A.ah[ax][s],
                km1 = E ? A.ke[ax][s] : A.kh[ax][s];
    // target components of psi1 / psi2 on this axis (x: y, z; y: z, x; z: x, y)
    // and their validity (the update masks of the target family)
    const int t1 = ax == 0 ? 1 : ax == 1 ? 2 : 0, t2 = ax == 0 ? 2 : ax == 1 ? 0 : 1;
    bool v1, v2;
    if (E) {
        v1 = ax == 0 ? k < nz - 1 : ax == 1 ? i < nx - 1 : j < ny - 1;
        v2 = ax == 0 ? j < ny - 1 : ax == 1 ? k < nz - 1 : i < nx - 1;
    } else {
        v1 = ax == 0 ? k > 0 : ax == 1 ? i > 0 : j > 0;
        v2 = ax == 0 ? j > 0 : ax == 1 ? k > 0 : i > 0;
    }
    float *lp1 = E ? A.lpe[2 * ax] : A.lph[2 * ax], *lp2 = E ? A.lpe[2 * ax + 1] : A.lph[2 * ax + 1];
    float *w1 = E ? A.we[2 * ax] : A.wh[2 * ax], *w2 = E ? A.we[2 * ax + 1] : A.wh[2 * ax + 1];
    if (v1) {
        float l = lp1[t], w;
        if (E) adj_psi(l, w, A.lf[t1][c], A.ce[t1][c], -1, bcoef, a, km1);
        else adj_psi(l, w, A.lf[3 + t1][c], 0.5f, +1, bcoef, a, km1);
        lp1[t] = l;
        w1[t] = w;
    } else {
        w1[t] = 0.f;
    }
    if (v2) {
        float l = lp2[t], w;
        if (E) adj_psi(l, w, A.lf[t2][c], A.ce[t2][c], +1, bcoef, a, km1);
        else adj_psi(l, w, A.lf[3 + t2][c], 0.5f, -1, bcoef, a, km1);
        lp2[t] = l;
        w2[t] = w;
    } else {
        w2[t] = 0.f;
    }
}

// ---------------------------------------------------------------------------
// Index helpers of the cell kernels, in the index type I of the launch
// (int32_t when every field and psi array has fewer than 2^31 elements):
// dense psi offsets, slab indices of a node, and whether any slab node of an
// axis sits at index x (then the cell takes the CPML terms).
// ---------------------------------------------------------------------------
template <typename I>
__device__ __forceinline__ I psi_x(int ny, int nz, int s, int j, int k) { return ((I)s * ny + j) * nz + k; }
template <typename I>
__device__ __forceinline__ I psi_y(int nz, int P, int i, int s, int k) { return ((I)i * (2 * P) + s) * nz + k; }
template <typename I>
__device__ __forceinline__ I psi_z(int ny, int P, int i, int j, int s) { return ((I)i * ny + j) * (2 * P) + s; }
__device__ __forceinline__ int slab_e(int x, int P, int n, int front, int back) {
    if (P == 0) return -1;
    if (front && x >= 1 && x <= P) return x - 1;
    if (back && x >= n - P - 1 && x <= n - 2) return P + x - (n - P - 1);
    return -1;
}
__device__ __forceinline__ int slab_h(int x, int P, int n, int front, int back) {
    if (P == 0) return -1;
    if (front && x >= 1 && x <= P) return x - 1;
    if (back && x >= n - P && x <= n - 1) return P + x - (n - P);
    return -1;
}
// k_adj_e reads the H nodes x and x+1 and the E node x: front nodes 1..P,
// back H nodes n-P..n-1 and E nodes n-P-1..n-2
__device__ __forceinline__ bool near_e(const Args &A, int a, int x, int n) {
    const int P = A.P[a];
    return P > 0 && ((A.front[a] && x <= P) || (A.back[a] && x >= n - P - 1));
}
// k_adj_h reads the E nodes x-1 and x
__device__ __forceinline__ bool near_h(const Args &A, int a, int x, int n) {
    const int P = A.P[a];
    return P > 0 && ((A.front[a] && x <= P + 1) || (A.back[a] && x >= n - P - 1));
}

// ---------------------------------------------------------------------------
// 2. reverse H part on E cells + gradient.  One thread per cell.  Every load
//    comes first, then the arithmetic, then the stores (a store could alias a
//    later load as far as the compiler knows, and loads placed after stores
//    would wait for them).  Cells with no CPML node skip the slab code.
// ---------------------------------------------------------------------------
template <typename I>
__global__ void __launch_bounds__(kB) k_adj_e(Args A) {
    const int k = blockIdx.x * kB + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    const int nx = (int)A.g.nx, ny = (int)A.g.ny, nz = (int)A.g.nz;
    if (k >= nz) return;
    const I X = (I)A.g.sx, Y = (I)A.g.sy, c = (I)i * X + (I)j * Y + k;
    // E update masks (2nd_order-Yee/Numpy/fdtd3d.py:10-13)
    const bool e0 = j < ny - 1 && k < nz - 1, e1 = i < nx - 1 && k < nz - 1, e2 = i < nx - 1 && j < ny - 1;
    const bool gin = !A.gbox || (i >= A.gb0[0] && i < A.gb1[0] && j >= A.gb0[1] && j < A.gb1[1] &&
                                 k >= A.gb0[2] && k < A.gb1[2]);
    const int Py = A.P[1], Pz = A.P[2];

    // ---- loads
    auto L = [&](const float *f, bool m, I o) { return m ? __ldg(f + c + o) : 0.f; };
    const float *lhx = A.lf[3], *lhy = A.lf[4], *lhz = A.lf[5];
    // adjoint H through the H update masks: the cell, and the +1 neighbours
    // each E component differentiates (loaded only where it is updated)
    const float hz0 = L(lhz, i > 0 && j > 0, 0), hy0 = L(lhy, i > 0 && k > 0, 0), hx0 = L(lhx, j > 0 && k > 0, 0);
    const float hzj = L(lhz, e0 && i > 0, Y), hyk = L(lhy, e0 && i > 0, 1);  // ex
    const float hxk = L(lhx, e1 && j > 0, 1), hzi = L(lhz, e1 && j > 0, X);  // ey
    const float hyi = L(lhy, e2 && k > 0, X), hxj = L(lhx, e2 && k > 0, Y);  // ez
    const float le0 = e0 ? A.lf[0][c] : 0.f, le1 = e1 ? A.lf[1][c] : 0.f, le2 = e2 ? A.lf[2][c] : 0.f;
    // slab nodes: H-node form at this index and one above (the w_h gathers),
    // E-node form at this index (the gradient's psi terms); -1 off the slabs
    int sxh0 = -1, sxh1 = -1, syh0 = -1, syh1 = -1, szh0 = -1, szh1 = -1, sxe = -1, sye = -1, sze = -1;
    // w_h per component, (+) at this index and (-) one above: ex: hzy (y, psi 0
    // of h) and hyz (z, psi 1); ey: hzx (x, psi 1) and hxz (z, psi 0); ez: hyx
    // (x, psi 0) and hxy (y, psi 1)
    float wx0 = 0.f, wx1 = 0.f, wx2 = 0.f, wx3 = 0.f, wy0 = 0.f, wy1 = 0.f, wy2 = 0.f, wy3 = 0.f;
    float wz0 = 0.f, wz1 = 0.f, wz2 = 0.f, wz3 = 0.f;
    if (near_e(A, 0, i, nx) || near_e(A, 1, j, ny) || near_e(A, 2, k, nz)) {
        sxh0 = slab_h(i, A.P[0], nx, A.front[0], A.back[0]);
        sxh1 = slab_h(i + 1, A.P[0], nx, A.front[0], A.back[0]);
        syh0 = slab_h(j, Py, ny, A.front[1], A.back[1]);
        syh1 = slab_h(j + 1, Py, ny, A.front[1], A.back[1]);
        szh0 = slab_h(k, Pz, nz, A.front[2], A.back[2]);
        szh1 = slab_h(k + 1, Pz, nz, A.front[2], A.back[2]);
        sxe = slab_e(i, A.P[0], nx, A.front[0], A.back[0]);
        sye = slab_e(j, Py, ny, A.front[1], A.back[1]);
        sze = slab_e(k, Pz, nz, A.front[2], A.back[2]);
        auto W = [&](int q, bool m, I p) { return m ? __ldg(A.wh[q] + p) : 0.f; };
        if (e0) {
            wx0 = W(2, syh0 >= 0, psi_y<I>(nz, Py, i, syh0, k));
            wx1 = W(2, syh1 >= 0, psi_y<I>(nz, Py, i, syh1, k));
            wx2 = W(5, szh0 >= 0, psi_z<I>(ny, Pz, i, j, szh0));
            wx3 = W(5, szh1 >= 0, psi_z<I>(ny, Pz, i, j, szh1));
        }
        if (e1) {
            wy0 = W(1, sxh0 >= 0, psi_x<I>(ny, nz, sxh0, j, k));
            wy1 = W(1, sxh1 >= 0, psi_x<I>(ny, nz, sxh1, j, k));
            wy2 = W(4, szh0 >= 0, psi_z<I>(ny, Pz, i, j, szh0));
            wy3 = W(4, szh1 >= 0, psi_z<I>(ny, Pz, i, j, szh1));
        }
        if (e2) {
            wz0 = W(0, sxh0 >= 0, psi_x<I>(ny, nz, sxh0, j, k));
            wz1 = W(0, sxh1 >= 0, psi_x<I>(ny, nz, sxh1, j, k));
            wz2 = W(3, syh0 >= 0, psi_y<I>(nz, Py, i, syh0, k));
            wz3 = W(3, syh1 >= 0, psi_y<I>(nz, Py, i, syh1, k));
        }
    }
    // gradient: forward H entering the step (unmasked), forward E-psi, accumulators
    float Hz0 = 0.f, Hzj = 0.f, Hzi = 0.f, Hy0 = 0.f, Hyk = 0.f, Hyi = 0.f, Hx0 = 0.f, Hxk = 0.f, Hxj = 0.f;
    float pe0 = 0.f, pe1 = 0.f, pe2 = 0.f, pe3 = 0.f, pe4 = 0.f, pe5 = 0.f, g0 = 0.f, g1 = 0.f, g2 = 0.f;
    if (gin) {
        const float *hx = A.hp[0], *hy = A.hp[1], *hz = A.hp[2];
        Hz0 = __ldg(hz + c);
        Hy0 = __ldg(hy + c);
        Hx0 = __ldg(hx + c);
        if (e0) {
            Hzj = __ldg(hz + c + Y);
            Hyk = __ldg(hy + c + 1);
            if (sye >= 0) pe3 = __ldg(A.pe[3] + psi_y<I>(nz, Py, i, sye, k));
            if (sze >= 0) pe4 = __ldg(A.pe[4] + psi_z<I>(ny, Pz, i, j, sze));
            g0 = A.gce[0][c];
        }
        if (e1) {
            Hxk = __ldg(hx + c + 1);
            Hzi = __ldg(hz + c + X);
            if (sxe >= 0) pe0 = __ldg(A.pe[0] + psi_x<I>(ny, nz, sxe, j, k));
            if (sze >= 0) pe5 = __ldg(A.pe[5] + psi_z<I>(ny, Pz, i, j, sze));
            g1 = A.gce[1][c];
        }
        if (e2) {
            Hyi = __ldg(hy + c + X);
            Hxj = __ldg(hx + c + Y);
            if (sxe >= 0) pe1 = __ldg(A.pe[1] + psi_x<I>(ny, nz, sxe, j, k));
            if (sye >= 0) pe2 = __ldg(A.pe[2] + psi_y<I>(nz, Py, i, sye, k));
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
// 4. reverse E part on H cells: lH += curl_b(CE*lE) + scatter of w_e.  Loads
//    first, as in k_adj_e; cells with no CPML node skip the slab code.
// ---------------------------------------------------------------------------
template <typename I>
__global__ void __launch_bounds__(kB) k_adj_h(Args A) {
    const int k = blockIdx.x * kB + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    const int nx = (int)A.g.nx, ny = (int)A.g.ny, nz = (int)A.g.nz;
    if (k >= nz) return;
    const I X = (I)A.g.sx, Y = (I)A.g.sy, c = (I)i * X + (I)j * Y + k;
    // H update masks (2nd_order-Yee/Numpy/fdtd3d.py:4-7)
    const bool h0 = j > 0 && k > 0, h1 = i > 0 && k > 0, h2 = i > 0 && j > 0;
    const int Py = A.P[1], Pz = A.P[2];

    // ---- loads
    // nu = CE * lE of component q at offset o, zero outside q's update mask m
    // (loaded only where an H component needs it)
    auto NU = [&](int q, bool need, bool m, I o) {
        return need && m ? fmul(__ldg(A.ce[q] + c + o), __ldg(A.lf[q] + c + o)) : 0.f;
    };
    const bool em0 = j < ny - 1 && k < nz - 1, em1 = i < nx - 1 && k < nz - 1, em2 = i < nx - 1 && j < ny - 1;
    const float n0 = NU(0, h1 || h2, em0, 0), n1 = NU(1, h0 || h2, em1, 0), n2 = NU(2, h0 || h1, em2, 0);
    const float n2j = NU(2, h0, i < nx - 1, -Y), n1k = NU(1, h0, i < nx - 1, -1);  // hx: (i, j-1), (i, k-1)
    const float n0k = NU(0, h1, j < ny - 1, -1), n2i = NU(2, h1, j < ny - 1, -X);  // hy: (k-1), (i-1)
    const float n1i = NU(1, h2, k < nz - 1, -X), n0j = NU(0, h2, k < nz - 1, -Y);  // hz: (i-1), (j-1)
    const float lh0 = h0 ? A.lf[3][c] : 0.f, lh1 = h1 ? A.lf[4][c] : 0.f, lh2 = h2 ? A.lf[5][c] : 0.f;
    // E-node slabs one below and at this index (H cell h: +w at node h-1, -w
    // at node h); -1 off the slabs
    int sx0 = -1, sx1 = -1, sy0 = -1, sy1 = -1, sz0 = -1, sz1 = -1;
    // w_e per component: hx: ezy (y, psi 0 of e) and eyz (z, psi 1); hy: ezx
    // (x, psi 1) and exz (z, psi 0); hz: eyx (x, psi 0) and exy (y, psi 1)
    float wx0 = 0.f, wx1 = 0.f, wx2 = 0.f, wx3 = 0.f, wy0 = 0.f, wy1 = 0.f, wy2 = 0.f, wy3 = 0.f;
    float wz0 = 0.f, wz1 = 0.f, wz2 = 0.f, wz3 = 0.f;
    if (near_h(A, 0, i, nx) || near_h(A, 1, j, ny) || near_h(A, 2, k, nz)) {
        sx0 = slab_e(i - 1, A.P[0], nx, A.front[0], A.back[0]);
        sx1 = slab_e(i, A.P[0], nx, A.front[0], A.back[0]);
        sy0 = slab_e(j - 1, Py, ny, A.front[1], A.back[1]);
        sy1 = slab_e(j, Py, ny, A.front[1], A.back[1]);
        sz0 = slab_e(k - 1, Pz, nz, A.front[2], A.back[2]);
        sz1 = slab_e(k, Pz, nz, A.front[2], A.back[2]);
        auto W = [&](int q, bool m, I p) { return m ? __ldg(A.we[q] + p) : 0.f; };
        if (h0) {
            wx0 = W(2, sy0 >= 0, psi_y<I>(nz, Py, i, sy0, k));
            wx1 = W(2, sy1 >= 0, psi_y<I>(nz, Py, i, sy1, k));
            wx2 = W(5, sz0 >= 0, psi_z<I>(ny, Pz, i, j, sz0));
            wx3 = W(5, sz1 >= 0, psi_z<I>(ny, Pz, i, j, sz1));
        }
        if (h1) {
            wy0 = W(1, sx0 >= 0, psi_x<I>(ny, nz, sx0, j, k));
            wy1 = W(1, sx1 >= 0, psi_x<I>(ny, nz, sx1, j, k));
            wy2 = W(4, sz0 >= 0, psi_z<I>(ny, Pz, i, j, sz0));
            wy3 = W(4, sz1 >= 0, psi_z<I>(ny, Pz, i, j, sz1));
        }
        if (h2) {
            wz0 = W(0, sx0 >= 0, psi_x<I>(ny, nz, sx0, j, k));
            wz1 = W(0, sx1 >= 0, psi_x<I>(ny, nz, sx1, j, k));
            wz2 = W(3, sy0 >= 0, psi_y<I>(nz, Py, i, sy0, k));
            wz3 = W(3, sy1 >= 0, psi_y<I>(nz, Py, i, sy1, k));
        }
    }

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
    // 32-bit offsets in the kernels when every field and psi array has fewer
    // than 2^31 elements
    int64_t most = g.nx * g.sx;
    PsiBlocks R{};
    for (int a = 0; a < 3; a++) {
        const int64_t np = 2 * (int64_t)A.P[a] * (n[0] * n[1] * n[2] / n[a]);
        most = std::max(most, np);
        const int64_t nb = (a ? R.nb[a - 1] : 0) + (np + kB - 1) / kB;
        if (nb >= ((int64_t)1 << 31)) return FDTD_ERR_UNSUPPORTED;
        R.nb[a] = (int32_t)nb;
    }
    const bool i32 = most < ((int64_t)1 << 31);
    if (R.nb[2] > 0) {
        if (i32) k_adj_psi3<false, int32_t><<<R.nb[2], kB, 0, st>>>(A, R);
        else k_adj_psi3<false, int64_t><<<R.nb[2], kB, 0, st>>>(A, R);
    }
    if (i32) k_adj_e<int32_t><<<cells(g), kB, 0, st>>>(A);
    else k_adj_e<int64_t><<<cells(g), kB, 0, st>>>(A);
    if (R.nb[2] > 0) {
        if (i32) k_adj_psi3<true, int32_t><<<R.nb[2], kB, 0, st>>>(A, R);
        else k_adj_psi3<true, int64_t><<<R.nb[2], kB, 0, st>>>(A, R);
    }
    if (i32) k_adj_h<int32_t><<<cells(g), kB, 0, st>>>(A);
    else k_adj_h<int64_t><<<cells(g), kB, 0, st>>>(A);
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
