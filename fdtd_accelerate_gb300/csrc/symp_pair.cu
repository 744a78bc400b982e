// Fused 4th-order symplectic stage pair: one H stage (or two in a row) and the
// following E stage, with their stage-wise CPML terms and the soft sources
// after the E stage, in ONE pass over HBM (sm_103a, TMA + mbarrier pipeline).
//
// Semantics are those of the in-place stage sequence of
// 4th_order-Symplectic/PyCUDA/100-base.py:124-141 (stencil and index ranges
// :17-43, operation grouping Python-C/dielectric.c:35-89), i.e. of
//   fdtd_symplectic_stage_f32(H, cl_a) [, fdtd_symplectic_stage_f32(H, cl_b)],
//   fdtd_symplectic_stage_f32(E, dl), sources,
// with the same round-to-nearest operations, so the result is bit-identical.
//
// Design
//  * Ping-pong state: the pass reads buffer `cur` (E, H) and writes `1-cur`;
//    the H psi slabs ping-pong too (halo H cells are recomputed from the
//    input psi), the E psi slabs are updated in place (only their owner
//    touches them).
//  * A CTA owns TZ = 32 (z, one cell per lane) x TY = 16 (y) cells for a chunk
//    of x planes and marches along x.  E_new(i) needs H_new on planes
//    i-1 .. i+2 and rows/columns -1 .. +2 around the tile; H_new(m) needs the
//    input E on planes m-2 .. m+1 and rows/columns -2 .. +1 around those.
//    So plane p of the input arrives (3-D TMA boxes: E with a 3-row, 4-column
//    halo, H with a 1-row halo, CE on the tile) and the CTA computes H_new(p-1)
//    on (TY+3) x (TZ+3) cells into a 4-plane ring in shared memory, then
//    E_new(p-3) on the tile.  Own H_new and E_new are stored as computed.
//  * Lane 0 of the last warp is the producer: it waits on the mbarriers and
//    issues every copy two iterations ahead.  Every wait is bounded (1 s);
//    on expiry the CTA records FDTD_ERR_TIMEOUT, drains its copies and stops.
#include <cuda.h>

#include <algorithm>
#include <vector>

#include "common.cuh"

namespace fdtd {
namespace sp {

constexpr int TZ = 32, TY = 16;
constexpr int BW = TZ + 8;          // box width: k0-4 .. k0+TZ+3
constexpr int ER = TY + 6;          // E box rows: j0-3 .. j0+TY+2
constexpr int HOR = TY + 3;         // H box rows: j0-1 .. j0+TY+1
constexpr int HNR = TY + 3;         // H_new rows: j0-1 .. j0+TY+1
constexpr int HNC = TZ + 3;         // H_new columns: k0-1 .. k0+TZ+1
constexpr int HNP = 36;             // H_new row pitch
constexpr int NE = 6, NH = 3, NC = 3, NHN = 4;  // ring depths (E, H, CE inputs; H_new)
constexpr int NCW = (HNR * HNC + 31) / 32;      // compute warps: one H_new cell per thread
constexpr int THREADS = (NCW + 1) * 32;         // + the producer warp
constexpr int MAX_SRC = 64;                     // sources per work item
constexpr uint64_t WAIT_NS = 1000000000ull;

constexpr int al128(int b) { return (b + 127) / 128 * 128; }
constexpr int EBOXB = al128(ER * BW * 4), HBOXB = al128(HOR * BW * 4), CBOXB = al128(TY * TZ * 4);
constexpr int HNB = al128(HNR * HNP * 4);
constexpr int OFF_E = 0;
constexpr int OFF_H = OFF_E + NE * 3 * EBOXB;
constexpr int OFF_C = OFF_H + NH * 3 * HBOXB;
constexpr int OFF_HN = OFF_C + NC * 3 * CBOXB;
constexpr int OFF_BAR = OFF_HN + NHN * 3 * HNB;
constexpr int SMEM = OFF_BAR + 128 + 128 /*align slack*/;
static_assert((NE + NH + NC) * 8 <= 128, "the mbarriers live in 128 bytes");

struct Maps {
    CUtensorMap e[3];   // ex, ey, ez of the input buffer, box (BW, ER, 1)
    CUtensorMap h[3];   // hx, hy, hz of the input buffer, box (BW, HOR, 1)
    CUtensorMap ce[3];  // cex, cey, cez, box (TZ, TY, 1)
};

struct Axis {
    int32_t P, front, back;
    const float *b, *a, *km1;  // tables of one stage (E tables for the E stage, H for H)
};

struct Params {
    int32_t nx, ny, nz;
    uint32_t sx, sy;
    int32_t ntz, nty, nxc, x_chunk;
    float *out[6];           // ex, ey, ez, hx, hy, hz of the output buffer
    const float *psi_h_in[6];
    float *psi_h_out[6];
    float *psi_e[6];         // in place
    Axis ha[3], hb[3], ea[3];  // CPML of H stage a, H stage b, E stage
    float cl_a, cl_b, dl, ch;
    float clch_a, clch_b;     // cl * ch as one single-precision product
    int32_t hh;               // 1: two H stages (a then b) before the E stage
    int32_t cpml;             // any slab
    int32_t nsrc;
    const int32_t *src_ijk, *src_comp;
    const float *src_amp;
    int64_t namp, t;          // amplitude table length and the index used
    int32_t *status;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t gtimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
// true on completion; false after WAIT_NS or once another CTA recorded a timeout
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, const int32_t *status) {
    if (mbar_try(bar, parity)) return true;
    const uint64_t t0 = gtimer();
    for (uint32_t n = 1;; n++) {
        if (mbar_try(bar, parity)) return true;
        if ((n & 255) == 0) {
            if (gtimer() - t0 > WAIT_NS) return false;
            if (status && *(volatile const int32_t *)status == FDTD_ERR_TIMEOUT) return false;
        }
    }
}
__device__ __forceinline__ void tma3(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1, int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

// slab index of a node along one axis (E or H nodes of a stage), -1 outside
__device__ __forceinline__ int slab(const Axis &A, int x, int n, bool e) {
    if (A.P <= 0) return -1;
    if (A.front && x >= 1 && x <= A.P) return x - 1;
    const int b0 = e ? n - A.P - 1 : n - A.P, b1 = e ? n - 2 : n - 1;
    if (A.back && x >= b0 && x <= b1) return A.P + x - b0;
    return -1;
}
// psi element of slab s along ax at (i, j, k)
__device__ __forceinline__ uint32_t psi_index(const Params &p, int ax, int s, int i, int j, int k, int P) {
    const uint32_t twoP = 2u * (uint32_t)P;
    return ax == 0 ? ((uint32_t)s * p.ny + j) * p.nz + k
                   : (ax == 1 ? ((uint32_t)i * twoP + s) * p.nz + k : ((uint32_t)i * p.ny + j) * twoP + s);
}
// psi <- b psi + a d; returns (coef * cv) * (km1 d + psi)
__device__ __forceinline__ float sterm(const Axis &A, int s, float &psi, float d, float coef, float cv) {
    psi = fadd(fmul(A.b[s], psi), fmul(A.a[s], d));
    return fmul(fmul(coef, cv), fadd(fmul(A.km1[s], d), psi));
}

__global__ void __launch_bounds__(THREADS, 1)
k_symp_pair(const __grid_constant__ Maps mk, const __grid_constant__ Params p) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem =
        reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + OFF_BAR);  // E[NE], H[NH], CE[NC]
    auto sE = [&](int sl, int c) { return reinterpret_cast<float *>(smem + OFF_E + (sl * 3 + c) * EBOXB); };
    auto sH = [&](int sl, int c) { return reinterpret_cast<float *>(smem + OFF_H + (sl * 3 + c) * HBOXB); };
    auto sC = [&](int sl, int c) { return reinterpret_cast<float *>(smem + OFF_C + (sl * 3 + c) * CBOXB); };
    auto sN = [&](int sl, int c) { return reinterpret_cast<float *>(smem + OFF_HN + (sl * 3 + c) * HNB); };
    __shared__ int s_abort, s_nls;
    __shared__ int s_ls_i[MAX_SRC], s_ls_j[MAX_SRC], s_ls_kc[MAX_SRC], s_ls_s[MAX_SRC];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool producer = tid == NCW * 32;
    if (tid == 0) {
        for (int s = 0; s < NE + NH + NC; s++) mbar_init(&bars[s]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        s_abort = 0;
    }
    // H_new cell of this thread (flat index over HNR x HNC) and E cell (warps 0..TY-1)
    const int hf = tid, hr = hf / HNC, hc = hf - hr * HNC;
    const bool h_thread = hf < HNR * HNC;
    const bool e_thread = warp < TY;

    uint32_t gE = 0, gH = 0, gC = 0;  // planes issued on each ring before the current item
    bool aborted = false;
    int64_t q_abort = 0, Q_abort = 0;
    const int64_t nitems = (int64_t)p.ntz * p.nty * p.nxc;
    for (int64_t item = blockIdx.x; item < nitems && !aborted; item += gridDim.x) {
        const int tzi = (int)(item % p.ntz), tyi = (int)((item / p.ntz) % p.nty);
        const int xci = (int)(item / ((int64_t)p.ntz * p.nty));
        const int k0 = tzi * TZ, j0 = tyi * TY, x0 = xci * p.x_chunk;
        const int x1 = min(x0 + p.x_chunk, p.nx);
        // iteration q: input plane p = x0 - 3 + q arrives; H_new(p-1) for
        // q >= 3, E_new(p-3) for q >= 6
        const int Q = x1 - x0 + 6;
        // ring uses: E at every iteration, H from iteration 3, CE from iteration 6;
        // u-th use of a ring lands in slot u % depth and completes phase (u / depth) & 1
        auto eslot = [&](int q) { return (int)((gE + (uint32_t)q) % NE); };
        auto hslot = [&](int q) { return (int)((gH + (uint32_t)(q - 3)) % NH); };
        auto cslot = [&](int q) { return (int)((gC + (uint32_t)(q - 6)) % NC); };
        auto ephase = [&](int q) { return ((gE + (uint32_t)q) / NE) & 1; };
        auto hphase = [&](int q) { return ((gH + (uint32_t)(q - 3)) / NH) & 1; };
        auto cphase = [&](int q) { return ((gC + (uint32_t)(q - 6)) / NC) & 1; };
        // copies needed at iteration q (issued two iterations ahead)
        auto issue = [&](int q) {
            const int pl = x0 - 3 + q;
            {   // E(p)
                const int sl = eslot(q);
                uint64_t *bar = &bars[sl];
                mbar_expect(bar, 3u * ER * BW * 4);
                for (int c = 0; c < 3; c++) tma3(sE(sl, c), &mk.e[c], bar, k0 - 4, j0 - 3, pl);
            }
            if (q >= 3) {  // H(p-1)
                const int sl = hslot(q);
                uint64_t *bar = &bars[NE + sl];
                mbar_expect(bar, 3u * HOR * BW * 4);
                for (int c = 0; c < 3; c++) tma3(sH(sl, c), &mk.h[c], bar, k0 - 4, j0 - 1, pl - 1);
            }
            if (q >= 6) {  // CE(p-3)
                const int sl = cslot(q);
                uint64_t *bar = &bars[NE + NH + sl];
                mbar_expect(bar, 3u * TY * TZ * 4);
                for (int c = 0; c < 3; c++) tma3(sC(sl, c), &mk.ce[c], bar, k0, j0, pl - 3);
            }
        };
        if (tid == 0) {  // sources of this item's tile, list order
            int n = 0;
            if (p.t >= 0 && p.t < p.namp)
                for (int s = 0; s < p.nsrc; s++) {
                    const int si = p.src_ijk[3 * s], sj = p.src_ijk[3 * s + 1], sk = p.src_ijk[3 * s + 2];
                    if (si >= x0 && si < x1 && sj >= j0 && sj < j0 + TY && sk >= k0 && sk < k0 + TZ) {
                        if (n < MAX_SRC) {
                            s_ls_i[n] = si;
                            s_ls_j[n] = sj;
                            s_ls_kc[n] = (sk << 2) | p.src_comp[s];
                            s_ls_s[n] = s;
                        }
                        n++;
                    }
                }
            if (n > MAX_SRC) {  // the host rejects such layouts; never drop a source silently
                atomicExch(p.status, FDTD_ERR_CAPACITY);
                n = MAX_SRC;
            }
            s_nls = n;
        }
        __syncthreads();  // previous item finished everywhere; source list ready
        if (producer) {
            issue(0);
            if (Q > 1) issue(1);
        }
        const int nls = s_nls;
        for (int q = 0; q < Q; q++) {
            const int pl = x0 - 3 + q;
            const int eS = eslot(q), hS = q >= 3 ? hslot(q) : 0, cS = q >= 6 ? cslot(q) : 0;
            if (producer) {
                bool ok = mbar_wait(&bars[eS], ephase(q), p.status);
                if (ok && q >= 3) ok = mbar_wait(&bars[NE + hS], hphase(q), p.status);
                if (ok && q >= 6) ok = mbar_wait(&bars[NE + NH + cS], cphase(q), p.status);
                if (!ok) s_abort = 1;
            }
            __syncthreads();  // (A) copies of iteration q visible; iteration q-1 done everywhere
            if (s_abort) {
                aborted = true;
                q_abort = q;
                Q_abort = Q;
                break;
            }
            if (producer && q + 2 < Q) issue(q + 2);

            // ---- H_new(m), m = p - 1: (TY+3) x (TZ+3) cells around the tile ----
            const int m = pl - 1;
            if (q >= 3 && h_thread && m >= 0 && m < p.nx) {
                const int j = j0 - 1 + hr, k = k0 - 1 + hc;
                if (j >= 0 && j < p.ny && k >= 0 && k < p.nz) {
                    // E slots of planes m-2 .. m+1 (iterations q-3 .. q)
                    const float *E0[3], *Em1[3], *Em2[3], *Ep1[3];
                    for (int c = 0; c < 3; c++) {
                        E0[c] = sE(eslot(q - 1), c);
                        Em1[c] = sE(eslot(q - 2), c);
                        Em2[c] = sE(eslot(q - 3), c);
                        Ep1[c] = sE(eS, c);
                    }
                    const int e = (hr + 2) * BW + hc + 3;  // E box: row j0-3+r, column k0-4+c
                    const int hb = hr * BW + hc + 3;       // H box: row j0-1+r
                    const float *ex = E0[0], *ey = E0[1], *ez = E0[2];
                    const float hx0 = sH(hS, 0)[hb], hy0 = sH(hS, 1)[hb], hz0 = sH(hS, 2)[hb];
                    const bool jin = j > 1 && j < p.ny - 1, kin = k > 1 && k < p.nz - 1, iin = m > 1 && m < p.nx - 1;
                    const bool own = hr >= 1 && hr <= TY && hc >= 1 && hc <= TZ && m >= x0 && m < x1;
                    int sx = -1, sy = -1, sz = -1;
                    if (p.cpml) {
                        sx = slab(p.ha[0], m, p.nx, false);
                        sy = slab(p.ha[1], j, p.ny, false);
                        sz = slab(p.ha[2], k, p.nz, false);
                    }
                    const int nst = p.hh ? 2 : 1;
                    float vx = hx0, vy = hy0, vz = hz0;
                    // the stage's differences do not change between the two H stages
                    if (jin && kin) {
                        const float n = curl4(ez[e], ez[e - BW], ey[e], ey[e - 1]);
                        const float f = curl4(ez[e + BW], ez[e - 2 * BW], ey[e + 1], ey[e - 2]);
                        const float d27 = fsub(fmul(27.0f, n), f);
                        const float dy = sy >= 0 ? fsub(fmul(27.0f, fsub(ez[e], ez[e - BW])), fsub(ez[e + BW], ez[e - 2 * BW])) : 0.f;
                        const float dz = sz >= 0 ? fsub(fmul(27.0f, fsub(ey[e], ey[e - 1])), fsub(ey[e + 1], ey[e - 2])) : 0.f;
                        float py = 0.f, pz = 0.f;
                        const uint32_t qy = sy >= 0 ? psi_index(p, 1, sy, m, j, k, p.ha[1].P) : 0u;
                        const uint32_t qz = sz >= 0 ? psi_index(p, 2, sz, m, j, k, p.ha[2].P) : 0u;
                        if (sy >= 0) py = p.psi_h_in[3][qy];
                        if (sz >= 0) pz = p.psi_h_in[4][qz];
                        for (int st = 0; st < nst; st++) {
                            const float cl = st ? p.cl_b : p.cl_a, clch = st ? p.clch_b : p.clch_a;
                            const Axis *A = st ? p.hb : p.ha;
                            vx = fsub(vx, fmul(clch, d27));
                            if (sy >= 0) vx = fsub(vx, sterm(A[1], sy, py, dy, cl, p.ch));
                            if (sz >= 0) vx = fadd(vx, sterm(A[2], sz, pz, dz, cl, p.ch));
                        }
                        if (own && sy >= 0) p.psi_h_out[3][qy] = py;
                        if (own && sz >= 0) p.psi_h_out[4][qz] = pz;
                    }
                    if (iin && kin) {
                        const float n = curl4(ex[e], ex[e - 1], ez[e], Em1[2][e]);
                        const float f = curl4(ex[e + 1], ex[e - 2], Ep1[2][e], Em2[2][e]);
                        const float d27 = fsub(fmul(27.0f, n), f);
                        const float dx = sx >= 0 ? fsub(fmul(27.0f, fsub(ez[e], Em1[2][e])), fsub(Ep1[2][e], Em2[2][e])) : 0.f;
                        const float dz = sz >= 0 ? fsub(fmul(27.0f, fsub(ex[e], ex[e - 1])), fsub(ex[e + 1], ex[e - 2])) : 0.f;
                        float px = 0.f, pz = 0.f;
                        const uint32_t qx = sx >= 0 ? psi_index(p, 0, sx, m, j, k, p.ha[0].P) : 0u;
                        const uint32_t qz = sz >= 0 ? psi_index(p, 2, sz, m, j, k, p.ha[2].P) : 0u;
                        if (sx >= 0) px = p.psi_h_in[0][qx];
                        if (sz >= 0) pz = p.psi_h_in[5][qz];
                        for (int st = 0; st < nst; st++) {
                            const float cl = st ? p.cl_b : p.cl_a, clch = st ? p.clch_b : p.clch_a;
                            const Axis *A = st ? p.hb : p.ha;
                            vy = fsub(vy, fmul(clch, d27));
                            if (sx >= 0) vy = fadd(vy, sterm(A[0], sx, px, dx, cl, p.ch));
                            if (sz >= 0) vy = fsub(vy, sterm(A[2], sz, pz, dz, cl, p.ch));
                        }
                        if (own && sx >= 0) p.psi_h_out[0][qx] = px;
                        if (own && sz >= 0) p.psi_h_out[5][qz] = pz;
                    }
                    if (iin && jin) {
                        const float n = curl4(ey[e], Em1[1][e], ex[e], ex[e - BW]);
                        const float f = curl4(Ep1[1][e], Em2[1][e], ex[e + BW], ex[e - 2 * BW]);
                        const float d27 = fsub(fmul(27.0f, n), f);
                        const float dx = sx >= 0 ? fsub(fmul(27.0f, fsub(ey[e], Em1[1][e])), fsub(Ep1[1][e], Em2[1][e])) : 0.f;
                        const float dy = sy >= 0 ? fsub(fmul(27.0f, fsub(ex[e], ex[e - BW])), fsub(ex[e + BW], ex[e - 2 * BW])) : 0.f;
                        float px = 0.f, py = 0.f;
                        const uint32_t qx = sx >= 0 ? psi_index(p, 0, sx, m, j, k, p.ha[0].P) : 0u;
                        const uint32_t qy = sy >= 0 ? psi_index(p, 1, sy, m, j, k, p.ha[1].P) : 0u;
                        if (sx >= 0) px = p.psi_h_in[1][qx];
                        if (sy >= 0) py = p.psi_h_in[2][qy];
                        for (int st = 0; st < nst; st++) {
                            const float cl = st ? p.cl_b : p.cl_a, clch = st ? p.clch_b : p.clch_a;
                            const Axis *A = st ? p.hb : p.ha;
                            vz = fsub(vz, fmul(clch, d27));
                            if (sx >= 0) vz = fsub(vz, sterm(A[0], sx, px, dx, cl, p.ch));
                            if (sy >= 0) vz = fadd(vz, sterm(A[1], sy, py, dy, cl, p.ch));
                        }
                        if (own && sx >= 0) p.psi_h_out[1][qx] = px;
                        if (own && sy >= 0) p.psi_h_out[2][qy] = py;
                    }
                    const int nsl = (int)((uint32_t)(m - (x0 - 4)) % NHN);  // ring slot of plane m
                    const int no = hr * HNP + hc;
                    sN(nsl, 0)[no] = vx;
                    sN(nsl, 1)[no] = vy;
                    sN(nsl, 2)[no] = vz;
                    if (own) {
                        const uint32_t g = (uint32_t)m * p.sx + (uint32_t)j * p.sy + k;
                        p.out[3][g] = vx;
                        p.out[4][g] = vy;
                        p.out[5][g] = vz;
                    }
                }
            }
            __syncthreads();  // (B) H_new(p-1) visible

            // ---- E_new(i), i = p - 3, on the tile ----
            const int i = pl - 3;
            if (q >= 6 && e_thread) {
                const int r = warp, j = j0 + r, k = k0 + lane;
                if (j < p.ny && k < p.nz) {
                    const float *N0[3], *Nm1[3], *Np1[3], *Np2[3];
                    for (int c = 0; c < 3; c++) {
                        N0[c] = sN((int)((uint32_t)(i - (x0 - 4)) % NHN), c);
                        Nm1[c] = sN((int)((uint32_t)(i - 1 - (x0 - 4)) % NHN), c);
                        Np1[c] = sN((int)((uint32_t)(i + 1 - (x0 - 4)) % NHN), c);
                        Np2[c] = sN((int)((uint32_t)(i + 2 - (x0 - 4)) % NHN), c);
                    }
                    const int h = (r + 1) * HNP + lane + 1;   // H_new: row j0-1+r', column k0-1+c'
                    const int e = (r + 3) * BW + lane + 4;    // E box of plane i
                    const int ce = r * TZ + lane;
                    const int eS3 = eslot(q - 3);
                    const float *hx = N0[0], *hy = N0[1], *hz = N0[2];
                    float vx = sE(eS3, 0)[e], vy = sE(eS3, 1)[e], vz = sE(eS3, 2)[e];
                    const bool jin = j > 0 && j < p.ny - 2, kin = k > 0 && k < p.nz - 2, iin = i > 0 && i < p.nx - 2;
                    int sx = -1, sy = -1, sz = -1;
                    if (p.cpml) {
                        sx = slab(p.ea[0], i, p.nx, true);
                        sy = slab(p.ea[1], j, p.ny, true);
                        sz = slab(p.ea[2], k, p.nz, true);
                    }
                    if (jin && kin) {
                        const float n = curl4(hz[h + HNP], hz[h], hy[h + 1], hy[h]);
                        const float f = curl4(hz[h + 2 * HNP], hz[h - HNP], hy[h + 2], hy[h - 1]);
                        const float cv = sC(cS, 0)[ce];
                        vx = fadd(vx, fmul(fmul(p.dl, cv), fsub(fmul(27.0f, n), f)));
                        if (sy >= 0) {
                            const uint32_t qi = psi_index(p, 1, sy, i, j, k, p.ea[1].P);
                            float ps = p.psi_e[3][qi];
                            const float d = fsub(fmul(27.0f, fsub(hz[h + HNP], hz[h])), fsub(hz[h + 2 * HNP], hz[h - HNP]));
                            vx = fadd(vx, sterm(p.ea[1], sy, ps, d, p.dl, cv));
                            p.psi_e[3][qi] = ps;
                        }
                        if (sz >= 0) {
                            const uint32_t qi = psi_index(p, 2, sz, i, j, k, p.ea[2].P);
                            float ps = p.psi_e[4][qi];
                            const float d = fsub(fmul(27.0f, fsub(hy[h + 1], hy[h])), fsub(hy[h + 2], hy[h - 1]));
                            vx = fsub(vx, sterm(p.ea[2], sz, ps, d, p.dl, cv));
                            p.psi_e[4][qi] = ps;
                        }
                    }
                    if (iin && kin) {
                        const float n = curl4(hx[h + 1], hx[h], Np1[2][h], hz[h]);
                        const float f = curl4(hx[h + 2], hx[h - 1], Np2[2][h], Nm1[2][h]);
                        const float cv = sC(cS, 1)[ce];
                        vy = fadd(vy, fmul(fmul(p.dl, cv), fsub(fmul(27.0f, n), f)));
                        if (sx >= 0) {
                            const uint32_t qi = psi_index(p, 0, sx, i, j, k, p.ea[0].P);
                            float ps = p.psi_e[0][qi];
                            const float d = fsub(fmul(27.0f, fsub(Np1[2][h], hz[h])), fsub(Np2[2][h], Nm1[2][h]));
                            vy = fsub(vy, sterm(p.ea[0], sx, ps, d, p.dl, cv));
                            p.psi_e[0][qi] = ps;
                        }
                        if (sz >= 0) {
                            const uint32_t qi = psi_index(p, 2, sz, i, j, k, p.ea[2].P);
                            float ps = p.psi_e[5][qi];
                            const float d = fsub(fmul(27.0f, fsub(hx[h + 1], hx[h])), fsub(hx[h + 2], hx[h - 1]));
                            vy = fadd(vy, sterm(p.ea[2], sz, ps, d, p.dl, cv));
                            p.psi_e[5][qi] = ps;
                        }
                    }
                    if (iin && jin) {
                        const float n = curl4(Np1[1][h], hy[h], hx[h + HNP], hx[h]);
                        const float f = curl4(Np2[1][h], Nm1[1][h], hx[h + 2 * HNP], hx[h - HNP]);
                        const float cv = sC(cS, 2)[ce];
                        vz = fadd(vz, fmul(fmul(p.dl, cv), fsub(fmul(27.0f, n), f)));
                        if (sx >= 0) {
                            const uint32_t qi = psi_index(p, 0, sx, i, j, k, p.ea[0].P);
                            float ps = p.psi_e[1][qi];
                            const float d = fsub(fmul(27.0f, fsub(Np1[1][h], hy[h])), fsub(Np2[1][h], Nm1[1][h]));
                            vz = fadd(vz, sterm(p.ea[0], sx, ps, d, p.dl, cv));
                            p.psi_e[1][qi] = ps;
                        }
                        if (sy >= 0) {
                            const uint32_t qi = psi_index(p, 1, sy, i, j, k, p.ea[1].P);
                            float ps = p.psi_e[2][qi];
                            const float d = fsub(fmul(27.0f, fsub(hx[h + HNP], hx[h])), fsub(hx[h + 2 * HNP], hx[h - HNP]));
                            vz = fsub(vz, sterm(p.ea[1], sy, ps, d, p.dl, cv));
                            p.psi_e[2][qi] = ps;
                        }
                    }
                    for (int s = 0; s < nls; s++) {  // soft sources, list order
                        if (s_ls_i[s] != i || s_ls_j[s] != j || (s_ls_kc[s] >> 2) != k) continue;
                        const float v = p.src_amp[(int64_t)s_ls_s[s] * p.namp + p.t];
                        const int comp = s_ls_kc[s] & 3;
                        if (comp == 0) vx = fadd(vx, v);
                        else if (comp == 1) vy = fadd(vy, v);
                        else vz = fadd(vz, v);
                    }
                    const uint32_t g = (uint32_t)i * p.sx + (uint32_t)j * p.sy + k;
                    p.out[0][g] = vx;
                    p.out[1][g] = vy;
                    p.out[2][g] = vz;
                }
            }
        }
        if (aborted) {
            if (producer) {
                atomicExch(p.status, FDTD_ERR_TIMEOUT);
                // let the copies in flight (iterations q and q+1) land before the
                // shared memory is released; each wait bounded
                for (int64_t q = q_abort; q < Q_abort && q < q_abort + 2; q++) {
                    const int qq = (int)q;
                    mbar_wait(&bars[eslot(qq)], ephase(qq), nullptr);
                    if (qq >= 3) mbar_wait(&bars[NE + hslot(qq)], hphase(qq), nullptr);
                    if (qq >= 6) mbar_wait(&bars[NE + NH + cslot(qq)], cphase(qq), nullptr);
                }
            }
            break;
        }
        gE += (uint32_t)Q;
        gH += (uint32_t)(Q - 3);
        gC += (uint32_t)(Q - 6);
    }
    if (aborted) __syncthreads();
}

}  // namespace sp
}  // namespace fdtd

using namespace fdtd;
using namespace fdtd::sp;

typedef CUresult (*EncodeFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                             const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                             CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeFn encode_fn() {
    static EncodeFn fn = nullptr;
    if (!fn) {
        void *ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        fn = reinterpret_cast<EncodeFn>(ptr);
    }
    return fn;
}

static int map3(EncodeFn enc, CUtensorMap *m, const float *ptr, const Grid &g, int bz, int by) {
    cuuint64_t dims[3] = {(cuuint64_t)g.nz, (cuuint64_t)g.ny, (cuuint64_t)g.nx};
    cuuint64_t strides[2] = {(cuuint64_t)g.sy * 4, (cuuint64_t)g.sx * 4};
    cuuint32_t box[3] = {(cuuint32_t)bz, (cuuint32_t)by, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(ptr), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? FDTD_OK : FDTD_ERR_CUDA;
}

struct fdtd_symp_plan {
    Grid g;
    Maps maps[2];
    Params base;
    float *f[2][6];
    const float *psi_h[2][6];
    int nblocks;
    int cur;
};

extern "C" {

int fdtd_symp_pair_plan_create(fdtd_symp_plan **out, const fdtd_grid *gp, const fdtd_symp_state *s,
                               const fdtd_sources *src, int32_t x_chunk, int32_t cur, int32_t *status_dev,
                               void *stream) {
    if (!out || !s || !status_dev || (cur != 0 && cur != 1)) return FDTD_ERR_ARG;
    *out = nullptr;
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (g.nx < 4 || g.ny < 4 || g.nz < 4) return FDTD_ERR_SHAPE;
    if ((g.sx & 3) || (g.sy & 3)) return FDTD_ERR_ALIGN;
    if (g.nx * g.sx >= ((int64_t)1 << 31)) return FDTD_ERR_UNSUPPORTED;  // 32-bit offsets
    auto a16 = [](const void *q) { return (reinterpret_cast<uintptr_t>(q) & 15) == 0; };
    for (int b = 0; b < 2; b++)
        for (int q = 0; q < 6; q++)
            if (!s->f[b][q] || !a16(s->f[b][q])) return s->f[b][q] ? FDTD_ERR_ALIGN : FDTD_ERR_ARG;
    for (int q = 0; q < 3; q++)
        if (!s->ce[q] || !a16(s->ce[q])) return s->ce[q] ? FDTD_ERR_ALIGN : FDTD_ERR_ARG;
    fdtd_symp_plan *pl = new fdtd_symp_plan();
    pl->g = g;
    pl->cur = cur;
    Params &p = pl->base;
    p = Params{};
    p.nx = (int32_t)g.nx; p.ny = (int32_t)g.ny; p.nz = (int32_t)g.nz;
    p.sx = (uint32_t)g.sx; p.sy = (uint32_t)g.sy;
    p.ntz = (int32_t)((g.nz + TZ - 1) / TZ);
    p.nty = (int32_t)((g.ny + TY - 1) / TY);
    if (x_chunk < 0) { delete pl; return FDTD_ERR_ARG; }
    p.x_chunk = (int32_t)std::min<int64_t>(x_chunk > 0 ? x_chunk : 128, g.nx);
    p.nxc = (int32_t)((g.nx + p.x_chunk - 1) / p.x_chunk);
    p.status = status_dev;
    for (int b = 0; b < 2; b++)
        for (int q = 0; q < 6; q++) {
            pl->f[b][q] = s->f[b][q];
            pl->psi_h[b][q] = s->psi_h[b][q];
        }
    for (int q = 0; q < 6; q++) p.psi_e[q] = s->psi_e[q];
    if (src && src->nsrc > 0) {
        if (!all_nonnull(src->ijk, src->comp, src->amp) || src->namp < 0) { delete pl; return FDTD_ERR_ARG; }
        p.nsrc = src->nsrc; p.src_ijk = src->ijk; p.src_comp = src->comp; p.src_amp = src->amp; p.namp = src->namp;
        // capacity: sources per tile (positions read on the caller's stream)
        std::vector<int32_t> h((size_t)3 * src->nsrc);
        cudaError_t e = cudaMemcpyAsync(h.data(), src->ijk, h.size() * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                        as_stream(stream));
        if (e == cudaSuccess) e = cudaStreamSynchronize(as_stream(stream));
        if (e != cudaSuccess) { set_cuda_error(e); delete pl; return FDTD_ERR_CUDA; }
        std::vector<int> count((size_t)p.ntz * p.nty * p.nxc, 0);
        for (int a = 0; a < src->nsrc; a++) {
            const int64_t si = h[3 * a], sj = h[3 * a + 1], sk = h[3 * a + 2];
            if (si < 0 || si >= g.nx || sj < 0 || sj >= g.ny || sk < 0 || sk >= g.nz) { delete pl; return FDTD_ERR_ARG; }
            const int64_t it = ((si / p.x_chunk) * p.nty + sj / TY) * p.ntz + sk / TZ;
            if (++count[it] > MAX_SRC) { delete pl; return FDTD_ERR_CAPACITY; }
        }
    }
    EncodeFn enc = encode_fn();
    if (!enc) { delete pl; return FDTD_ERR_CUDA; }
    int st = FDTD_OK;
    for (int b = 0; b < 2 && st == FDTD_OK; b++)
        for (int q = 0; q < 3 && st == FDTD_OK; q++) {
            st = map3(enc, &pl->maps[b].e[q], s->f[b][q], g, BW, ER);
            if (st == FDTD_OK) st = map3(enc, &pl->maps[b].h[q], s->f[b][3 + q], g, BW, HOR);
            if (st == FDTD_OK) st = map3(enc, &pl->maps[b].ce[q], s->ce[q], g, TZ, TY);
        }
    if (st != FDTD_OK) { delete pl; return st; }
    int dev = 0, nsm = 0, occ = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaFuncSetAttribute((const void *)k_symp_pair, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void *)k_symp_pair, THREADS, SMEM);
    if (e != cudaSuccess) { set_cuda_error(e); delete pl; return FDTD_ERR_CUDA; }
    if (occ < 1) { delete pl; return FDTD_ERR_UNSUPPORTED; }
    const int64_t nitems = (int64_t)p.ntz * p.nty * p.nxc;
    pl->nblocks = (int)std::min<int64_t>(nitems, (int64_t)nsm * occ);
    *out = pl;
    return FDTD_OK;
}

int fdtd_symp_pair_run(fdtd_symp_plan *pl, const fdtd_cpml *ch_tabs_a, const fdtd_cpml *ch_tabs_b,
                       const fdtd_cpml *ce_tabs, float cl_a, float cl_b, int32_t two_h, float dl, float ch,
                       int64_t src_t, void *stream) {
    if (!pl || (two_h != 0 && two_h != 1)) return FDTD_ERR_ARG;
    const int in = pl->cur, ob = 1 - pl->cur;
    Params p = pl->base;
    for (int q = 0; q < 6; q++) {
        p.out[q] = pl->f[ob][q];
        p.psi_h_in[q] = pl->psi_h[in][q];
        p.psi_h_out[q] = const_cast<float *>(pl->psi_h[ob][q]);
    }
    p.cl_a = cl_a;
    p.cl_b = cl_b;
    p.dl = dl;
    p.ch = ch;
    p.clch_a = cl_a * ch;  // one IEEE single-precision product, as fdtd_symplectic_stage_f32
    p.clch_b = cl_b * ch;
    p.hh = two_h;
    p.t = src_t;
    const int64_t n3[3] = {pl->g.nx, pl->g.ny, pl->g.nz};
    const fdtd_cpml *tabs[3] = {ch_tabs_a, two_h ? ch_tabs_b : ch_tabs_a, ce_tabs};
    Axis *dst[3] = {p.ha, p.hb, p.ea};
    for (int w = 0; w < 3; w++) {
        const fdtd_cpml *c = tabs[w];
        for (int ax = 0; ax < 3; ax++) {
            Axis A{0, 0, 0, nullptr, nullptr, nullptr};
            if (c && c->npml[ax] > 0 && ((c->faces >> (2 * ax)) & 3)) {
                if (n3[ax] < 2 * (int64_t)c->npml[ax] + 2) return FDTD_ERR_SHAPE;
                A.P = c->npml[ax];
                A.front = (c->faces >> (2 * ax)) & 1;
                A.back = (c->faces >> (2 * ax + 1)) & 1;
                const bool e = w == 2;
                A.b = e ? c->b_e[ax] : c->b_h[ax];
                A.a = e ? c->a_e[ax] : c->a_h[ax];
                A.km1 = e ? c->km1_e[ax] : c->km1_h[ax];
                if (!all_nonnull(A.b, A.a, A.km1)) return FDTD_ERR_ARG;
                if (!(e ? p.psi_e[2 * ax] && p.psi_e[2 * ax + 1]
                        : p.psi_h_in[2 * ax] && p.psi_h_in[2 * ax + 1] && p.psi_h_out[2 * ax] && p.psi_h_out[2 * ax + 1]))
                    return FDTD_ERR_ARG;
                p.cpml = 1;
            }
            dst[w][ax] = A;
        }
    }
    k_symp_pair<<<pl->nblocks, THREADS, SMEM, as_stream(stream)>>>(pl->maps[in], p);
    FDTD_TRY(check_launch());
    pl->cur = ob;
    return FDTD_OK;
}

int fdtd_symp_pair_plan_current(const fdtd_symp_plan *pl) { return pl ? pl->cur : -1; }

int fdtd_symp_pair_plan_set_current(fdtd_symp_plan *pl, int32_t cur) {
    if (!pl || (cur != 0 && cur != 1)) return FDTD_ERR_ARG;
    pl->cur = cur;
    return FDTD_OK;
}

int fdtd_symp_pair_plan_destroy(fdtd_symp_plan *pl) {
    delete pl;
    return FDTD_OK;
}

}  // extern "C"
