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
// Design (2.5-D blocking)
//  * Ping-pong state: the pass reads buffer `cur` (E, H) and writes `1-cur`;
//    the H psi slabs ping-pong too (halo H cells are recomputed from the
//    input psi), the E psi slabs are updated in place (only their owner
//    touches them).
//  * A CTA owns TZ = 32 (z) x TY = 16 (y) cells for a chunk of x planes and
//    marches along x.  E_new(i) needs H_new on planes i-1 .. i+2 and on the
//    rows/columns -1 .. +2 around the tile, so H_new is computed on
//    (TY+3) x (TZ+3) cells: one thread per cell column (j, k), the 512 tile
//    columns first, then the 153 halo columns.  Each thread keeps the x
//    neighbours it needs in registers: the input E of planes m-2 .. m+1 for
//    H_new(m), and its own H_new of planes i-1 .. i+2 for E_new(i).  Shared
//    memory holds one plane with its y/z halo: input E boxes (4-slot ring),
//    input H and CE boxes (3-slot rings, 3-D TMA, issued two planes ahead)
//    and H_new (3-slot ring).
//  * Iteration q: input plane p arrives; every thread computes H_new(p-1) at
//    its column; tile threads then compute E_new(p-3).  One CTA barrier per
//    iteration: H_new(p-1) is read by neighbours two iterations later.
//  * Lane 0 of the last warp is the producer: it waits on the mbarriers and
//    issues the copies.  Every wait is bounded (1 s); on expiry the CTA
//    records FDTD_ERR_TIMEOUT, drains its copies and stops.
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
constexpr int NE = 4, NH = 3, NC = 3, NHN = 3;  // ring depths (E, H, CE inputs; H_new)
constexpr int NOWN = TY * TZ;                   // tile columns (threads 0 .. NOWN-1)
constexpr int NHALO = HNR * HNC - NOWN;         // halo H columns
constexpr int NCW = (NOWN + NHALO + 31) / 32;   // compute warps
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
// try_wait with a suspend-time hint: the waiting thread sleeps (up to the hint)
// until the phase completes instead of spinning on issue slots
__device__ __forceinline__ bool mbar_try(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(20000u)
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
// 4th-order difference of an H node: 27 (F0 - Fm1) - (Fp1 - Fm2)
__device__ __forceinline__ float d4h(float fm2, float fm1, float f0, float fp1) {
    return fsub(fmul(27.0f, fsub(f0, fm1)), fsub(fp1, fm2));
}
// 4th-order difference of an E node: 27 (Fp1 - F0) - (Fp2 - Fm1)
__device__ __forceinline__ float d4e(float fm1, float f0, float fp1, float fp2) {
    return fsub(fmul(27.0f, fsub(fp1, f0)), fsub(fp2, fm1));
}

__global__ void __launch_bounds__(THREADS, 1)
k_symp_pair(const __grid_constant__ Maps mk, const __grid_constant__ Params p) {
    extern __shared__ unsigned char smem_raw[];
    // 128-byte aligned base, computed from the shared-window offset so the
    // pointer stays in the shared address space (shared loads, not generic ones)
    unsigned char *smem =
        smem_raw + ((128u - (static_cast<uint32_t>(__cvta_generic_to_shared(smem_raw)) & 127u)) & 127u);
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
    // the H_new column (hr, hc) of this thread: tile columns first (warp = row,
    // lane = column), then the halo: rows j0-1, j0+TY, j0+TY+1, then the
    // columns k0-1, k0+TZ, k0+TZ+1 of the tile rows
    int hr = 0, hc = 0;
    const bool e_thread = tid < NOWN, h_thread = tid < NOWN + NHALO;
    if (e_thread) {
        hr = warp + 1;
        hc = lane + 1;
    } else if (h_thread) {
        const int h = tid - NOWN;
        if (h < 3 * HNC) {
            const int band = h / HNC;
            hr = band == 0 ? 0 : TY + band;
            hc = h - band * HNC;
        } else {
            const int g = (h - 3 * HNC) / TY;
            hr = 1 + (h - 3 * HNC) - g * TY;
            hc = g == 0 ? 0 : TZ + g;
        }
    }
    const int eo = (hr + 2) * BW + hc + 3;   // E box element of the column (row j0-3.., column k0-4..)
    const int ho = hr * BW + hc + 3;         // H box element (row j0-1..)
    const int no = hr * HNP + hc;            // H_new element (row j0-1.., column k0-1..)
    const int co = warp * TZ + lane;         // CE element (tile threads)

    uint32_t gE = 0, gH = 0, gC = 0;  // ring uses before the current item
    bool aborted = false;
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
        // the u-th use of a ring lands in slot u % depth and completes phase (u / depth) & 1
        auto eslot = [&](int q) { return (int)((gE + (uint32_t)q) % NE); };
        auto hslot = [&](int q) { return (int)((gH + (uint32_t)(q - 3)) % NH); };
        auto cslot = [&](int q) { return (int)((gC + (uint32_t)(q - 6)) % NC); };
        auto ephase = [&](int q) { return ((gE + (uint32_t)q) / NE) & 1; };
        auto hphase = [&](int q) { return ((gH + (uint32_t)(q - 3)) / NH) & 1; };
        auto cphase = [&](int q) { return ((gC + (uint32_t)(q - 6)) / NC) & 1; };
        auto issue = [&](int q) {  // copies needed at iteration q (issued two iterations ahead)
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
            issue(1);
        }
        const int nls = s_nls;
        const int j = j0 - 1 + hr, k = k0 - 1 + hc;
        const bool col_in = h_thread && j >= 0 && j < p.ny && k >= 0 && k < p.nz;
        const bool jin_h = j > 1 && j < p.ny - 1, kin_h = k > 1 && k < p.nz - 1;
        const bool jin_e = j > 0 && j < p.ny - 2, kin_e = k > 0 && k < p.nz - 2;
        const bool own_col = e_thread;
        // y/z slab indices of the column (H nodes for the H stages, E nodes for the E stage)
        int syh = -1, szh = -1, sye = -1, sze = -1;
        if (p.cpml && col_in) {
            syh = slab(p.ha[1], j, p.ny, false);
            szh = slab(p.ha[2], k, p.nz, false);
            sye = slab(p.ea[1], j, p.ny, true);
            sze = slab(p.ea[2], k, p.nz, true);
        }
        // register queues of the column: input E of planes p-3 .. p-1 (ex, ey, ez),
        // own H_new of planes p-4 .. p-2 (hy, hz)
        float e0x = 0.f, e0y = 0.f, e0z = 0.f, e1x = 0.f, e1y = 0.f, e1z = 0.f, e2x = 0.f, e2y = 0.f, e2z = 0.f;
        float n0y = 0.f, n0z = 0.f, n1y = 0.f, n1z = 0.f, n2y = 0.f, n2z = 0.f;
        int q_abort = 0;
        for (int q = 0; q < Q; q++) {
            const int pl = x0 - 3 + q;
            const int eS = eslot(q);
            if (producer) {
                bool ok = mbar_wait(&bars[eS], ephase(q), p.status);
                if (ok && q >= 3) ok = mbar_wait(&bars[NE + hslot(q)], hphase(q), p.status);
                if (ok && q >= 6) ok = mbar_wait(&bars[NE + NH + cslot(q)], cphase(q), p.status);
                if (!ok) s_abort = 1;
            }
            __syncthreads();  // copies of iteration q visible; iteration q-1 done everywhere
            if (s_abort) {
                aborted = true;
                q_abort = q;
                break;
            }
            if (producer && q + 2 < Q) issue(q + 2);

            // input E of plane p at this column
            float e3x = 0.f, e3y = 0.f, e3z = 0.f;
            if (h_thread) {
                e3x = sE(eS, 0)[eo];
                e3y = sE(eS, 1)[eo];
                e3z = sE(eS, 2)[eo];
            }
            // ---- H_new(m), m = p - 1, at this column ----
            const int m = pl - 1;
            float hny = 0.f, hnz = 0.f;
            if (q >= 3 && col_in && m >= 0 && m < p.nx) {
                const int eSm = eslot(q - 1), hS = hslot(q);
                const float *ex = sE(eSm, 0), *ey = sE(eSm, 1), *ez = sE(eSm, 2);
                const float hx0 = sH(hS, 0)[ho], hy0 = sH(hS, 1)[ho], hz0 = sH(hS, 2)[ho];
                const bool iin = m > 1 && m < p.nx - 1;
                const bool own = own_col && m >= x0 && m < x1;
                const int sxh = p.cpml ? slab(p.ha[0], m, p.nx, false) : -1;
                const int nst = p.hh ? 2 : 1;
                float vx = hx0, vy = hy0, vz = hz0;
                const int e = eo;
                if (jin_h && kin_h) {  // hx: ez along y, ey along z (plane m)
                    const float ezm2 = ez[e - 2 * BW], ezm1 = ez[e - BW], ezp1 = ez[e + BW];
                    const float eym2 = ey[e - 2], eym1 = ey[e - 1], eyp1 = ey[e + 1];
                    const float n = curl4(e2z, ezm1, e2y, eym1);
                    const float f = curl4(ezp1, ezm2, eyp1, eym2);
                    const float d27 = fsub(fmul(27.0f, n), f);
                    float py = 0.f, pz = 0.f;
                    uint32_t qy = 0, qz = 0;
                    if (syh >= 0) { qy = psi_index(p, 1, syh, m, j, k, p.ha[1].P); py = p.psi_h_in[3][qy]; }
                    if (szh >= 0) { qz = psi_index(p, 2, szh, m, j, k, p.ha[2].P); pz = p.psi_h_in[4][qz]; }
                    const float dy = syh >= 0 ? d4h(ezm2, ezm1, e2z, ezp1) : 0.f;
                    const float dz = szh >= 0 ? d4h(eym2, eym1, e2y, eyp1) : 0.f;
                    for (int st = 0; st < nst; st++) {
                        const float cl = st ? p.cl_b : p.cl_a, clch = st ? p.clch_b : p.clch_a;
                        const Axis *A = st ? p.hb : p.ha;
                        vx = fsub(vx, fmul(clch, d27));
                        if (syh >= 0) vx = fsub(vx, sterm(A[1], syh, py, dy, cl, p.ch));
                        if (szh >= 0) vx = fadd(vx, sterm(A[2], szh, pz, dz, cl, p.ch));
                    }
                    if (own && syh >= 0) p.psi_h_out[3][qy] = py;
                    if (own && szh >= 0) p.psi_h_out[4][qz] = pz;
                }
                if (iin && kin_h) {  // hy: ex along z (plane m), ez along x (queue)
                    const float exm2 = ex[e - 2], exm1 = ex[e - 1], exp1 = ex[e + 1];
                    const float n = curl4(e2x, exm1, e2z, e1z);
                    const float f = curl4(exp1, exm2, e3z, e0z);
                    const float d27 = fsub(fmul(27.0f, n), f);
                    float px = 0.f, pz = 0.f;
                    uint32_t qx = 0, qz = 0;
                    if (sxh >= 0) { qx = psi_index(p, 0, sxh, m, j, k, p.ha[0].P); px = p.psi_h_in[0][qx]; }
                    if (szh >= 0) { qz = psi_index(p, 2, szh, m, j, k, p.ha[2].P); pz = p.psi_h_in[5][qz]; }
                    const float dx = sxh >= 0 ? d4h(e0z, e1z, e2z, e3z) : 0.f;
                    const float dz = szh >= 0 ? d4h(exm2, exm1, e2x, exp1) : 0.f;
                    for (int st = 0; st < nst; st++) {
                        const float cl = st ? p.cl_b : p.cl_a, clch = st ? p.clch_b : p.clch_a;
                        const Axis *A = st ? p.hb : p.ha;
                        vy = fsub(vy, fmul(clch, d27));
                        if (sxh >= 0) vy = fadd(vy, sterm(A[0], sxh, px, dx, cl, p.ch));
                        if (szh >= 0) vy = fsub(vy, sterm(A[2], szh, pz, dz, cl, p.ch));
                    }
                    if (own && sxh >= 0) p.psi_h_out[0][qx] = px;
                    if (own && szh >= 0) p.psi_h_out[5][qz] = pz;
                }
                if (iin && jin_h) {  // hz: ey along x (queue), ex along y (plane m)
                    const float exm2 = ex[e - 2 * BW], exm1 = ex[e - BW], exp1 = ex[e + BW];
                    const float n = curl4(e2y, e1y, e2x, exm1);
                    const float f = curl4(e3y, e0y, exp1, exm2);
                    const float d27 = fsub(fmul(27.0f, n), f);
                    float px = 0.f, py = 0.f;
                    uint32_t qx = 0, qy = 0;
                    if (sxh >= 0) { qx = psi_index(p, 0, sxh, m, j, k, p.ha[0].P); px = p.psi_h_in[1][qx]; }
                    if (syh >= 0) { qy = psi_index(p, 1, syh, m, j, k, p.ha[1].P); py = p.psi_h_in[2][qy]; }
                    const float dx = sxh >= 0 ? d4h(e0y, e1y, e2y, e3y) : 0.f;
                    const float dy = syh >= 0 ? d4h(exm2, exm1, e2x, exp1) : 0.f;
                    for (int st = 0; st < nst; st++) {
                        const float cl = st ? p.cl_b : p.cl_a, clch = st ? p.clch_b : p.clch_a;
                        const Axis *A = st ? p.hb : p.ha;
                        vz = fsub(vz, fmul(clch, d27));
                        if (sxh >= 0) vz = fsub(vz, sterm(A[0], sxh, px, dx, cl, p.ch));
                        if (syh >= 0) vz = fadd(vz, sterm(A[1], syh, py, dy, cl, p.ch));
                    }
                    if (own && sxh >= 0) p.psi_h_out[1][qx] = px;
                    if (own && syh >= 0) p.psi_h_out[2][qy] = py;
                }
                const int nsl = (m - (x0 - 1)) % NHN;
                sN(nsl, 0)[no] = vx;
                sN(nsl, 1)[no] = vy;
                sN(nsl, 2)[no] = vz;
                hny = vy;
                hnz = vz;
                if (own) {
                    const uint32_t g = (uint32_t)m * p.sx + (uint32_t)j * p.sy + k;
                    p.out[3][g] = vx;
                    p.out[4][g] = vy;
                    p.out[5][g] = vz;
                }
            }

            // ---- E_new(i), i = p - 3, at tile columns ----
            const int i = pl - 3;
            if (q >= 6 && own_col && col_in) {
                // H_new at planes i-1 .. i+2 of this column: n0 (i-1), n1 (i), n2 (i+1), new (i+2);
                // H_new(i) neighbours from the ring (written two iterations ago)
                const int nsl = (i - (x0 - 1)) % NHN;
                const float *hx = sN(nsl, 0), *hy = sN(nsl, 1), *hz = sN(nsl, 2);
                const int cS = cslot(q);
                const int h = no;
                float vx = e0x, vy = e0y, vz = e0z;  // input E of plane i
                const bool iin = i > 0 && i < p.nx - 2;
                const int sxe = p.cpml ? slab(p.ea[0], i, p.nx, true) : -1;
                if (jin_e && kin_e) {  // ex: hz along y, hy along z (plane i)
                    const float hzm1 = hz[h - HNP], hzp1 = hz[h + HNP], hzp2 = hz[h + 2 * HNP];
                    const float hym1 = hy[h - 1], hyp1 = hy[h + 1], hyp2 = hy[h + 2];
                    const float n = curl4(hzp1, n1z, hyp1, n1y);
                    const float f = curl4(hzp2, hzm1, hyp2, hym1);
                    const float cv = sC(cS, 0)[co];
                    vx = fadd(vx, fmul(fmul(p.dl, cv), fsub(fmul(27.0f, n), f)));
                    if (sye >= 0) {
                        const uint32_t qi = psi_index(p, 1, sye, i, j, k, p.ea[1].P);
                        float ps = p.psi_e[3][qi];
                        vx = fadd(vx, sterm(p.ea[1], sye, ps, d4e(hzm1, n1z, hzp1, hzp2), p.dl, cv));
                        p.psi_e[3][qi] = ps;
                    }
                    if (sze >= 0) {
                        const uint32_t qi = psi_index(p, 2, sze, i, j, k, p.ea[2].P);
                        float ps = p.psi_e[4][qi];
                        vx = fsub(vx, sterm(p.ea[2], sze, ps, d4e(hym1, n1y, hyp1, hyp2), p.dl, cv));
                        p.psi_e[4][qi] = ps;
                    }
                }
                if (iin && kin_e) {  // ey: hx along z (plane i), hz along x (queue)
                    const float hx0 = hx[h], hxm1 = hx[h - 1], hxp1 = hx[h + 1], hxp2 = hx[h + 2];
                    const float n = curl4(hxp1, hx0, n2z, n1z);
                    const float f = curl4(hxp2, hxm1, hnz, n0z);
                    const float cv = sC(cS, 1)[co];
                    vy = fadd(vy, fmul(fmul(p.dl, cv), fsub(fmul(27.0f, n), f)));
                    if (sxe >= 0) {
                        const uint32_t qi = psi_index(p, 0, sxe, i, j, k, p.ea[0].P);
                        float ps = p.psi_e[0][qi];
                        vy = fsub(vy, sterm(p.ea[0], sxe, ps, d4e(n0z, n1z, n2z, hnz), p.dl, cv));
                        p.psi_e[0][qi] = ps;
                    }
                    if (sze >= 0) {
                        const uint32_t qi = psi_index(p, 2, sze, i, j, k, p.ea[2].P);
                        float ps = p.psi_e[5][qi];
                        vy = fadd(vy, sterm(p.ea[2], sze, ps, d4e(hxm1, hx0, hxp1, hxp2), p.dl, cv));
                        p.psi_e[5][qi] = ps;
                    }
                }
                if (iin && jin_e) {  // ez: hy along x (queue), hx along y (plane i)
                    const float hx0 = hx[h], hxm1 = hx[h - HNP], hxp1 = hx[h + HNP], hxp2 = hx[h + 2 * HNP];
                    const float n = curl4(n2y, n1y, hxp1, hx0);
                    const float f = curl4(hny, n0y, hxp2, hxm1);
                    const float cv = sC(cS, 2)[co];
                    vz = fadd(vz, fmul(fmul(p.dl, cv), fsub(fmul(27.0f, n), f)));
                    if (sxe >= 0) {
                        const uint32_t qi = psi_index(p, 0, sxe, i, j, k, p.ea[0].P);
                        float ps = p.psi_e[1][qi];
                        vz = fadd(vz, sterm(p.ea[0], sxe, ps, d4e(n0y, n1y, n2y, hny), p.dl, cv));
                        p.psi_e[1][qi] = ps;
                    }
                    if (sye >= 0) {
                        const uint32_t qi = psi_index(p, 1, sye, i, j, k, p.ea[1].P);
                        float ps = p.psi_e[2][qi];
                        vz = fsub(vz, sterm(p.ea[1], sye, ps, d4e(hxm1, hx0, hxp1, hxp2), p.dl, cv));
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
            // advance the queues
            e0x = e1x; e0y = e1y; e0z = e1z;
            e1x = e2x; e1y = e2y; e1z = e2z;
            e2x = e3x; e2y = e3y; e2z = e3z;
            n0y = n1y; n0z = n1z;
            n1y = n2y; n1z = n2z;
            n2y = hny; n2z = hnz;
        }
        if (aborted) {
            if (producer) {
                atomicExch(p.status, FDTD_ERR_TIMEOUT);
                // let the copies in flight (iterations q and q+1) land before the
                // shared memory is released; each wait bounded
                for (int q = q_abort; q < Q && q < q_abort + 2; q++) {
                    mbar_wait(&bars[eslot(q)], ephase(q), nullptr);
                    if (q >= 3) mbar_wait(&bars[NE + hslot(q)], hphase(q), nullptr);
                    if (q >= 6) mbar_wait(&bars[NE + NH + cslot(q)], cphase(q), nullptr);
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
    NvtxRange nvtx_range("fdtd_symp_pair");
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
