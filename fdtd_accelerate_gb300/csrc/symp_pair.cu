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
// Design (2.5-D blocking, 4 z cells per thread)
//  * Ping-pong state: the pass reads buffer `cur` (E, H) and writes `1-cur`;
//    the H psi slabs ping-pong too (halo H cells are recomputed from the
//    input psi), the E psi slabs are updated in place (only their owner
//    touches them).
//  * A CTA owns TZ = 32 (z) x TY = 16 (y) cells for a chunk of x planes and
//    marches along x.  E_new(i) needs H_new on planes i-1 .. i+2 and on the
//    rows/columns -1 .. +2 around the tile, so H_new is computed on the rows
//    j0-1 .. j0+TY+1 and the columns k0-4 .. k0+TZ+3, in groups of 4 z cells:
//    one thread per group, the 128 tile groups first (those threads also
//    compute E_new of their group), then the 62 halo groups.  Every group is
//    16-byte aligned, so its z window (the group and the neighbouring
//    groups) is three 16-byte shared loads.
//  * Each thread keeps the x neighbours it needs in registers: the input E of
//    planes m-3 .. m-1 for H_new(m-1), and its own H_new (hy, hz) of planes
//    i-1 .. i+1 for E_new(i).  Shared memory holds one plane with its y/z
//    halo: input E boxes (4-slot ring) and H boxes (3-slot ring), both issued
//    two planes ahead, CE boxes (2-slot ring, one plane ahead) and H_new
//    (3-slot ring).  About 108 KB, two CTAs per SM.
//  * Iteration q: input plane p arrives; every thread computes H_new(p-1) for
//    its group; tile threads then compute E_new(p-3).  One CTA barrier per
//    iteration: H_new(p-1) is read by neighbours two iterations later.
//  * Warps whose groups lie in no CPML slab on a plane outside the x slabs
//    take a path without psi code; the others run the CPML terms cell by
//    cell in the operation order of the stage kernels, each component's psi
//    values of the 4 cells loaded together.
//  * CTAs draw work items from a device queue (two ints the caller provides,
//    cleared by the last CTA of each launch).  With y or z slabs the edge
//    tiles, which carry them, are handed out first, so a launch ends on
//    interior tiles.
//  * Lane 31 of the last warp is the producer: it waits on the mbarriers and
//    issues the copies.  Every wait is bounded (1 s); on expiry the CTA
//    records FDTD_ERR_TIMEOUT, drains its copies and stops.
#include <cuda.h>

#include <algorithm>
#include <vector>

#include "common.cuh"

namespace fdtd {
namespace sp {

constexpr int TZ = 32, TY = 16;
constexpr int NG = TZ / 4 + 2;      // groups per H row: columns k0-4 .. k0+TZ+3
constexpr int BW = TZ + 8;          // row width of the E, H and H_new boxes (column k0-4 first)
constexpr int ER = TY + 6;          // E box rows: j0-3 .. j0+TY+2
constexpr int HOR = TY + 3;         // H and H_new rows: j0-1 .. j0+TY+1
constexpr int NE = 4, NH = 3, NC = 2, NHN = 3;  // ring depths (E, H, CE inputs; H_new)
constexpr int NTILE = TY * (TZ / 4);            // tile groups (threads 0 .. NTILE-1)
constexpr int NHALO = HOR * NG - NTILE;         // halo groups
constexpr int THREADS = (NTILE + NHALO + 1 + 31) / 32 * 32;
constexpr int PRODUCER = THREADS - 1;
constexpr int MAX_SRC = 64;                     // sources per work item
constexpr uint64_t WAIT_NS = 1000000000ull;
static_assert(NTILE + NHALO < PRODUCER, "the producer lane computes no group");

constexpr int al128(int b) { return (b + 127) / 128 * 128; }
constexpr int EBOXB = al128(ER * BW * 4), HBOXB = al128(HOR * BW * 4), CBOXB = al128(TY * TZ * 4);
constexpr int OFF_E = 0;
constexpr int OFF_H = OFF_E + NE * 3 * EBOXB;
constexpr int OFF_C = OFF_H + NH * 3 * HBOXB;
constexpr int OFF_HN = OFF_C + NC * 3 * CBOXB;
constexpr int OFF_BAR = OFF_HN + NHN * 3 * HBOXB;
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
    int32_t edge_first;       // y or z slabs: edge tiles first in the work order
    int32_t nsrc;
    const int32_t *src_ijk, *src_comp;
    const float *src_amp;
    int64_t namp, t;          // amplitude table length and the index used
    int32_t *status;
    // work queue: [0] next item, [1] CTAs finished; zero between launches (the
    // last CTA to finish clears both)
    int32_t *queue;
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
// CPML tables of one stage along one axis
struct Tab {
    const float *b, *a, *km1;
};
__device__ __forceinline__ Tab tab(const Axis &A) { return Tab{A.b, A.a, A.km1}; }
// the tables of H stage b (st = 1) or a, selected by value
__device__ __forceinline__ Tab tab_h(const Params &p, int st, int ax) {
    return Tab{st ? p.hb[ax].b : p.ha[ax].b, st ? p.hb[ax].a : p.ha[ax].a, st ? p.hb[ax].km1 : p.ha[ax].km1};
}
// psi <- b psi + a d; returns (coef * cv) * (km1 d + psi)
__device__ __forceinline__ float sterm(const Tab &T, int s, float &psi, float d, float coef, float cv) {
    psi = fadd(fmul(__ldg(T.b + s), psi), fmul(__ldg(T.a + s), d));
    return fmul(fmul(coef, cv), fadd(fmul(__ldg(T.km1 + s), d), psi));
}
// 4th-order difference of an H node: 27 (F0 - Fm1) - (Fp1 - Fm2)
__device__ __forceinline__ float d4h(float fm2, float fm1, float f0, float fp1) {
    return fsub(fmul(27.0f, fsub(f0, fm1)), fsub(fp1, fm2));
}
// 4th-order difference of an E node: 27 (Fp1 - F0) - (Fp2 - Fm1)
__device__ __forceinline__ float d4e(float fm1, float f0, float fp1, float fp2) {
    return fsub(fmul(27.0f, fsub(fp1, f0)), fsub(fp2, fm1));
}

// four consecutive floats of shared memory (16-byte aligned)
struct V4 {
    float v[4];
};
__device__ __forceinline__ V4 lds4(const float *s) {
    const float4 t = *reinterpret_cast<const float4 *>(s);
    return V4{{t.x, t.y, t.z, t.w}};
}
__device__ __forceinline__ void sts4(float *s, const V4 &a) {
    *reinterpret_cast<float4 *>(s) = make_float4(a.v[0], a.v[1], a.v[2], a.v[3]);
}
// z window of a group: w(d) = the value at z offset d (-4 .. 7) from the
// group's first cell, from the loads of the groups left (L), own (C), right (R)
struct ZW {
    V4 L, C, R;
    __device__ __forceinline__ float at(int d) const {
        return d < 0 ? L.v[d + 4] : (d < 4 ? C.v[d] : R.v[d - 4]);
    }
};

// global store of a group's 4 values (cells k .. k+3 of a row); cells at
// z >= nz are not stored
__device__ __forceinline__ void stg4(float *row, int k, int nz, const V4 &a) {
    if (k + 3 < nz) {
        *reinterpret_cast<float4 *>(row + k) = make_float4(a.v[0], a.v[1], a.v[2], a.v[3]);
    } else {
#pragma unroll
        for (int c = 0; c < 4; c++)
            if (k + c < nz) row[k + c] = a.v[c];
    }
}

// Work item u -> tile (tzi, tyi) and x chunk xci.  The y/z edge tiles (first
// or last tile row or column) of every x chunk come first, then the interior
// tiles; inside each part the z tile runs fastest, then the y tile, then the
// x chunk.
__device__ __forceinline__ void item_tile(const Params &p, int u, int &tzi, int &tyi, int &xci) {
    const int nz = p.ntz, ny = p.nty;
    const int ni = (nz > 2 && ny > 2) ? (nz - 2) * (ny - 2) : 0;  // interior tiles per chunk
    const int ne = nz * ny - ni;                                   // edge tiles per chunk
    if (!p.edge_first) {  // z tile fastest, then y tile, then x chunk
        tzi = u % nz;
        tyi = (u / nz) % ny;
        xci = u / (nz * ny);
        return;
    }
    if (u < ne * p.nxc) {
        xci = u / ne;
        const int e = u - xci * ne;
        if (e < 2 * nz || ni == 0) {  // the first and last tile rows (all tiles when ni == 0)
            const int r = ni == 0 ? e / nz : (e < nz ? 0 : ny - 1);
            tyi = r;
            tzi = ni == 0 ? e - r * nz : (e < nz ? e : e - nz);
        } else {                      // the first and last tile of each inner row
            const int f = e - 2 * nz;
            tyi = 1 + (f >> 1);
            tzi = (f & 1) ? nz - 1 : 0;
        }
    } else {
        const int v = u - ne * p.nxc;
        xci = v / ni;
        const int r = v - xci * ni;
        tyi = 1 + r / (nz - 2);
        tzi = 1 + r % (nz - 2);
    }
}

// HH: two H stages before the E stage (the pass that merges the closing H
// stage of a step with the opening one of the next)
template <bool HH>
__global__ void __launch_bounds__(THREADS, 2)
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
    auto sN = [&](int sl, int c) { return reinterpret_cast<float *>(smem + OFF_HN + (sl * 3 + c) * HBOXB); };
    __shared__ int s_abort, s_nls, s_item;
    __shared__ int s_ls_i[MAX_SRC], s_ls_j[MAX_SRC], s_ls_kc[MAX_SRC], s_ls_s[MAX_SRC];

    const int tid = threadIdx.x;
    const bool producer = tid == PRODUCER;
    if (tid == 0) {
        for (int s = 0; s < NE + NH + NC; s++) mbar_init(&bars[s]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        s_abort = 0;
    }
    // the group of this thread: H row hr (j0-1+hr), group g (columns
    // k0-4+4g .. k0-1+4g).  Tile groups first (row hr = 1 + tid/8, groups
    // 1 .. 8), then the halo: rows 0, TY+1, TY+2 (all groups), then groups 0
    // and NG-1 of the tile rows.
    int hr = 0, g = 0;
    const bool e_thread = tid < NTILE, h_thread = tid < NTILE + NHALO;
    if (e_thread) {
        hr = 1 + tid / (TZ / 4);
        g = 1 + tid % (TZ / 4);
    } else if (h_thread) {
        const int h = tid - NTILE;
        if (h < 3 * NG) {
            const int band = h / NG;
            hr = band == 0 ? 0 : TY + band;
            g = h - band * NG;
        } else {
            const int u = h - 3 * NG;
            hr = 1 + (u >> 1);
            g = (u & 1) ? NG - 1 : 0;
        }
    }
    const int col = 4 * g;                                   // first box column of the group
    const int colL = g == 0 ? col : col - 4;                 // left and right neighbour groups (clamped:
    const int colR = g == NG - 1 ? col : col + 4;            // the cells that would use them are not needed)
    const int eo = (hr + 2) * BW + col;                      // E box element of the group (row j0-3..)
    const int ho = hr * BW + col;                            // H and H_new box element (row j0-1..)
    const int co = (hr - 1) * TZ + col - 4;                  // CE box element (tile threads)

    uint32_t gE = 0, gH = 0, gC = 0;  // ring uses before the current item
    bool aborted = false;
    const int64_t nitems = (int64_t)p.ntz * p.nty * p.nxc;
    // items from the work queue (item_tile gives the order: the y/z edge tiles,
    // which carry the y and z CPML slabs, first): CTAs that drew cheaper tiles
    // take more of them, and the last items of a launch are interior tiles
    if (tid == 0) s_item = atomicAdd(&p.queue[0], 1);
    __syncthreads();
    for (int64_t item = s_item; item < nitems && !aborted;) {
        int tzi, tyi, xci;
        item_tile(p, (int)item, tzi, tyi, xci);
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
        auto issue_eh = [&](int q) {  // E and H copies of iteration q (issued two iterations ahead)
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
        };
        auto issue_c = [&](int q) {  // CE(p-3) of iteration q >= 6 (issued one iteration ahead)
            const int sl = cslot(q);
            uint64_t *bar = &bars[NE + NH + sl];
            mbar_expect(bar, 3u * TY * TZ * 4);
            for (int c = 0; c < 3; c++) tma3(sC(sl, c), &mk.ce[c], bar, k0, j0, x0 + q - 6);
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
            issue_eh(0);
            if (Q > 1) issue_eh(1);
        }
        const int nls = s_nls;
        const int j = j0 - 1 + hr, kg = k0 - 4 + col;   // row and first z cell of the group
        const bool row_in = h_thread && j >= 0 && j < p.ny;
        const bool jin_h = j > 1 && j < p.ny - 1, jin_e = j > 0 && j < p.ny - 2;
        // per-cell z masks of the group (bit c: cell kg+c)
        uint32_t kin_h = 0, kin_e = 0, k_in = 0;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const int k = kg + c;
            kin_h |= (uint32_t)(k > 1 && k < p.nz - 1) << c;
            kin_e |= (uint32_t)(k > 0 && k < p.nz - 2) << c;
            k_in |= (uint32_t)(k >= 0 && k < p.nz) << c;
        }
        // CPML: y slab of the row (H and E nodes); any z-slab cell in the group
        int syh = -1, sye = -1;
        bool zh_any = false, ze_any = false;
        if (p.cpml && row_in) {
            syh = slab(p.ha[1], j, p.ny, false);
            sye = slab(p.ea[1], j, p.ny, true);
#pragma unroll
            for (int c = 0; c < 4; c++) {
                zh_any |= slab(p.ha[2], kg + c, p.nz, false) >= 0;
                ze_any |= slab(p.ea[2], kg + c, p.nz, true) >= 0;
            }
        }
        // the path choice is made per warp: a warp with any slab cell runs the
        // CPML path for all its lanes (it handles plain cells as well), so it
        // never runs both paths one after the other
        const bool yz_h = __any_sync(0xffffffffu, syh >= 0 || zh_any);
        const bool yz_e = __any_sync(0xffffffffu, sye >= 0 || ze_any);

        // register queue of the group: input E of planes p-3 and p-2 (ex, ey,
        // ez); planes p-1 and p are still in the E ring, and the group's own
        // H_new of the planes around E_new(i) in the H_new ring
        V4 e0x{}, e0y{}, e0z{}, e1x{}, e1y{}, e1z{};
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
            if (producer) {
                if (q + 2 < Q) issue_eh(q + 2);
                if (q + 1 < Q && q + 1 >= 6) issue_c(q + 1);
            }

            // input E of planes p-1 and p at this group
            V4 e2x{}, e2y{}, e2z{}, e3x{}, e3y{}, e3z{};
            if (h_thread) {
                e3x = lds4(sE(eS, 0) + eo);
                e3y = lds4(sE(eS, 1) + eo);
                e3z = lds4(sE(eS, 2) + eo);
                if (q >= 1) {
                    const int eSp = eslot(q - 1);
                    e2x = lds4(sE(eSp, 0) + eo);
                    e2y = lds4(sE(eSp, 1) + eo);
                    e2z = lds4(sE(eSp, 2) + eo);
                }
            }
            // own H_new (hy, hz) of plane p-4 for E_new(p-3): its ring slot
            // takes H_new(p-1) below
            V4 n0y{}, n0z{};
            if (q >= 6 && e_thread) {
                const int nsl0 = (pl - 4 - (x0 - 1)) % NHN;
                n0y = lds4(sN(nsl0, 1) + ho);
                n0z = lds4(sN(nsl0, 2) + ho);
            }
            // ---- H_new(m), m = p - 1, at this group ----
            const int m = pl - 1;
            V4 hny{}, hnz{};
            if (q >= 3 && row_in && m >= 0 && m < p.nx) {
                const int eSm = eslot(q - 1), hS = hslot(q);
                const float *ex = sE(eSm, 0), *ey = sE(eSm, 1), *ez = sE(eSm, 2);
                const V4 hx0 = lds4(sH(hS, 0) + ho), hy0 = lds4(sH(hS, 1) + ho), hz0 = lds4(sH(hS, 2) + ho);
                // rows j-2, j-1, j+1 of ez (hx) and ex (hz); z windows of ey (hx) and ex (hy)
                const V4 ezm2 = lds4(ez + eo - 2 * BW), ezm1 = lds4(ez + eo - BW), ezp1 = lds4(ez + eo + BW);
                const V4 exm2 = lds4(ex + eo - 2 * BW), exm1 = lds4(ex + eo - BW), exp1 = lds4(ex + eo + BW);
                const ZW wy{lds4(ey + eo - col + colL), e2y, lds4(ey + eo - col + colR)};
                const ZW wx{lds4(ex + eo - col + colL), e2x, lds4(ex + eo - col + colR)};
                const bool iin = m > 1 && m < p.nx - 1;
                const bool own = e_thread && m >= x0 && m < x1;
                const int sxh = p.cpml ? slab(p.ha[0], m, p.nx, false) : -1;
                constexpr bool hh = HH;
                V4 vx = hx0, vy = hy0, vz = hz0;
                if (!yz_h && sxh < 0) {
                    // no CPML term at any cell of the group on this plane
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        {   // hx: ez along y, ey along z (plane m)
                            const float n = curl4(e2z.v[c], ezm1.v[c], wy.at(c), wy.at(c - 1));
                            const float f = curl4(ezp1.v[c], ezm2.v[c], wy.at(c + 1), wy.at(c - 2));
                            const float d27 = fsub(fmul(27.0f, n), f);
                            float v = fsub(vx.v[c], fmul(p.clch_a, d27));
                            if (hh) v = fsub(v, fmul(p.clch_b, d27));
                            if (jin_h && ((kin_h >> c) & 1)) vx.v[c] = v;
                        }
                        {   // hy: ex along z (plane m), ez along x (queue)
                            const float n = curl4(e2x.v[c], wx.at(c - 1), e2z.v[c], e1z.v[c]);
                            const float f = curl4(wx.at(c + 1), wx.at(c - 2), e3z.v[c], e0z.v[c]);
                            const float d27 = fsub(fmul(27.0f, n), f);
                            float v = fsub(vy.v[c], fmul(p.clch_a, d27));
                            if (hh) v = fsub(v, fmul(p.clch_b, d27));
                            if (iin && ((kin_h >> c) & 1)) vy.v[c] = v;
                        }
                        {   // hz: ey along x (queue), ex along y (plane m)
                            const float n = curl4(e2y.v[c], e1y.v[c], e2x.v[c], exm1.v[c]);
                            const float f = curl4(e3y.v[c], e0y.v[c], exp1.v[c], exm2.v[c]);
                            const float d27 = fsub(fmul(27.0f, n), f);
                            float v = fsub(vz.v[c], fmul(p.clch_a, d27));
                            if (hh) v = fsub(v, fmul(p.clch_b, d27));
                            if (iin && jin_h) vz.v[c] = v;
                        }
                    }
                } else {
                    // CPML path: per component the main term of the 4 cells, then
                    // the CPML terms on the slab cells, stage by stage (the
                    // operation order of the stage kernels).  psi offsets: the x
                    // and y slabs hold the group's cells contiguously, the z slab
                    // at the cells' slab indices.
                    const uint32_t ux = jin_h ? kin_h : 0u, uy = iin ? kin_h : 0u, uz = iin && jin_h ? k_in : 0u;
                    const uint32_t offx = sxh >= 0 ? ((uint32_t)sxh * p.ny + j) * p.nz + kg : 0u;
                    const uint32_t offy = syh >= 0 ? ((uint32_t)m * (2u * p.ha[1].P) + syh) * p.nz + kg : 0u;
                    const uint32_t offz = ((uint32_t)m * p.ny + j) * (2u * p.ha[2].P);
                    int szh[4];
#pragma unroll
                    for (int c = 0; c < 4; c++) szh[c] = slab(p.ha[2], kg + c, p.nz, false);
                    {   // hx: ez along y, ey along z; y term subtracted, z term added
                        float ps1[4], ps2[4], d27[4];
#pragma unroll
                        for (int c = 0; c < 4; c++) {
                            const bool up = (ux >> c) & 1;
                            ps1[c] = up && syh >= 0 ? __ldg(p.psi_h_in[3] + offy + c) : 0.f;
                            ps2[c] = up && szh[c] >= 0 ? __ldg(p.psi_h_in[4] + offz + szh[c]) : 0.f;
                            const float n = curl4(e2z.v[c], ezm1.v[c], wy.at(c), wy.at(c - 1));
                            const float f = curl4(ezp1.v[c], ezm2.v[c], wy.at(c + 1), wy.at(c - 2));
                            d27[c] = fsub(fmul(27.0f, n), f);
                        }
#pragma unroll
                        for (int st = 0; st < (HH ? 2 : 1); st++) {
                            const float clch = st ? p.clch_b : p.clch_a, cl = st ? p.cl_b : p.cl_a;
                            const Tab T1 = tab_h(p, st, 1), T2 = tab_h(p, st, 2);
#pragma unroll
                            for (int c = 0; c < 4; c++) {
                                if (!((ux >> c) & 1)) continue;
                                float v = fsub(vx.v[c], fmul(clch, d27[c]));
                                if (syh >= 0)
                                    v = fsub(v, sterm(T1, syh, ps1[c], d4h(ezm2.v[c], ezm1.v[c], e2z.v[c], ezp1.v[c]), cl, p.ch));
                                if (szh[c] >= 0)
                                    v = fadd(v, sterm(T2, szh[c], ps2[c], d4h(wy.at(c - 2), wy.at(c - 1), wy.at(c), wy.at(c + 1)), cl, p.ch));
                                vx.v[c] = v;
                            }
                        }
                        if (own) {
#pragma unroll
                            for (int c = 0; c < 4; c++) {
                                if (!((ux >> c) & 1)) continue;
                                if (syh >= 0) p.psi_h_out[3][offy + c] = ps1[c];
                                if (szh[c] >= 0) p.psi_h_out[4][offz + szh[c]] = ps2[c];
                            }
                        }
                    }
                    {   // hy: ex along z (plane m), ez along x (queue); x term added, z term subtracted
                        float ps1[4], ps2[4], d27[4];
#pragma unroll
                        for (int c = 0; c < 4; c++) {
                            const bool up = (uy >> c) & 1;
                            ps1[c] = up && sxh >= 0 ? __ldg(p.psi_h_in[0] + offx + c) : 0.f;
                            ps2[c] = up && szh[c] >= 0 ? __ldg(p.psi_h_in[5] + offz + szh[c]) : 0.f;
                            const float n = curl4(e2x.v[c], wx.at(c - 1), e2z.v[c], e1z.v[c]);
                            const float f = curl4(wx.at(c + 1), wx.at(c - 2), e3z.v[c], e0z.v[c]);
                            d27[c] = fsub(fmul(27.0f, n), f);
                        }
#pragma unroll
                        for (int st = 0; st < (HH ? 2 : 1); st++) {
                            const float clch = st ? p.clch_b : p.clch_a, cl = st ? p.cl_b : p.cl_a;
                            const Tab T0 = tab_h(p, st, 0), T2 = tab_h(p, st, 2);
#pragma unroll
                            for (int c = 0; c < 4; c++) {
                                if (!((uy >> c) & 1)) continue;
                                float v = fsub(vy.v[c], fmul(clch, d27[c]));
                                if (sxh >= 0)
                                    v = fadd(v, sterm(T0, sxh, ps1[c], d4h(e0z.v[c], e1z.v[c], e2z.v[c], e3z.v[c]), cl, p.ch));
                                if (szh[c] >= 0)
                                    v = fsub(v, sterm(T2, szh[c], ps2[c], d4h(wx.at(c - 2), wx.at(c - 1), wx.at(c), wx.at(c + 1)), cl, p.ch));
                                vy.v[c] = v;
                            }
                        }
                        if (own) {
#pragma unroll
                            for (int c = 0; c < 4; c++) {
                                if (!((uy >> c) & 1)) continue;
                                if (sxh >= 0) p.psi_h_out[0][offx + c] = ps1[c];
                                if (szh[c] >= 0) p.psi_h_out[5][offz + szh[c]] = ps2[c];
                            }
                        }
                    }
                    {   // hz: ey along x (queue), ex along y (plane m); x term subtracted, y term added
                        float ps1[4], ps2[4], d27[4];
#pragma unroll
                        for (int c = 0; c < 4; c++) {
                            const bool up = (uz >> c) & 1;
                            ps1[c] = up && sxh >= 0 ? __ldg(p.psi_h_in[1] + offx + c) : 0.f;
                            ps2[c] = up && syh >= 0 ? __ldg(p.psi_h_in[2] + offy + c) : 0.f;
                            const float n = curl4(e2y.v[c], e1y.v[c], e2x.v[c], exm1.v[c]);
                            const float f = curl4(e3y.v[c], e0y.v[c], exp1.v[c], exm2.v[c]);
                            d27[c] = fsub(fmul(27.0f, n), f);
                        }
#pragma unroll
                        for (int st = 0; st < (HH ? 2 : 1); st++) {
                            const float clch = st ? p.clch_b : p.clch_a, cl = st ? p.cl_b : p.cl_a;
                            const Tab T0 = tab_h(p, st, 0), T1 = tab_h(p, st, 1);
#pragma unroll
                            for (int c = 0; c < 4; c++) {
                                if (!((uz >> c) & 1)) continue;
                                float v = fsub(vz.v[c], fmul(clch, d27[c]));
                                if (sxh >= 0)
                                    v = fsub(v, sterm(T0, sxh, ps1[c], d4h(e0y.v[c], e1y.v[c], e2y.v[c], e3y.v[c]), cl, p.ch));
                                if (syh >= 0)
                                    v = fadd(v, sterm(T1, syh, ps2[c], d4h(exm2.v[c], exm1.v[c], e2x.v[c], exp1.v[c]), cl, p.ch));
                                vz.v[c] = v;
                            }
                        }
                        if (own) {
#pragma unroll
                            for (int c = 0; c < 4; c++) {
                                if (!((uz >> c) & 1)) continue;
                                if (sxh >= 0) p.psi_h_out[1][offx + c] = ps1[c];
                                if (syh >= 0) p.psi_h_out[2][offy + c] = ps2[c];
                            }
                        }
                    }
                }
                const int nsl = (m - (x0 - 1)) % NHN;
                sts4(sN(nsl, 0) + ho, vx);
                sts4(sN(nsl, 1) + ho, vy);
                sts4(sN(nsl, 2) + ho, vz);
                hny = vy;
                hnz = vz;
                if (own) {
                    const uint32_t rowo = (uint32_t)m * p.sx + (uint32_t)j * p.sy;
                    stg4(p.out[3] + rowo, kg, p.nz, vx);
                    stg4(p.out[4] + rowo, kg, p.nz, vy);
                    stg4(p.out[5] + rowo, kg, p.nz, vz);
                }
            }

            // ---- E_new(i), i = p - 3, at tile groups ----
            const int i = pl - 3;
            if (q >= 6 && e_thread && row_in && (k_in & 1)) {
                // H_new at planes i-1 .. i+2 of this group: n0 (i-1), n1 (i), n2 (i+1), hn (i+2);
                // H_new(i) neighbours from the ring (written two iterations ago)
                const int nsl = (i - (x0 - 1)) % NHN, nsl2 = (i + 1 - (x0 - 1)) % NHN;
                const float *hx = sN(nsl, 0), *hy = sN(nsl, 1), *hz = sN(nsl, 2);
                const V4 n1y = lds4(hy + ho), n1z = lds4(hz + ho);                      // plane i
                const V4 n2y = lds4(sN(nsl2, 1) + ho), n2z = lds4(sN(nsl2, 2) + ho);  // plane i+1
                const int cS = cslot(q);
                const V4 cvx = lds4(sC(cS, 0) + co), cvy = lds4(sC(cS, 1) + co), cvz = lds4(sC(cS, 2) + co);
                // rows j-1, j+1, j+2 of hz (ex) and hx (ez); z windows of hy (ex) and hx (ey)
                const V4 hzm1 = lds4(hz + ho - BW), hzp1 = lds4(hz + ho + BW), hzp2 = lds4(hz + ho + 2 * BW);
                const V4 hxm1 = lds4(hx + ho - BW), hxp1 = lds4(hx + ho + BW), hxp2 = lds4(hx + ho + 2 * BW);
                const ZW wy{lds4(hy + ho - 4), n1y, lds4(hy + ho + 4)};
                const ZW wx{lds4(hx + ho - 4), lds4(hx + ho), lds4(hx + ho + 4)};
                V4 vx = e0x, vy = e0y, vz = e0z;  // input E of plane i
                const bool iin = i > 0 && i < p.nx - 2;
                const int sxe = p.cpml ? slab(p.ea[0], i, p.nx, true) : -1;
                if (!yz_e && sxe < 0) {
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        {   // ex: hz along y, hy along z (plane i)
                            const float n = curl4(hzp1.v[c], n1z.v[c], wy.at(c + 1), n1y.v[c]);
                            const float f = curl4(hzp2.v[c], hzm1.v[c], wy.at(c + 2), wy.at(c - 1));
                            const float v = fadd(vx.v[c], fmul(fmul(p.dl, cvx.v[c]), fsub(fmul(27.0f, n), f)));
                            if (jin_e && ((kin_e >> c) & 1)) vx.v[c] = v;
                        }
                        {   // ey: hx along z (plane i), hz along x (queue)
                            const float n = curl4(wx.at(c + 1), wx.at(c), n2z.v[c], n1z.v[c]);
                            const float f = curl4(wx.at(c + 2), wx.at(c - 1), hnz.v[c], n0z.v[c]);
                            const float v = fadd(vy.v[c], fmul(fmul(p.dl, cvy.v[c]), fsub(fmul(27.0f, n), f)));
                            if (iin && ((kin_e >> c) & 1)) vy.v[c] = v;
                        }
                        {   // ez: hy along x (queue), hx along y (plane i)
                            const float n = curl4(n2y.v[c], n1y.v[c], hxp1.v[c], wx.at(c));
                            const float f = curl4(hny.v[c], n0y.v[c], hxp2.v[c], hxm1.v[c]);
                            const float v = fadd(vz.v[c], fmul(fmul(p.dl, cvz.v[c]), fsub(fmul(27.0f, n), f)));
                            if (iin && jin_e) vz.v[c] = v;
                        }
                    }
                } else {
                    // CPML path (E psi in place: only this thread touches these values)
                    const uint32_t ux = jin_e ? kin_e : 0u, uy = iin ? kin_e : 0u, uz = iin && jin_e ? k_in : 0u;
                    const uint32_t offx = sxe >= 0 ? ((uint32_t)sxe * p.ny + j) * p.nz + kg : 0u;
                    const uint32_t offy = sye >= 0 ? ((uint32_t)i * (2u * p.ea[1].P) + sye) * p.nz + kg : 0u;
                    const uint32_t offz = ((uint32_t)i * p.ny + j) * (2u * p.ea[2].P);
                    int sze[4];
#pragma unroll
                    for (int c = 0; c < 4; c++) sze[c] = slab(p.ea[2], kg + c, p.nz, true);
                    const Tab T0 = tab(p.ea[0]), T1 = tab(p.ea[1]), T2 = tab(p.ea[2]);
                    {   // ex: hz along y, hy along z; y term added, z term subtracted
                        float ps1[4], ps2[4];
#pragma unroll
                        for (int c = 0; c < 4; c++) {
                            const bool up = (ux >> c) & 1;
                            ps1[c] = up && sye >= 0 ? p.psi_e[3][offy + c] : 0.f;
                            ps2[c] = up && sze[c] >= 0 ? p.psi_e[4][offz + sze[c]] : 0.f;
                        }
#pragma unroll
                        for (int c = 0; c < 4; c++) {
                            if (!((ux >> c) & 1)) continue;
                            const float n = curl4(hzp1.v[c], n1z.v[c], wy.at(c + 1), n1y.v[c]);
                            const float f = curl4(hzp2.v[c], hzm1.v[c], wy.at(c + 2), wy.at(c - 1));
                            const float cv = cvx.v[c];
                            float v = fadd(vx.v[c], fmul(fmul(p.dl, cv), fsub(fmul(27.0f, n), f)));
                            if (sye >= 0) {
                                v = fadd(v, sterm(T1, sye, ps1[c], d4e(hzm1.v[c], n1z.v[c], hzp1.v[c], hzp2.v[c]), p.dl, cv));
                                p.psi_e[3][offy + c] = ps1[c];
                            }
                            if (sze[c] >= 0) {
                                v = fsub(v, sterm(T2, sze[c], ps2[c], d4e(wy.at(c - 1), n1y.v[c], wy.at(c + 1), wy.at(c + 2)), p.dl, cv));
                                p.psi_e[4][offz + sze[c]] = ps2[c];
                            }
                            vx.v[c] = v;
                        }
                    }
                    {   // ey: hx along z (plane i), hz along x (queue); x term subtracted, z term added
                        float ps1[4], ps2[4];
#pragma unroll
                        for (int c = 0; c < 4; c++) {
                            const bool up = (uy >> c) & 1;
                            ps1[c] = up && sxe >= 0 ? p.psi_e[0][offx + c] : 0.f;
                            ps2[c] = up && sze[c] >= 0 ? p.psi_e[5][offz + sze[c]] : 0.f;
                        }
#pragma unroll
                        for (int c = 0; c < 4; c++) {
                            if (!((uy >> c) & 1)) continue;
                            const float n = curl4(wx.at(c + 1), wx.at(c), n2z.v[c], n1z.v[c]);
                            const float f = curl4(wx.at(c + 2), wx.at(c - 1), hnz.v[c], n0z.v[c]);
                            const float cv = cvy.v[c];
                            float v = fadd(vy.v[c], fmul(fmul(p.dl, cv), fsub(fmul(27.0f, n), f)));
                            if (sxe >= 0) {
                                v = fsub(v, sterm(T0, sxe, ps1[c], d4e(n0z.v[c], n1z.v[c], n2z.v[c], hnz.v[c]), p.dl, cv));
                                p.psi_e[0][offx + c] = ps1[c];
                            }
                            if (sze[c] >= 0) {
                                v = fadd(v, sterm(T2, sze[c], ps2[c], d4e(wx.at(c - 1), wx.at(c), wx.at(c + 1), wx.at(c + 2)), p.dl, cv));
                                p.psi_e[5][offz + sze[c]] = ps2[c];
                            }
                            vy.v[c] = v;
                        }
                    }
                    {   // ez: hy along x (queue), hx along y (plane i); x term added, y term subtracted
                        float ps1[4], ps2[4];
#pragma unroll
                        for (int c = 0; c < 4; c++) {
                            const bool up = (uz >> c) & 1;
                            ps1[c] = up && sxe >= 0 ? p.psi_e[1][offx + c] : 0.f;
                            ps2[c] = up && sye >= 0 ? p.psi_e[2][offy + c] : 0.f;
                        }
#pragma unroll
                        for (int c = 0; c < 4; c++) {
                            if (!((uz >> c) & 1)) continue;
                            const float n = curl4(n2y.v[c], n1y.v[c], hxp1.v[c], wx.at(c));
                            const float f = curl4(hny.v[c], n0y.v[c], hxp2.v[c], hxm1.v[c]);
                            const float cv = cvz.v[c];
                            float v = fadd(vz.v[c], fmul(fmul(p.dl, cv), fsub(fmul(27.0f, n), f)));
                            if (sxe >= 0) {
                                v = fadd(v, sterm(T0, sxe, ps1[c], d4e(n0y.v[c], n1y.v[c], n2y.v[c], hny.v[c]), p.dl, cv));
                                p.psi_e[1][offx + c] = ps1[c];
                            }
                            if (sye >= 0) {
                                v = fsub(v, sterm(T1, sye, ps2[c], d4e(hxm1.v[c], wx.at(c), hxp1.v[c], hxp2.v[c]), p.dl, cv));
                                p.psi_e[2][offy + c] = ps2[c];
                            }
                            vz.v[c] = v;
                        }
                    }
                }
                for (int s = 0; s < nls; s++) {  // soft sources, list order
                    const int sk = s_ls_kc[s] >> 2;
                    if (s_ls_i[s] != i || s_ls_j[s] != j || sk < kg || sk >= kg + 4) continue;
                    const float v = p.src_amp[(int64_t)s_ls_s[s] * p.namp + p.t];
                    const int comp = s_ls_kc[s] & 3, c = sk - kg;
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        if (u != c) continue;
                        if (comp == 0) vx.v[u] = fadd(vx.v[u], v);
                        else if (comp == 1) vy.v[u] = fadd(vy.v[u], v);
                        else vz.v[u] = fadd(vz.v[u], v);
                    }
                }
                const uint32_t rowo = (uint32_t)i * p.sx + (uint32_t)j * p.sy;
                stg4(p.out[0] + rowo, kg, p.nz, vx);
                stg4(p.out[1] + rowo, kg, p.nz, vy);
                stg4(p.out[2] + rowo, kg, p.nz, vz);
            }
            // advance the queue
            e0x = e1x; e0y = e1y; e0z = e1z;
            e1x = e2x; e1y = e2y; e1z = e2z;
        }
        if (aborted) {
            if (producer) {
                atomicExch(p.status, FDTD_ERR_TIMEOUT);
                // let the copies in flight land before the shared memory is
                // released (E and H of iterations q, q+1; CE of iteration q),
                // each wait bounded
                for (int q = q_abort; q < Q && q < q_abort + 2; q++) {
                    mbar_wait(&bars[eslot(q)], ephase(q), nullptr);
                    if (q >= 3) mbar_wait(&bars[NE + hslot(q)], hphase(q), nullptr);
                }
                if (q_abort >= 6) mbar_wait(&bars[NE + NH + cslot(q_abort)], cphase(q_abort), nullptr);
            }
            break;
        }
        gE += (uint32_t)Q;
        gH += (uint32_t)(Q - 3);
        gC += (uint32_t)(Q - 6);
        // every thread read s_item before this item's first barrier
        if (tid == 0) s_item = atomicAdd(&p.queue[0], 1);
        __syncthreads();
        item = s_item;
    }
    if (aborted) __syncthreads();
    if (tid == 0) {
        // the last CTA to finish clears the queue for the next launch
        __threadfence();
        if (atomicAdd(&p.queue[1], 1) == (int)gridDim.x - 1) {
            p.queue[0] = 0;
            p.queue[1] = 0;
            __threadfence();
        }
    }
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
                               int32_t *queue_dev, void *stream) {
    if (!out || !s || !status_dev || !queue_dev || (cur != 0 && cur != 1)) return FDTD_ERR_ARG;
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
    p.queue = queue_dev;
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
    int occ1 = 0;
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute((const void *)k_symp_pair<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute((const void *)k_symp_pair<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void *)k_symp_pair<false>, THREADS, SMEM);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ1, (const void *)k_symp_pair<true>, THREADS, SMEM);
    occ = std::min(occ, occ1);
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
                if (ax > 0) p.edge_first = 1;
            }
            dst[w][ax] = A;
        }
    }
    if (two_h)
        k_symp_pair<true><<<pl->nblocks, THREADS, SMEM, as_stream(stream)>>>(pl->maps[in], p);
    else
        k_symp_pair<false><<<pl->nblocks, THREADS, SMEM, as_stream(stream)>>>(pl->maps[in], p);
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
