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
// Design: the pair kernel on the grid's inside, edge kernels on a thin shell
//  * Ping-pong state: a pass reads buffer `cur` (E, H) and writes `1-cur`;
//    the H psi slabs ping-pong too, the E psi slabs are updated in place
//    (only their owner touches them).
//  * Split: the pair kernel owns rows [j_lo, j_hi) and columns [k_lo, k_hi),
//    every x plane, with j_lo = P+2 and j_hi = ny-P-2 (and the same along z,
//    k_lo rounded up to 4): E_new there needs H_new of rows j_lo-1 .. j_hi+1,
//    where no y or z CPML node lies.  So the pair kernel carries the x-slab
//    terms only.  The rest of the grid (the y and z slabs plus two cells) is
//    the edge shell, advanced by one-thread-per-cell kernels (k_edge_*), out
//    of place, after the pair kernel has written the inside H_new.
//  * Pair kernel, 2.5-D blocking: a CTA owns TZ = 32 (z) x TY = 16 (y) cells
//    for a chunk of x planes and marches along x.  E_new(i) needs H_new on
//    planes i-1 .. i+2 and on the rows/columns -1 .. +2 around the tile, so
//    H_new is computed on the rows j0-1 .. j0+TY+1 and the columns
//    k0-4 .. k0+TZ+3, in groups of 4 z cells: one thread per group, the 128
//    tile groups first (those threads also compute E_new of their group),
//    then the 62 halo groups.  Every group is 16-byte aligned, so its z window
//    (the group and the neighbouring groups) is three 16-byte shared loads.
//    z tiles keep TZ-column boundaries (128-byte rows); cells outside the
//    kernel's columns are computed but not written.
//  * Registers hold the input E of planes p-3 and p-2 of the group; shared
//    memory holds one plane with its y/z halo: input E boxes (4-slot ring)
//    and H boxes (3-slot ring), both issued two planes ahead, CE boxes (2-slot
//    ring, one plane ahead) and H_new (3-slot ring).  About 108 KB, two CTAs
//    per SM.
//  * Iteration q: input plane p arrives; every thread computes H_new(p-1) for
//    its group; tile threads then compute E_new(p-3).  One CTA barrier per
//    iteration: H_new(p-1) is read by neighbours two iterations later.
//  * CTAs draw work items from a device queue (two ints the caller provides,
//    cleared by the last CTA of each launch).
//  * Lane 31 of the last warp is the producer: it waits on the mbarriers and
//    issues the copies.  Every wait is bounded (1 s); on expiry the CTA
//    records FDTD_ERR_TIMEOUT, drains its copies and stops.
#include <cuda.h>

#include <algorithm>
#include <functional>
#include <queue>
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
    // this kernel's region: rows [j_lo, j_hi), columns [k_lo, k_hi) (k_lo a
    // multiple of 4), every x plane, tiled from (j_lo, k_lo) into nty_in x
    // ntz_in tiles; its H regions hold no y or z CPML node.  The rest of the
    // grid is the edge shell of the edge kernels.
    int32_t j_lo, j_hi, k_lo, k_hi, nty_in, ntz_in;
    int32_t kt0;              // first z tile origin (k_lo rounded down to TZ)
    const float *in[6];       // ex, ey, ez, hx, hy, hz of the input buffer (edge kernels)
    const float *ce[3];
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

// extents (elements) of a field array and of a psi slab array along axis ax
// with P cells per face, for the bounds-checked build
__device__ __forceinline__ int64_t fext(const Params &p) { return (int64_t)p.nx * p.sx; }
__device__ __forceinline__ int64_t pext(const Params &p, int ax, int P) {
    return ax == 0 ? 2LL * P * p.ny * p.nz : (ax == 1 ? 2LL * p.nx * P * p.nz : 2LL * p.nx * p.ny * P);
}
// a read-only global load through the non-coherent path, checked in the debug build
#define LDG(a, i, n) (FDTD_IN(i, n) ? __ldg((a) + (i)) : 0.f)

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

// global store of a group's 4 values (elements g .. g+3 of a field array of
// n elements): the cells whose bit is set in mask (all four: one 16-byte store)
__device__ __forceinline__ void stg4(float *f, int64_t g, uint32_t mask, const V4 &a, int64_t n) {
    if (mask == 0xFu) {
        if (FDTD_IN(g + 3, n) && FDTD_IN(g, n))
            *reinterpret_cast<float4 *>(f + g) = make_float4(a.v[0], a.v[1], a.v[2], a.v[3]);
    } else {
#pragma unroll
        for (int c = 0; c < 4; c++)
            if (((mask >> c) & 1) && FDTD_IN(g + c, n)) f[g + c] = a.v[c];
    }
}

// Work item u -> tile (tzi, tyi) and x chunk xci over the kernel's tiles:
// z tile fastest, then y tile, then x chunk.
__device__ __forceinline__ void item_tile(const Params &p, int u, int &tzi, int &tyi, int &xci) {
    tzi = u % p.ntz_in;
    tyi = (u / p.ntz_in) % p.nty_in;
    xci = u / (p.ntz_in * p.nty_in);
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
    const int64_t nitems = (int64_t)p.ntz_in * p.nty_in * p.nxc;
    // items from the work queue: CTAs that drew cheaper items (no x slab
    // plane, no source) take more of them
    if (tid == 0) s_item = atomicAdd(&p.queue[0], 1);
    __syncthreads();
    for (int64_t item = s_item; item < nitems && !aborted;) {
        int tzi, tyi, xci;
        item_tile(p, (int)item, tzi, tyi, xci);
        const int k0 = p.kt0 + tzi * TZ, j0 = p.j_lo + tyi * TY, x0 = xci * p.x_chunk;
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
                    if (si >= x0 && si < x1 && sj >= j0 && sj < min(j0 + TY, p.j_hi) && sk >= max(k0, p.k_lo) &&
                        sk < min(k0 + TZ, p.k_hi)) {
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
        const bool own_row = e_thread && row_in && j < p.j_hi;  // rows this kernel writes
        const bool jin_h = j > 1 && j < p.ny - 1, jin_e = j > 0 && j < p.ny - 2;
        // per-cell z masks of the group (bit c: cell kg+c); kown: cells this kernel writes
        const int kmax = min(p.nz, p.k_hi);
        uint32_t kin_h = 0, kin_e = 0, k_in = 0, kown = 0;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const int k = kg + c;
            kin_h |= (uint32_t)(k > 1 && k < p.nz - 1) << c;
            kin_e |= (uint32_t)(k > 0 && k < p.nz - 2) << c;
            k_in |= (uint32_t)(k >= 0 && k < p.nz) << c;
            kown |= (uint32_t)(own_row && k >= p.k_lo && k < kmax) << c;
        }

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
            // The kernel's tiles meet no y or z slab; on an x-slab plane hy and
            // hz take their x term after the main term (the operation order of
            // the stage kernels), stage by stage.
            const int m = pl - 1;
            V4 hny{}, hnz{};
            if (q >= 3 && row_in && m >= 0 && m < p.nx) {
                const int eSm = eslot(q - 1), hS = hslot(q);
                const float *ex = sE(eSm, 0), *ey = sE(eSm, 1), *ez = sE(eSm, 2);
                V4 vx = lds4(sH(hS, 0) + ho), vy = lds4(sH(hS, 1) + ho), vz = lds4(sH(hS, 2) + ho);
                // rows j-2, j-1, j+1 of ez (hx) and ex (hz); z windows of ey (hx) and ex (hy)
                const V4 ezm2 = lds4(ez + eo - 2 * BW), ezm1 = lds4(ez + eo - BW), ezp1 = lds4(ez + eo + BW);
                const V4 exm2 = lds4(ex + eo - 2 * BW), exm1 = lds4(ex + eo - BW), exp1 = lds4(ex + eo + BW);
                const ZW wy{lds4(ey + eo - col + colL), e2y, lds4(ey + eo - col + colR)};
                const ZW wx{lds4(ex + eo - col + colL), e2x, lds4(ex + eo - col + colR)};
                const bool iin = m > 1 && m < p.nx - 1;
                const bool own = own_row && m >= x0 && m < x1;
                const int sxh = p.cpml ? slab(p.ha[0], m, p.nx, false) : -1;  // uniform over the CTA
                const uint32_t ux = jin_h ? kin_h : 0u, uy = iin ? kin_h : 0u, uz = iin && jin_h ? k_in : 0u;
                const uint32_t offx = sxh >= 0 ? ((uint32_t)sxh * p.ny + j) * p.nz + kg : 0u;
                float py[4], pz[4];  // x psi of hy and hz (x-slab planes)
                if (sxh >= 0) {
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        py[c] = (uy >> c) & 1 ? LDG(p.psi_h_in[0], offx + c, pext(p, 0, p.ha[0].P)) : 0.f;
                        pz[c] = (uz >> c) & 1 ? LDG(p.psi_h_in[1], offx + c, pext(p, 0, p.ha[0].P)) : 0.f;
                    }
                }
                if (sxh < 0) {
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        {   // hx: ez along y, ey along z (plane m)
                            const float n = curl4(e2z.v[c], ezm1.v[c], wy.at(c), wy.at(c - 1));
                            const float f = curl4(ezp1.v[c], ezm2.v[c], wy.at(c + 1), wy.at(c - 2));
                            const float d27 = fsub(fmul(27.0f, n), f);
                            float v = fsub(vx.v[c], fmul(p.clch_a, d27));
                            if (HH) v = fsub(v, fmul(p.clch_b, d27));
                            if ((ux >> c) & 1) vx.v[c] = v;
                        }
                        {   // hy: ex along z (plane m), ez along x (queue); x term added
                            const float n = curl4(e2x.v[c], wx.at(c - 1), e2z.v[c], e1z.v[c]);
                            const float f = curl4(wx.at(c + 1), wx.at(c - 2), e3z.v[c], e0z.v[c]);
                            const float d27 = fsub(fmul(27.0f, n), f);
                            float v = fsub(vy.v[c], fmul(p.clch_a, d27));
                            if (HH) v = fsub(v, fmul(p.clch_b, d27));
                            if ((uy >> c) & 1) vy.v[c] = v;
                        }
                        {   // hz: ey along x (queue), ex along y (plane m); x term subtracted
                            const float n = curl4(e2y.v[c], e1y.v[c], e2x.v[c], exm1.v[c]);
                            const float f = curl4(e3y.v[c], e0y.v[c], exp1.v[c], exm2.v[c]);
                            const float d27 = fsub(fmul(27.0f, n), f);
                            float v = fsub(vz.v[c], fmul(p.clch_a, d27));
                            if (HH) v = fsub(v, fmul(p.clch_b, d27));
                            if ((uz >> c) & 1) vz.v[c] = v;
                        }
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        {   // hx: ez along y, ey along z (plane m)
                            const float n = curl4(e2z.v[c], ezm1.v[c], wy.at(c), wy.at(c - 1));
                            const float f = curl4(ezp1.v[c], ezm2.v[c], wy.at(c + 1), wy.at(c - 2));
                            const float d27 = fsub(fmul(27.0f, n), f);
                            float v = fsub(vx.v[c], fmul(p.clch_a, d27));
                            if (HH) v = fsub(v, fmul(p.clch_b, d27));
                            if ((ux >> c) & 1) vx.v[c] = v;
                        }
                        {   // hy: ex along z (plane m), ez along x (queue); x term added
                            const float n = curl4(e2x.v[c], wx.at(c - 1), e2z.v[c], e1z.v[c]);
                            const float f = curl4(wx.at(c + 1), wx.at(c - 2), e3z.v[c], e0z.v[c]);
                            const float d27 = fsub(fmul(27.0f, n), f);
                            float v = fsub(vy.v[c], fmul(p.clch_a, d27));
                            if (sxh >= 0) {
                                const float d = d4h(e0z.v[c], e1z.v[c], e2z.v[c], e3z.v[c]);
                                v = fadd(v, sterm(tab(p.ha[0]), sxh, py[c], d, p.cl_a, p.ch));
                                if (HH) {
                                    v = fsub(v, fmul(p.clch_b, d27));
                                    v = fadd(v, sterm(tab(p.hb[0]), sxh, py[c], d, p.cl_b, p.ch));
                                }
                            } else if (HH) {
                                v = fsub(v, fmul(p.clch_b, d27));
                            }
                            if ((uy >> c) & 1) vy.v[c] = v;
                        }
                        {   // hz: ey along x (queue), ex along y (plane m); x term subtracted
                            const float n = curl4(e2y.v[c], e1y.v[c], e2x.v[c], exm1.v[c]);
                            const float f = curl4(e3y.v[c], e0y.v[c], exp1.v[c], exm2.v[c]);
                            const float d27 = fsub(fmul(27.0f, n), f);
                            float v = fsub(vz.v[c], fmul(p.clch_a, d27));
                            if (sxh >= 0) {
                                const float d = d4h(e0y.v[c], e1y.v[c], e2y.v[c], e3y.v[c]);
                                v = fsub(v, sterm(tab(p.ha[0]), sxh, pz[c], d, p.cl_a, p.ch));
                                if (HH) {
                                    v = fsub(v, fmul(p.clch_b, d27));
                                    v = fsub(v, sterm(tab(p.hb[0]), sxh, pz[c], d, p.cl_b, p.ch));
                                }
                            } else if (HH) {
                                v = fsub(v, fmul(p.clch_b, d27));
                            }
                            if ((uz >> c) & 1) vz.v[c] = v;
                        }
                    }
                }
                if (own && sxh >= 0) {
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        if (((uy & kown) >> c & 1) && FDTD_IN(offx + c, pext(p, 0, p.ha[0].P)))
                            p.psi_h_out[0][offx + c] = py[c];
                        if (((uz & kown) >> c & 1) && FDTD_IN(offx + c, pext(p, 0, p.ha[0].P)))
                            p.psi_h_out[1][offx + c] = pz[c];
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
                    stg4(p.out[3], (int64_t)rowo + kg, kown, vx, fext(p));
                    stg4(p.out[4], (int64_t)rowo + kg, kown, vy, fext(p));
                    stg4(p.out[5], (int64_t)rowo + kg, kown, vz, fext(p));
                }
            }

            // ---- E_new(i), i = p - 3, at tile groups ----
            const int i = pl - 3;
            if (q >= 6 && own_row && kown) {
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
                const int sxe = p.cpml ? slab(p.ea[0], i, p.nx, true) : -1;  // uniform over the CTA
                const uint32_t ux = jin_e ? kin_e : 0u, uy = (iin ? kin_e : 0u) & kown,
                               uz = (iin && jin_e ? k_in : 0u) & kown;
                const uint32_t offx = sxe >= 0 ? ((uint32_t)sxe * p.ny + j) * p.nz + kg : 0u;
                float py[4], pz[4];  // x psi of ey and ez (x-slab planes), in place
                if (sxe >= 0) {
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        py[c] = ((uy >> c) & 1) && FDTD_IN(offx + c, pext(p, 0, p.ea[0].P)) ? p.psi_e[0][offx + c] : 0.f;
                        pz[c] = ((uz >> c) & 1) && FDTD_IN(offx + c, pext(p, 0, p.ea[0].P)) ? p.psi_e[1][offx + c] : 0.f;
                    }
                }
                if (sxe < 0) {
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        {   // ex: hz along y, hy along z (plane i)
                            const float n = curl4(hzp1.v[c], n1z.v[c], wy.at(c + 1), n1y.v[c]);
                            const float f = curl4(hzp2.v[c], hzm1.v[c], wy.at(c + 2), wy.at(c - 1));
                            const float v = fadd(vx.v[c], fmul(fmul(p.dl, cvx.v[c]), fsub(fmul(27.0f, n), f)));
                            if ((ux >> c) & 1) vx.v[c] = v;
                        }
                        {   // ey: hx along z (plane i), hz along x; x term subtracted
                            const float n = curl4(wx.at(c + 1), wx.at(c), n2z.v[c], n1z.v[c]);
                            const float f = curl4(wx.at(c + 2), wx.at(c - 1), hnz.v[c], n0z.v[c]);
                            const float cv = cvy.v[c];
                            float v = fadd(vy.v[c], fmul(fmul(p.dl, cv), fsub(fmul(27.0f, n), f)));
                            if ((uy >> c) & 1) vy.v[c] = v;
                        }
                        {   // ez: hy along x, hx along y (plane i); x term added
                            const float n = curl4(n2y.v[c], n1y.v[c], hxp1.v[c], wx.at(c));
                            const float f = curl4(hny.v[c], n0y.v[c], hxp2.v[c], hxm1.v[c]);
                            const float cv = cvz.v[c];
                            float v = fadd(vz.v[c], fmul(fmul(p.dl, cv), fsub(fmul(27.0f, n), f)));
                            if ((uz >> c) & 1) vz.v[c] = v;
                        }
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        {   // ex: hz along y, hy along z (plane i)
                            const float n = curl4(hzp1.v[c], n1z.v[c], wy.at(c + 1), n1y.v[c]);
                            const float f = curl4(hzp2.v[c], hzm1.v[c], wy.at(c + 2), wy.at(c - 1));
                            const float v = fadd(vx.v[c], fmul(fmul(p.dl, cvx.v[c]), fsub(fmul(27.0f, n), f)));
                            if ((ux >> c) & 1) vx.v[c] = v;
                        }
                        {   // ey: hx along z (plane i), hz along x; x term subtracted
                            const float n = curl4(wx.at(c + 1), wx.at(c), n2z.v[c], n1z.v[c]);
                            const float f = curl4(wx.at(c + 2), wx.at(c - 1), hnz.v[c], n0z.v[c]);
                            const float cv = cvy.v[c];
                            float v = fadd(vy.v[c], fmul(fmul(p.dl, cv), fsub(fmul(27.0f, n), f)));
                            if (sxe >= 0)
                                v = fsub(v, sterm(tab(p.ea[0]), sxe, py[c], d4e(n0z.v[c], n1z.v[c], n2z.v[c], hnz.v[c]), p.dl, cv));
                            if ((uy >> c) & 1) vy.v[c] = v;
                        }
                        {   // ez: hy along x, hx along y (plane i); x term added
                            const float n = curl4(n2y.v[c], n1y.v[c], hxp1.v[c], wx.at(c));
                            const float f = curl4(hny.v[c], n0y.v[c], hxp2.v[c], hxm1.v[c]);
                            const float cv = cvz.v[c];
                            float v = fadd(vz.v[c], fmul(fmul(p.dl, cv), fsub(fmul(27.0f, n), f)));
                            if (sxe >= 0)
                                v = fadd(v, sterm(tab(p.ea[0]), sxe, pz[c], d4e(n0y.v[c], n1y.v[c], n2y.v[c], hny.v[c]), p.dl, cv));
                            if ((uz >> c) & 1) vz.v[c] = v;
                        }
                    }
                }
                if (sxe >= 0) {
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        if (((uy >> c) & 1) && FDTD_IN(offx + c, pext(p, 0, p.ea[0].P))) p.psi_e[0][offx + c] = py[c];
                        if (((uz >> c) & 1) && FDTD_IN(offx + c, pext(p, 0, p.ea[0].P))) p.psi_e[1][offx + c] = pz[c];
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
                stg4(p.out[0], (int64_t)rowo + kg, kown, vx, fext(p));
                stg4(p.out[1], (int64_t)rowo + kg, kown, vy, fext(p));
                stg4(p.out[2], (int64_t)rowo + kg, kown, vz, fext(p));
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

// ---------------------------------------------------------------------------
// Edge shell: the cells outside the pair kernel's tiles (the y and z CPML
// slabs and a tile of margin), one thread per cell, out of place:
//   k_edge_h         H_out = H_in - clch_a curl4(E_in) with its CPML terms
//                    (psi_h_in -> psi_h_out); in a two-H pass the second
//                    stage follows in registers (same E_in, psi carried);
//   k_edge_e         E_out = E_in + dl ce curl4(H_out) with its CPML terms
//                    (psi_e in place), once the pair kernel has written the
//                    interior H_out;
//   k_edge_src       the soft sources on edge cells, in list order.
// Same expressions and operation order as the stage kernels.  The pair
// kernel's tiles never read a y or z slab cell, so the two parts meet only
// through H_out, which k_edge_e reads after both have written it.
// ---------------------------------------------------------------------------
struct Edge {
    int32_t n;                           // boxes
    int32_t j0[4], j1[4], k0[4], k1[4];  // rows [j0, j1), columns [k0, k1), every x plane
    uint32_t off[5];                     // first cell of each box within one x plane
    uint32_t rcp[4];                     // ceil(2^32 / width) of each box (division by the width)
};
constexpr int EDGE_BLOCK = 128;

// launch: blockIdx.y = x plane, blockIdx.x * EDGE_BLOCK + threadIdx.x = cell of
// the plane's part of the shell (box by box, z fastest)
__device__ __forceinline__ bool edge_cell(const Edge &eb, int &i, int &j, int &k) {
    const uint32_t u = blockIdx.x * EDGE_BLOCK + threadIdx.x;
    if (u >= eb.off[eb.n]) return false;
    int b = 0;
    while (b + 1 < eb.n && u >= eb.off[b + 1]) b++;
    const uint32_t v = u - eb.off[b], nk = (uint32_t)(eb.k1[b] - eb.k0[b]);
    uint32_t r = __umulhi(v, eb.rcp[b]);  // v / nk, or one off
    if (r * nk > v) r--;
    else if ((r + 1) * nk <= v) r++;
    k = eb.k0[b] + (int)(v - r * nk);
    j = eb.j0[b] + (int)r;
    i = blockIdx.y;
    return true;
}

template <bool HH>
__global__ void __launch_bounds__(EDGE_BLOCK)
k_edge_h(const __grid_constant__ Params p, const __grid_constant__ Edge eb) {
    int i, j, k;
    if (!edge_cell(eb, i, j, k)) return;
    const uint32_t X = p.sx, Y = p.sy, c = (uint32_t)i * X + (uint32_t)j * Y + (uint32_t)k;
    const float *ex = p.in[0], *ey = p.in[1], *ez = p.in[2];
    [[maybe_unused]] const int64_t FE = fext(p);
    [[maybe_unused]] const int64_t PE0 = pext(p, 0, p.ha[0].P), PE1 = PE0, PE2 = pext(p, 1, p.ha[1].P),
                                   PE3 = PE2, PE4 = pext(p, 2, p.ha[2].P), PE5 = PE4;
    const bool jin = j > 1 && j < p.ny - 1, kin = k > 1 && k < p.nz - 1, iin = i > 1 && i < p.nx - 1;
    const int sx = slab(p.ha[0], i, p.nx, false), sy = slab(p.ha[1], j, p.ny, false),
              sz = slab(p.ha[2], k, p.nz, false);
    // One component: the input H, then per stage (a, then b in a two-H pass)
    // the main term and the two CPML terms (signs s1, s2: +1 adds), psi
    // carried from stage a to stage b in registers; E_in is the same for both
    // stages, so are d27 and the one-axis differences.
    auto comp = [&](int q, bool upd, float d27, int a1, int s1, int q1, float d1, int a2, int s2, int q2, float d2) {
        float v = LDG(p.in[3 + q], c, FE);
        if (upd) {
            const int sl1 = a1 == 0 ? sx : (a1 == 1 ? sy : sz), sl2 = a2 == 0 ? sx : (a2 == 1 ? sy : sz);
            [[maybe_unused]] const int64_t pe1 = a1 == 0 ? PE0 : (a1 == 1 ? PE2 : PE4),
                                           pe2 = a2 == 0 ? PE0 : (a2 == 1 ? PE2 : PE4);
            uint32_t i1 = 0, i2 = 0;
            float ps1 = 0.f, ps2 = 0.f;
            if (sl1 >= 0) {
                i1 = psi_index(p, a1, sl1, i, j, k, p.ha[a1].P);
                ps1 = FDTD_IN(i1, pe1) ? p.psi_h_in[q1][i1] : 0.f;
            }
            if (sl2 >= 0) {
                i2 = psi_index(p, a2, sl2, i, j, k, p.ha[a2].P);
                ps2 = FDTD_IN(i2, pe2) ? p.psi_h_in[q2][i2] : 0.f;
            }
#pragma unroll
            for (int st = 0; st < (HH ? 2 : 1); st++) {
                const float clch = st ? p.clch_b : p.clch_a, cl = st ? p.cl_b : p.cl_a;
                v = fsub(v, fmul(clch, d27));
                if (sl1 >= 0) {
                    const float t = sterm(tab_h(p, st, a1), sl1, ps1, d1, cl, p.ch);
                    v = s1 > 0 ? fadd(v, t) : fsub(v, t);
                }
                if (sl2 >= 0) {
                    const float t = sterm(tab_h(p, st, a2), sl2, ps2, d2, cl, p.ch);
                    v = s2 > 0 ? fadd(v, t) : fsub(v, t);
                }
            }
            if (sl1 >= 0 && FDTD_IN(i1, pe1)) p.psi_h_out[q1][i1] = ps1;
            if (sl2 >= 0 && FDTD_IN(i2, pe2)) p.psi_h_out[q2][i2] = ps2;
        }
        if (FDTD_IN(c, FE)) p.out[3 + q][c] = v;
    };
    {   // hx: y term subtracted, z term added
        float d27 = 0.f, dy = 0.f, dz = 0.f;
        if (jin && kin) {
            const float n = curl4(LDG(ez, c, FE), LDG(ez, c - Y, FE), LDG(ey, c, FE), LDG(ey, c - 1, FE));
            const float f = curl4(LDG(ez, c + Y, FE), LDG(ez, c - 2 * Y, FE), LDG(ey, c + 1, FE), LDG(ey, c - 2, FE));
            d27 = fsub(fmul(27.0f, n), f);
            if (sy >= 0) dy = d4h(LDG(ez, c - 2 * Y, FE), LDG(ez, c - Y, FE), LDG(ez, c, FE), LDG(ez, c + Y, FE));
            if (sz >= 0) dz = d4h(LDG(ey, c - 2, FE), LDG(ey, c - 1, FE), LDG(ey, c, FE), LDG(ey, c + 1, FE));
        }
        comp(0, jin && kin, d27, 1, -1, 3, dy, 2, +1, 4, dz);
    }
    {   // hy: x term added, z term subtracted
        float d27 = 0.f, dx = 0.f, dz = 0.f;
        if (iin && kin) {
            const float n = curl4(LDG(ex, c, FE), LDG(ex, c - 1, FE), LDG(ez, c, FE), LDG(ez, c - X, FE));
            const float f = curl4(LDG(ex, c + 1, FE), LDG(ex, c - 2, FE), LDG(ez, c + X, FE), LDG(ez, c - 2 * X, FE));
            d27 = fsub(fmul(27.0f, n), f);
            if (sx >= 0) dx = d4h(LDG(ez, c - 2 * X, FE), LDG(ez, c - X, FE), LDG(ez, c, FE), LDG(ez, c + X, FE));
            if (sz >= 0) dz = d4h(LDG(ex, c - 2, FE), LDG(ex, c - 1, FE), LDG(ex, c, FE), LDG(ex, c + 1, FE));
        }
        comp(1, iin && kin, d27, 0, +1, 0, dx, 2, -1, 5, dz);
    }
    {   // hz: x term subtracted, y term added
        float d27 = 0.f, dx = 0.f, dy = 0.f;
        if (iin && jin) {
            const float n = curl4(LDG(ey, c, FE), LDG(ey, c - X, FE), LDG(ex, c, FE), LDG(ex, c - Y, FE));
            const float f = curl4(LDG(ey, c + X, FE), LDG(ey, c - 2 * X, FE), LDG(ex, c + Y, FE), LDG(ex, c - 2 * Y, FE));
            d27 = fsub(fmul(27.0f, n), f);
            if (sx >= 0) dx = d4h(LDG(ey, c - 2 * X, FE), LDG(ey, c - X, FE), LDG(ey, c, FE), LDG(ey, c + X, FE));
            if (sy >= 0) dy = d4h(LDG(ex, c - 2 * Y, FE), LDG(ex, c - Y, FE), LDG(ex, c, FE), LDG(ex, c + Y, FE));
        }
        comp(2, iin && jin, d27, 0, -1, 1, dx, 1, +1, 2, dy);
    }
}

__global__ void __launch_bounds__(EDGE_BLOCK)
k_edge_e(const __grid_constant__ Params p, const __grid_constant__ Edge eb) {
    int i, j, k;
    if (!edge_cell(eb, i, j, k)) return;
    const uint32_t X = p.sx, Y = p.sy, c = (uint32_t)i * X + (uint32_t)j * Y + (uint32_t)k;
    const float *hx = p.out[3], *hy = p.out[4], *hz = p.out[5];
    [[maybe_unused]] const int64_t FE = fext(p);
    [[maybe_unused]] const int64_t PE0 = pext(p, 0, p.ea[0].P), PE1 = PE0, PE2 = pext(p, 1, p.ea[1].P),
                                   PE3 = PE2, PE4 = pext(p, 2, p.ea[2].P), PE5 = PE4;
    const Tab T0 = tab(p.ea[0]), T1 = tab(p.ea[1]), T2 = tab(p.ea[2]);
    const bool jin = j > 0 && j < p.ny - 2, kin = k > 0 && k < p.nz - 2, iin = i > 0 && i < p.nx - 2;
    const int sx = slab(p.ea[0], i, p.nx, true), sy = slab(p.ea[1], j, p.ny, true),
              sz = slab(p.ea[2], k, p.nz, true);
    {   // ex: y term added, z term subtracted
        float v = LDG(p.in[0], c, FE);
        if (jin && kin) {
            const float n = curl4(LDG(hz, c + Y, FE), LDG(hz, c, FE), LDG(hy, c + 1, FE), LDG(hy, c, FE));
            const float f = curl4(LDG(hz, c + 2 * Y, FE), LDG(hz, c - Y, FE), LDG(hy, c + 2, FE), LDG(hy, c - 1, FE));
            const float cv = LDG(p.ce[0], c, FE);
            v = fadd(v, fmul(fmul(p.dl, cv), fsub(fmul(27.0f, n), f)));
            if (sy >= 0) {
                const uint32_t q = psi_index(p, 1, sy, i, j, k, p.ea[1].P);
                float ps = FDTD_IN(q, PE3) ? p.psi_e[3][q] : 0.f;
                v = fadd(v, sterm(T1, sy, ps, d4e(LDG(hz, c - Y, FE), LDG(hz, c, FE), LDG(hz, c + Y, FE), LDG(hz, c + 2 * Y, FE)), p.dl, cv));
                if (FDTD_IN(q, PE3)) p.psi_e[3][q] = ps;
            }
            if (sz >= 0) {
                const uint32_t q = psi_index(p, 2, sz, i, j, k, p.ea[2].P);
                float ps = FDTD_IN(q, PE4) ? p.psi_e[4][q] : 0.f;
                v = fsub(v, sterm(T2, sz, ps, d4e(LDG(hy, c - 1, FE), LDG(hy, c, FE), LDG(hy, c + 1, FE), LDG(hy, c + 2, FE)), p.dl, cv));
                if (FDTD_IN(q, PE4)) p.psi_e[4][q] = ps;
            }
        }
        if (FDTD_IN(c, FE)) p.out[0][c] = v;
    }
    {   // ey: x term subtracted, z term added
        float v = LDG(p.in[1], c, FE);
        if (iin && kin) {
            const float n = curl4(LDG(hx, c + 1, FE), LDG(hx, c, FE), LDG(hz, c + X, FE), LDG(hz, c, FE));
            const float f = curl4(LDG(hx, c + 2, FE), LDG(hx, c - 1, FE), LDG(hz, c + 2 * X, FE), LDG(hz, c - X, FE));
            const float cv = LDG(p.ce[1], c, FE);
            v = fadd(v, fmul(fmul(p.dl, cv), fsub(fmul(27.0f, n), f)));
            if (sx >= 0) {
                const uint32_t q = psi_index(p, 0, sx, i, j, k, p.ea[0].P);
                float ps = FDTD_IN(q, PE0) ? p.psi_e[0][q] : 0.f;
                v = fsub(v, sterm(T0, sx, ps, d4e(LDG(hz, c - X, FE), LDG(hz, c, FE), LDG(hz, c + X, FE), LDG(hz, c + 2 * X, FE)), p.dl, cv));
                if (FDTD_IN(q, PE0)) p.psi_e[0][q] = ps;
            }
            if (sz >= 0) {
                const uint32_t q = psi_index(p, 2, sz, i, j, k, p.ea[2].P);
                float ps = FDTD_IN(q, PE5) ? p.psi_e[5][q] : 0.f;
                v = fadd(v, sterm(T2, sz, ps, d4e(LDG(hx, c - 1, FE), LDG(hx, c, FE), LDG(hx, c + 1, FE), LDG(hx, c + 2, FE)), p.dl, cv));
                if (FDTD_IN(q, PE5)) p.psi_e[5][q] = ps;
            }
        }
        if (FDTD_IN(c, FE)) p.out[1][c] = v;
    }
    {   // ez: x term added, y term subtracted
        float v = LDG(p.in[2], c, FE);
        if (iin && jin) {
            const float n = curl4(LDG(hy, c + X, FE), LDG(hy, c, FE), LDG(hx, c + Y, FE), LDG(hx, c, FE));
            const float f = curl4(LDG(hy, c + 2 * X, FE), LDG(hy, c - X, FE), LDG(hx, c + 2 * Y, FE), LDG(hx, c - Y, FE));
            const float cv = LDG(p.ce[2], c, FE);
            v = fadd(v, fmul(fmul(p.dl, cv), fsub(fmul(27.0f, n), f)));
            if (sx >= 0) {
                const uint32_t q = psi_index(p, 0, sx, i, j, k, p.ea[0].P);
                float ps = FDTD_IN(q, PE1) ? p.psi_e[1][q] : 0.f;
                v = fadd(v, sterm(T0, sx, ps, d4e(LDG(hy, c - X, FE), LDG(hy, c, FE), LDG(hy, c + X, FE), LDG(hy, c + 2 * X, FE)), p.dl, cv));
                if (FDTD_IN(q, PE1)) p.psi_e[1][q] = ps;
            }
            if (sy >= 0) {
                const uint32_t q = psi_index(p, 1, sy, i, j, k, p.ea[1].P);
                float ps = FDTD_IN(q, PE2) ? p.psi_e[2][q] : 0.f;
                v = fsub(v, sterm(T1, sy, ps, d4e(LDG(hx, c - Y, FE), LDG(hx, c, FE), LDG(hx, c + Y, FE), LDG(hx, c + 2 * Y, FE)), p.dl, cv));
                if (FDTD_IN(q, PE2)) p.psi_e[2][q] = ps;
            }
        }
        if (FDTD_IN(c, FE)) p.out[2][c] = v;
    }
}

// soft sources on edge cells, list order (one thread: a list holds a few sources)
__global__ void k_edge_src(const __grid_constant__ Params p, const __grid_constant__ Edge eb) {
    if (threadIdx.x != 0 || blockIdx.x != 0 || p.t < 0 || p.t >= p.namp) return;
    for (int s = 0; s < p.nsrc; s++) {
        const int si = p.src_ijk[3 * s], sj = p.src_ijk[3 * s + 1], sk = p.src_ijk[3 * s + 2];
        bool in = false;
        for (int b = 0; b < eb.n; b++)
            in |= sj >= eb.j0[b] && sj < eb.j1[b] && sk >= eb.k0[b] && sk < eb.k1[b];
        if (!in) continue;
        float *f = p.out[p.src_comp[s]];
        const int64_t c = (int64_t)si * p.sx + (int64_t)sj * p.sy + sk;
        if (FDTD_IN(c, fext(p))) f[c] = fadd(f[c], p.src_amp[(int64_t)s * p.namp + p.t]);
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

// x planes per work item when the caller leaves the choice to the plan: of
// the chunks 48 .. 256 (steps of 8), the one whose greedy schedule of a
// pass's items over the resident CTAs ends first.  The queue hands items out
// x chunk by x chunk; an item costs its planes (x-slab planes, which carry
// the CPML terms, twice) plus the 6 iterations that fill the pipeline.  The
// largest chunk wins ties (fewer fills).
static int choose_x_chunk(int nx, int64_t tiles, int slots, int pf, int pb) {
    int best = std::min(nx, 128);
    int64_t best_t = -1;
    std::vector<int64_t> heap;
    int last = -1;
    for (int xc = 256; xc >= 48; xc -= 8) {
        const int c = std::min(xc, nx);
        if (c == last) continue;  // chunks past nx are all the whole grid
        last = c;
        heap.assign((size_t)slots, 0);
        for (int x0 = 0; x0 < nx; x0 += c) {
            const int x1 = std::min(nx, x0 + c);
            int64_t cost = 6;
            for (int i = x0; i < x1; i++) cost += ((pf > 0 && i <= pf + 1) || (pb > 0 && i >= nx - pb - 2)) ? 2 : 1;
            for (int64_t t = 0; t < tiles; t++) {  // the CTA free first takes the item
                std::pop_heap(heap.begin(), heap.end(), std::greater<int64_t>());
                heap.back() += cost;
                std::push_heap(heap.begin(), heap.end(), std::greater<int64_t>());
            }
        }
        const int64_t t = *std::max_element(heap.begin(), heap.end());
        if (best_t < 0 || t < best_t) {
            best_t = t;
            best = c;
        }
    }
    return best;
}

struct fdtd_symp_plan {
    Grid g;
    Maps maps[2];
    Params base;
    float *f[2][6];
    const float *psi_h[2][6];
    std::vector<int32_t> src_ijk;  // host copy of the source positions
    int slots;                     // resident CTAs of the pair kernel (SMs x CTAs per SM)
    int cur;
    bool auto_chunk;               // x_chunk chosen per tiling (the caller passed 0)
    int64_t chunk_key[4] = {-1, -1, -1, -1};  // tiling the cached choice was made for
    int chunk_val = 0;
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
    pl->auto_chunk = x_chunk == 0;  // chosen per tiling at run time; 128 until then
    p.x_chunk = (int32_t)std::min<int64_t>(x_chunk > 0 ? x_chunk : 128, g.nx);
    p.nxc = (int32_t)((g.nx + p.x_chunk - 1) / p.x_chunk);
    for (int q = 0; q < 3; q++) p.ce[q] = s->ce[q];
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
        pl->src_ijk = h;
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
    pl->slots = nsm * occ;
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
    for (int q = 0; q < 6; q++) p.in[q] = pl->f[in][q];
    // the pair kernel's region: E_new of rows [j_lo, j_hi) needs H_new of rows
    // j_lo-1 .. j_hi+1, which must hold no y-slab node of any stage (front
    // nodes 1 .. P, back nodes n-P-1 .. n-1): j_lo = P+2, j_hi = n-P-2; the
    // same along z
    auto pf = [&](int ax) {
        int v = 0;
        for (const Axis *A : {&p.ha[ax], &p.hb[ax], &p.ea[ax]}) v = std::max(v, A->front ? A->P : 0);
        return v;
    };
    auto pb = [&](int ax) {
        int v = 0;
        for (const Axis *A : {&p.ha[ax], &p.hb[ax], &p.ea[ax]}) v = std::max(v, A->back ? A->P : 0);
        return v;
    };
    const int64_t ny = pl->g.ny, nz = pl->g.nz;
    p.j_lo = pf(1) > 0 ? pf(1) + 2 : 0;
    p.j_hi = (int32_t)(pb(1) > 0 ? ny - pb(1) - 2 : ny);
    // z edge boxes of whole 64-byte row segments: k_lo rounded up and k_hi
    // rounded down to 16 cells
    p.k_lo = pf(2) > 0 ? (pf(2) + 2 + 15) / 16 * 16 : 0;
    p.k_hi = (int32_t)(pb(2) > 0 ? (nz - pb(2) - 2) / 16 * 16 : nz);
    p.nty_in = p.j_hi > p.j_lo ? (p.j_hi - p.j_lo + TY - 1) / TY : 0;
    // z tiles stay on TZ-column boundaries (128-byte rows for the boxes and the
    // stores): they start at k_lo rounded down and mask the columns outside
    // [k_lo, k_hi)
    p.kt0 = p.k_lo / TZ * TZ;
    p.ntz_in = p.k_hi > p.k_lo ? (p.k_hi - p.kt0 + TZ - 1) / TZ : 0;
    if (pl->auto_chunk && p.nty_in > 0 && p.ntz_in > 0) {
        const int64_t key[4] = {p.nty_in, p.ntz_in, pf(0), pb(0)};
        if (!std::equal(key, key + 4, pl->chunk_key)) {
            pl->chunk_val = choose_x_chunk(p.nx, (int64_t)p.nty_in * p.ntz_in, pl->slots, pf(0), pb(0));
            std::copy(key, key + 4, pl->chunk_key);
        }
        p.x_chunk = pl->chunk_val;
        p.nxc = (p.nx + p.x_chunk - 1) / p.x_chunk;
    }
    // the edge shell: rows outside [j_lo, j_hi), then the columns outside
    // [k_lo, k_hi) of those rows (every x plane)
    Edge eb{};
    auto add_box = [&](int64_t j0, int64_t j1, int64_t k0, int64_t k1) {
        if (j1 <= j0 || k1 <= k0) return;
        eb.j0[eb.n] = (int)j0; eb.j1[eb.n] = (int)j1; eb.k0[eb.n] = (int)k0; eb.k1[eb.n] = (int)k1;
        eb.off[eb.n + 1] = eb.off[eb.n] + (uint32_t)((j1 - j0) * (k1 - k0));
        eb.rcp[eb.n] = (uint32_t)std::min<uint64_t>((((uint64_t)1 << 32) + (uint64_t)(k1 - k0) - 1) / (uint64_t)(k1 - k0),
                                                    0xFFFFFFFFull);
        eb.n++;
    };
    if (p.nty_in == 0 || p.ntz_in == 0) {
        p.nty_in = p.ntz_in = 0;
        add_box(0, ny, 0, nz);
    } else {
        add_box(0, p.j_lo, 0, nz);
        add_box(p.j_hi, ny, 0, nz);
        add_box(p.j_lo, p.j_hi, 0, p.k_lo);
        add_box(p.j_lo, p.j_hi, p.k_hi, nz);
    }
    // sources per tile of this tiling (the kernel stages at most MAX_SRC per tile)
    if (p.nty_in > 0 && p.ntz_in > 0 && pl->src_ijk.size() / 3 > (size_t)MAX_SRC) {
        std::vector<int> count((size_t)p.nty_in * p.ntz_in * p.nxc, 0);
        for (size_t a = 0; a + 2 < pl->src_ijk.size(); a += 3) {
            const int si = pl->src_ijk[a], sj = pl->src_ijk[a + 1], sk = pl->src_ijk[a + 2];
            if (sj < p.j_lo || sj >= p.j_hi || sk < p.k_lo || sk >= p.k_hi) continue;
            const size_t it = ((size_t)(si / p.x_chunk) * p.nty_in + (sj - p.j_lo) / TY) * p.ntz_in + (sk - p.kt0) / TZ;
            if (++count[it] > MAX_SRC) return FDTD_ERR_CAPACITY;
        }
    }
    cudaStream_t st = as_stream(stream);
    const int64_t items = (int64_t)p.nty_in * p.ntz_in * p.nxc;
    if (items > 0) {
        const int nb = (int)std::min<int64_t>(items, pl->slots);
        if (two_h)
            k_symp_pair<true><<<nb, THREADS, SMEM, st>>>(pl->maps[in], p);
        else
            k_symp_pair<false><<<nb, THREADS, SMEM, st>>>(pl->maps[in], p);
    }
    const int64_t ecells = eb.off[eb.n];  // per x plane
    if (ecells > 0) {
        const dim3 nb((unsigned)((ecells + EDGE_BLOCK - 1) / EDGE_BLOCK), (unsigned)pl->g.nx);
        if (two_h)
            k_edge_h<true><<<nb, EDGE_BLOCK, 0, st>>>(p, eb);
        else
            k_edge_h<false><<<nb, EDGE_BLOCK, 0, st>>>(p, eb);
        k_edge_e<<<nb, EDGE_BLOCK, 0, st>>>(p, eb);
        bool esrc = false;
        for (size_t a = 0; a + 2 < pl->src_ijk.size(); a += 3)
            for (int b = 0; b < eb.n; b++)
                esrc |= pl->src_ijk[a + 1] >= eb.j0[b] && pl->src_ijk[a + 1] < eb.j1[b] &&
                        pl->src_ijk[a + 2] >= eb.k0[b] && pl->src_ijk[a + 2] < eb.k1[b];
        if (esrc && src_t >= 0 && src_t < p.namp) k_edge_src<<<1, 32, 0, st>>>(p, eb);
    }
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
