// Fused Yee time step: E update + E-CPML + soft sources + H update + H-CPML
// in ONE pass over HBM per time step (sm_103a, TMA + mbarrier pipeline).
//
// Semantics are exactly those of the in-place sequence
//   update_e -> cpml_e -> sources -> update_h -> cpml_h
// (2nd_order-Yee/CUDA/fdtd3d_201_250x250x320cell_15npml_100000tstep.cu:718-742,
//  operation grouping of 2nd_order-Yee/Numpy/fdtd3d.py:4-13), computed with
// the same round-to-nearest operations, so the result is bit-identical to
// the unfused kernels and to the FP32 oracle.
//
// Design
//  * The state lives in two buffers (ping-pong): a step reads buffer `cur`
//    and writes buffer `1-cur`.  E-psi slabs are ping-ponged too; H-psi is
//    updated in place (only its owner touches it).
//  * A CTA owns a tile of TZ=64 (z) x TY (y) cells for a chunk of x planes
//    and marches along x.  For plane i it needs H(i), H(i+1), E(i), CE(i)
//    with a one-cell halo at j0-1 / k0-1 (and j0+TY / k0+TZ for H).  These
//    arrive by 3-D TMA box loads (cp.async.bulk.tensor) into a ring of NS
//    shared-memory stages, completion tracked by mbarriers.
//  * E_new is computed on the tile plus the j0-1 row and k0-1 column
//    (halo cells are recomputed from the untouched input buffer, never read
//    from a neighbour), then H_new(i) for the tile uses E_new(i) from shared
//    memory and E_new(i-1) kept in registers.
//  * A chunk starting at x0 > 0 recomputes E_new(x0-1) without storing it.
//  * Every mbarrier wait is bounded; on expiry the kernel records
//    FDTD_ERR_TIMEOUT in a device status word and the CTA leaves its loop.
#pragma once
#include <cuda.h>

#include "common.cuh"

namespace fdtd {
namespace fused {

// Tile: TZ cells along z (two per lane: lanes work on float2 pairs) x TY rows.
constexpr int TZ = 64;
constexpr int HC = TZ + 8;   // H box:    k0-4 .. k0+TZ+3 (needs k0-1 .. k0+TZ)
constexpr int EC = TZ + 4;   // E/CE box: k0-4 .. k0+TZ-1 (needs k0-1 .. k0+TZ-1)
constexpr int NCW = TZ + 4;  // E_new row stride; column c holds k = k0-2+c
constexpr int MAX_LOCAL_SRC = 128;
constexpr int MAX_BAND_SRC = 32;
constexpr uint64_t WAIT_NS = 1000000000ull;  // a wait gives up after 1 s

constexpr int al128(int b) { return (b + 127) / 128 * 128; }

// Shared-memory layout of one CTA for tile height TY and NS pipeline stages.
// Warps 0..TY-1 own rows j0..j0+TY-1 (E and H); warp TY recomputes E_new on
// the halo row j0-1; warp TY+1 recomputes E_new on the halo column k0-1;
// lane 0 of warp TY+2 is the producer (mbarrier waits, TMA issue).
template <int TY, int NS>
struct Layout {
    static constexpr int HR = TY + 2, ER = TY + 1;
    static constexpr int HBOX = HR * HC, EBOX = ER * EC;  // floats per component box
    static constexpr int HBOXB = al128(HBOX * 4), EBOXB = al128(EBOX * 4);
    static constexpr int STAGE = 3 * HBOXB + 6 * EBOXB;  // H(3), E(3), CE(3)
    static constexpr uint32_t TX = 3 * HBOX * 4 + 6 * EBOX * 4;
    // a stage completes on two barriers: H (needed one plane early, as H(i+1))
    // and E + CE (needed on its own plane only)
    static constexpr uint32_t TX_H = 3 * HBOX * 4, TX_E = 6 * EBOX * 4;
    static constexpr int NR = TY + 1;
    static constexpr int ENEWC = NR * NCW;  // floats per component
    // TY row warps, the halo-row warp, the halo-column warp, the producer warp
    static constexpr int THREADS = (TY + 3) * 32;
    static constexpr int ENEW = al128(3 * ENEWC * 4);
    // psi ring: 2 slots x 4 boxes (E psi 1, 2 and H psi 1, 2 of one axis)
    static constexpr int PSIRING = 2 * 4 * EBOXB;
    static constexpr uint32_t PSI_TX = EBOX * 4;
    static constexpr int SMEM = NS * STAGE + ENEW + 128 /*barriers*/ + PSIRING + 128 /*align slack*/;
    // CTAs per SM the register budget is sized for (shared memory may allow fewer)
    static constexpr int MINB = TY == 4 ? 3 : (TY == 8 ? 2 : 1);
};

struct TMaps {
    CUtensorMap h[3];   // hx, hy, hz of the input buffer, box (HC, TY+2, 1)
    CUtensorMap e[3];   // ex, ey, ez of the input buffer, box (EC, TY+1, 1)
    CUtensorMap ce[3];  // cex, cey, cez,                  box (EC, TY+1, 1)
    // x/y CPML psi slabs, box (EC, TY+1, 1): x arrays (2P, ny, nz) at (k0-4, j0-1, s),
    // y arrays (nx, 2P, nz) at (k0-4, first slab index of the tile, i)
    CUtensorMap xpe[2];  // eyx, ezx of the input buffer
    CUtensorMap xph[2];  // hyx, hzx
    CUtensorMap ype[2];  // ezy, exy of the input buffer
    CUtensorMap yph[2];  // hzy, hxy
};

struct Params {
    int64_t nx, ny, nz, sx, sy;
    int32_t ntz, nty, nxc, x_chunk;
    float *out[6];  // ex, ey, ez, hx, hy, hz of the output buffer
    const float *psi_e_in[6];
    float *psi_e_out[6];
    float *psi_h[6];
    int32_t P[3];
    int32_t faces;
    const float *tb_e[3], *ta_e[3], *tk_e[3];
    const float *tb_h[3], *ta_h[3], *tk_h[3];
    int32_t nsrc;
    const int32_t *src_ijk;
    const int32_t *src_comp;
    const float *src_amp;
    int64_t namp;
    int64_t t;
    int32_t *status;
    int32_t stage_bytes;  // bytes per pipeline stage
    int32_t xypsi;        // 1: x/y psi slabs arrive by TMA in the psi ring
    // z band (1 when a z face has CPML): the z-slab CPML is finished by the
    // band kernels.  The fused kernel leaves them the E z-psi correction, the
    // sources on E z-slab nodes and every H cell of the band (k in [1, P+1]
    // and [n-P-1, n-1]).
    int32_t zfix;
    const float *in[6];   // input buffer fields (read by the band kernels)
    const float *in_ce[3];
    // sources on E z-slab nodes, applied by the E band kernel in list order;
    // nbsrc < 0: more than MAX_BAND_SRC of them, the band kernel scans the list
    int32_t nbsrc;
    int32_t bsrc[MAX_BAND_SRC];
    // Drude box (drude = 1): cells [i0, i0+ni) x [j0, j0+nj) x [k0, k0+nk); dense J, CJA, CJB;
    // J is read from dj_in and written to dj_out (ping-pong like E-psi)
    int32_t drude;
    int64_t dbox[6];  // i0, j0, k0, ni, nj, nk
    const float *dj_in[3];
    float *dj_out[3];
    const float *dcja[3], *dcjb[3];
    // TFSF plane wave (tfsf = 1): box corners tp1, tp2 (p2 = pt2 + 1), face bits, axis;
    // incident table per half (0: E faces read th1d, 1: H faces read te1d), face, slot:
    // coefficient and 1-D index (tix >= 0: fixed; < 0: coordinate along the axis + tvo)
    int32_t tfsf, tfaces, taxis, tvo;
    int32_t tp1[3], tp2[3];
    float tcoef[2][6][2];
    int32_t tix[2][6][2];
    const float *te1d, *th1d;
    // test hook of single-grid plans (plan creation sets 0 and -1): wait_ns > 0
    // replaces the 1 s wait limit; test_withhold >= 0 makes CTA 0 skip the
    // copies of that plane of its first work item, so its wait runs out with
    // no copy in flight.
    uint64_t wait_ns;
    int32_t test_withhold;
};

// extents (elements) of a field array and of psi array q (0, 1: x slab;
// 2, 3: y slab; 4, 5: z slab), for the bounds-checked build
__host__ __device__ __forceinline__ int64_t fext_y(const Params &p) { return p.nx * p.sx; }
__host__ __device__ __forceinline__ int64_t pext_y(const Params &p, int q) {
    const int ax = q / 2;
    const int64_t P2 = 2 * (int64_t)p.P[ax];
    return ax == 0 ? P2 * p.ny * p.nz : (ax == 1 ? p.nx * P2 * p.nz : p.nx * p.ny * P2);
}

// Many independent grids advanced by one launch: work items of all grids are
// numbered consecutively; item_off[s] is the first item of grid s.
struct BatchDesc {
    int32_t nsims;
    int32_t cur;             // buffer holding the current state (same for every grid)
    int64_t t;               // step number (source amplitude index)
    const Params *params;    // [2*nsims]: grid s reading buffer b at params[2*s + b]
    const TMaps *maps;       // [2*nsims]: tensor maps of grid s, input buffer b
    const int64_t *item_off; // [nsims + 1]
    int32_t stage_bytes;     // pipeline stage size (max over grids)
    // work queue: [0] next item, [1] CTAs finished; zero between launches (the
    // last CTA to finish clears both)
    int32_t *queue;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
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

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait: true on completion; false after limit_ns, or early when
// another CTA has already recorded a timeout in the status word (status may
// be null: then only the deadline applies).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, const int32_t *status,
                                                  uint64_t limit_ns = WAIT_NS) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t n = 1;; n++) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((n & 255) == 0) {
            if (globaltimer_ns() - t0 > limit_ns) return false;
            if (status && *(volatile const int32_t *)status == FDTD_ERR_TIMEOUT) return false;
        }
    }
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1,
                                            int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void prefetch_tmap(const CUtensorMap *map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// CPML slab index of an E node / H node along one axis, or -1.
__device__ __forceinline__ int slab_e(int64_t idx, int P, int64_t n, int front, int back) {
    if (P <= 0) return -1;
    if (front && idx >= 1 && idx <= P) return (int)(idx - 1);
    if (back && idx >= n - P - 1 && idx <= n - 2) return (int)(P + idx - (n - P - 1));
    return -1;
}
__device__ __forceinline__ int slab_h(int64_t idx, int P, int64_t n, int front, int back) {
    if (P <= 0) return -1;
    if (front && idx >= 1 && idx <= P) return (int)(idx - 1);
    if (back && idx >= n - P && idx <= n - 1) return (int)(P + idx - (n - P));
    return -1;
}

// H cells whose update reads an E z-slab node or that carry a z psi:
// k in [1, P+1] (front) or [n-P-1, n-1] (back)
__device__ __forceinline__ bool in_zband_h(int64_t k, int P, int64_t n, int front, int back) {
    if (P <= 0) return false;
    return (front && k >= 1 && k <= P + 1) || (back && k >= n - P - 1 && k <= n - 1);
}

__device__ __forceinline__ float cpml_corr(float &psi, float b, float a, float km1, float d) {
    psi = fadd(fmul(b, psi), fmul(a, d));
    return fadd(fmul(km1, d), psi);
}

__device__ __forceinline__ float2 ld2(const float *p) { return *reinterpret_cast<const float2 *>(p); }
__device__ __forceinline__ void st2(float *p, float2 v) { *reinterpret_cast<float2 *>(p) = v; }
#ifndef FDTD_PACKED_F32X2
#define FDTD_PACKED_F32X2 0
#endif
#if FDTD_PACKED_F32X2
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b rounds exactly like a + (-b)
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
#else
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return make_float2(fadd(a.x, b.x), fadd(a.y, b.y)); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return make_float2(fsub(a.x, b.x), fsub(a.y, b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return make_float2(fmul(a.x, b.x), fmul(a.y, b.y)); }
#endif
__device__ __forceinline__ float2 curl4x2(float2 a, float2 b, float2 c, float2 d) {
    return add2(sub2(sub2(a, b), c), d);
}
__device__ __forceinline__ float get(const float2 &v, int e) { return e ? v.y : v.x; }
__device__ __forceinline__ void set(float2 &v, int e, float x) {
    if (e) v.y = x; else v.x = x;
}

// CPML table entry of one slab node (b, a, 1/kappa - 1).
struct Coef {
    float b, a, km;
};

// psi <- b psi + a d; returns km1 d + psi (the CPML correction term)
__device__ __forceinline__ float corr(float &psi, const Coef &c, float d) {
    psi = fadd(fmul(c.b, psi), fmul(c.a, d));
    return fadd(fmul(c.km, d), psi);
}

// Coefficients of slab node s from the shared-memory tables of one axis
// (base = first of the six tables, n2 = 2P entries each; eh = 0 E, 1 H).
__device__ __forceinline__ Coef tab_coef(const float *tabs, int base, int n2, int eh, int s) {
    const float *t = tabs + base + eh * 3 * n2;
    return Coef{t[s], t[n2 + s], t[2 * n2 + s]};
}

// TFSF correction of one face slot: v += 0.5 (c * F1d[idx]) (kuFDTD/v0.2.0/dim3/tfsf.py:79-89)
__device__ __forceinline__ void tfsf_add(const Params &p, int half, int f, int slot, const float *f1d, int64_t ax,
                                         float &v) {
    const int32_t ix = p.tix[half][f][slot];
    const float c = p.tcoef[half][f][slot];
    // the 1-D grid is read-only inside the fused kernel: read-only data cache
    v = fadd(v, fmul(0.5f, fmul(c, __ldg(f1d + (ix >= 0 ? (int64_t)ix : ax + p.tvo)))));
}
__device__ __forceinline__ bool tin(int64_t x, int32_t lo, int32_t hi) { return x >= lo && x <= hi; }

// Per item and lane: for each cell e of the pair, component and face family
// (the two face axes that can correct that component, in face order), a
// 2-bit code from the cell's (j, k): 0 none, 1 front face, 2 back face, 3 one of
// the two x faces (decided per plane).  Layout: bit (e*12 + (comp*2 + fam)*2).
// E (tfsf.py:154-186 e1/e2 slices): ex (y face, z face), ey (x face, z face),
// ez (x face, y face); H: hx (y, z), hy (x, z), hz (x, y).
__device__ __forceinline__ uint32_t tfsf_lane_codes(const Params &p, int eh, int64_t j, int64_t k0c, bool in0,
                                                    bool in1) {
    const int32_t j1 = p.tp1[1], k1 = p.tp1[2], j2 = p.tp2[1], k2 = p.tp2[2];
    const int32_t f = p.tfaces;
    auto code = [&](bool cand, bool back, int face_front) -> uint32_t {
        if (!cand) return 0;
        const int face = face_front + (back ? 1 : 0);
        return ((f >> face) & 1) ? (back ? 2u : 1u) : 0u;
    };
    uint32_t m = 0;
#pragma unroll
    for (int e = 0; e < 2; e++) {
        if (!(e ? in1 : in0)) continue;
        const int64_t k = k0c + e;
        uint32_t c[6];
        if (eh == 0) {
            const int32_t je0 = j1 - 1, ke0 = k1 - 1;  // E faces at p1-1 and p2
            c[0] = code((j == je0 || j == j2) && tin(k, k1, k2 - 1), j == j2, 2);     // ex, y face
            c[1] = code((k == ke0 || k == k2) && tin(j, j1, j2 - 1), k == k2, 4);     // ex, z face
            c[2] = tin(j, j1, j2) && tin(k, k1, k2 - 1) ? 3u : 0u;                    // ey, x face
            c[3] = code((k == ke0 || k == k2) && tin(j, j1, j2), k == k2, 4);         // ey, z face
            c[4] = tin(j, j1, j2 - 1) && tin(k, k1, k2) ? 3u : 0u;                    // ez, x face
            c[5] = code((j == je0 || j == j2) && tin(k, k1, k2), j == j2, 2);         // ez, y face
        } else {                                       // H faces at p1 and p2
            c[0] = code((j == j1 || j == j2) && tin(k, k1, k2), j == j2, 2);          // hx, y face
            c[1] = code((k == k1 || k == k2) && tin(j, j1, j2), k == k2, 4);          // hx, z face
            c[2] = tin(j, j1, j2 - 1) && tin(k, k1, k2) ? 3u : 0u;                    // hy, x face
            c[3] = code((k == k1 || k == k2) && tin(j, j1, j2 - 1), k == k2, 4);      // hy, z face
            c[4] = tin(j, j1, j2) && tin(k, k1, k2 - 1) ? 3u : 0u;                    // hz, x face
            c[5] = code((j == j1 || j == j2) && tin(k, k1, k2 - 1), j == j2, 2);      // hz, y face
        }
#pragma unroll
        for (int q = 0; q < 6; q++) m |= c[q] << (e * 12 + q * 2);
    }
    return m;
}

// Apply the TFSF terms of one cell (codes = its 12 bits) to the three
// components of the E (eh = 0) or H (eh = 1) field just updated at plane i.
// Slot and face of each family as tfsf.py:154-186; the x faces of E at p1-1 and
// p2, of H at p1 and p2; for H the two families apply in face order.
__device__ __forceinline__ void tfsf_apply(const Params &p, int eh, uint32_t codes, int64_t i, int64_t j, int64_t k,
                                           float &vx, float &vy, float &vz) {
    const int32_t i1 = p.tp1[0], i2 = p.tp2[0];
    const int64_t ax = p.taxis == 0 ? i : (p.taxis == 1 ? j : k);
    const float *f1d = eh == 0 ? p.th1d : p.te1d;
    const bool xf = eh == 0 ? i == i1 - 1 : i == i1, xb = i == i2;  // x face planes
    const bool xface = (xf && (p.tfaces & 1)) || (xb && ((p.tfaces >> 1) & 1));
    const int xid = xf ? 0 : 1;
    // x-range of the y and z families: [i1, i2] or [i1, i2-1] per component
    const bool ir = tin(i, i1, i2), irm = tin(i, i1, i2 - 1);
    const uint32_t c0 = codes & 3, c1 = (codes >> 2) & 3, c2 = (codes >> 4) & 3, c3 = (codes >> 6) & 3,
                   c4 = (codes >> 8) & 3, c5 = (codes >> 10) & 3;
    if (eh == 0) {
        if (c0 && ir) tfsf_add(p, 0, 2 + (int)c0 - 1, 1, f1d, ax, vx);      // ex += y face (slot e2)
        if (c1 && ir) tfsf_add(p, 0, 4 + (int)c1 - 1, 0, f1d, ax, vx);      // ex += z face (e1)
        if (c2 && xface) tfsf_add(p, 0, xid, 0, f1d, ax, vy);               // ey += x face (e1)
        if (c3 && irm) tfsf_add(p, 0, 4 + (int)c3 - 1, 1, f1d, ax, vy);     // ey += z face (e2)
        if (c4 && xface) tfsf_add(p, 0, xid, 1, f1d, ax, vz);               // ez += x face (e2)
        if (c5 && irm) tfsf_add(p, 0, 2 + (int)c5 - 1, 0, f1d, ax, vz);     // ez += y face (e1)
    } else {
        if (c0 && irm) tfsf_add(p, 1, 2 + (int)c0 - 1, 1, f1d, ax, vx);     // hx += y face (h2)
        if (c1 && irm) tfsf_add(p, 1, 4 + (int)c1 - 1, 0, f1d, ax, vx);     //    then z face (h1)
        if (c2 && xface) tfsf_add(p, 1, xid, 0, f1d, ax, vy);               // hy += x face (h1)
        if (c3 && ir) tfsf_add(p, 1, 4 + (int)c3 - 1, 1, f1d, ax, vy);      //    then z face (h2)
        if (c4 && xface) tfsf_add(p, 1, xid, 1, f1d, ax, vz);               // hz += x face (h2)
        if (c5 && ir) tfsf_add(p, 1, 2 + (int)c5 - 1, 0, f1d, ax, vz);      //    then y face (h1)
    }
}

// EXT: 0 = neither the Drude box nor the TFSF faces are compiled in, 1 = the
// Drude box, 2 = both.  A plan launches the smallest variant its grid needs:
// code a step does not use still costs it registers and instruction-cache
// space (the plain step ran 3.5 % slower with both compiled in).
template <int TY, int NS, bool BATCH, int EXT>
__global__ void __launch_bounds__(Layout<TY, NS>::THREADS, Layout<TY, NS>::MINB)
k_yee_fused(const __grid_constant__ TMaps mk, const __grid_constant__ Params pk, const __grid_constant__ BatchDesc bd) {
    using L = Layout<TY, NS>;
    // A stage is released one iteration after its plane was consumed, and each
    // iteration holds two planes: fewer than 3 stages would wait on a plane
    // that is only issued after the wait.
    static_assert(NS >= 3, "the fused pipeline needs at least 3 stages");
    static_assert((2 * NS + 2) * 8 <= 128, "the mbarriers live in 128 bytes");
    extern __shared__ unsigned char smem_raw[];
    // 128-byte aligned base, computed from the shared-window offset so the
    // pointer stays in the shared address space (shared loads, not generic ones)
    unsigned char *smem =
        smem_raw + ((128u - (static_cast<uint32_t>(__cvta_generic_to_shared(smem_raw)) & 127u)) & 127u);
    // stage size: read from the kernel parameters at each use (a constant-bank
    // operand) rather than held in a register
#define FDTD_SB (BATCH ? bd.stage_bytes : pk.stage_bytes)
    float *enew = reinterpret_cast<float *>(smem + NS * FDTD_SB);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + NS * FDTD_SB + L::ENEW);
    float *Nx = enew, *Ny = enew + L::ENEWC, *Nz = enew + 2 * L::ENEWC;
    // psi ring (2 slots of 4 boxes), then the CPML tables:
    // tab[(axis*2 + eh)*3 + {b,a,km}] has 2P[axis] entries
    unsigned char *psiring = smem + NS * FDTD_SB + L::ENEW + 128;
    float *tabs = reinterpret_cast<float *>(psiring + L::PSIRING);
    // batched launches: parameters of the grid the current item belongs to
    __shared__ __align__(16) Params s_p;

    __shared__ int s_abort;
    __shared__ int s_nls;
    // sources of the current work item, list order: (i << 16 | j), (k << 2 | comp), list index
    __shared__ uint32_t s_ls_ij[MAX_LOCAL_SRC];
    __shared__ int s_ls_kc[MAX_LOCAL_SRC], s_ls_s[MAX_LOCAL_SRC];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // Roles.  E phase: warps 0..TY-1 -> own row r = warp+1 (j = j0+warp), pair
    // k = k0+2*lane; warp TY -> halo row r = 0 (j = j0-1); warp TY+1 -> halo
    // column: lane r <= TY computes the pair at k0-2, k0-1 of row r (only the
    // k0-1 value is used).  H phase: warps 0..TY-1, own pairs.
    const bool col_warp = warp == TY + 1;
    // producer: lane 0 of warp TY+2 waits on the mbarriers and issues the TMA
    // copies, so that no stencil warp carries that work on its critical path
    const bool producer = tid == (TY + 2) * 32;
    const bool e_active = warp <= TY || (col_warp && lane <= TY);
    const bool h_active = warp < TY;
    const int er = warp < TY ? warp + 1 : (warp == TY ? 0 : lane);
    const int eko = col_warp ? -2 : 2 * lane;  // pair start relative to k0
    const bool own_row = warp < TY;

    auto stage_ptr = [&](int st) { return smem + st * FDTD_SB; };
    auto sH = [&](int st, int c) { return reinterpret_cast<float *>(stage_ptr(st) + c * L::HBOXB); };
    auto sE = [&](int st, int c) { return reinterpret_cast<float *>(stage_ptr(st) + 3 * L::HBOXB + c * L::EBOXB); };
    auto sC = [&](int st, int c) {
        return reinterpret_cast<float *>(stage_ptr(st) + 3 * L::HBOXB + (3 + c) * L::EBOXB);
    };
    // psi box b (0, 1 = E psi, 2, 3 = H psi of the x or y slab) of ring slot sl
    auto sP = [&](int sl, int b) { return reinterpret_cast<float *>(psiring + (sl * 4 + b) * L::EBOXB); };
    const Params &p = BATCH ? s_p : pk;

    // stage the CPML coefficient tables of the current grid (a few hundred floats)
    auto stage_tables = [&]() {
        int off = 0;
        auto copy = [&](const float *src, int n2) {
            for (int x = tid; x < n2; x += blockDim.x) tabs[off + x] = src[x];
            off += n2;
        };
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int n2 = 2 * p.P[a];
            copy(p.tb_e[a], n2);
            copy(p.ta_e[a], n2);
            copy(p.tk_e[a], n2);
            copy(p.tb_h[a], n2);
            copy(p.ta_h[a], n2);
            copy(p.tk_h[a], n2);
        }
    };

    if (tid == 0) {
        // stage H barriers, stage E+CE barriers, then the 2 psi slots
        for (int s = 0; s < 2 * NS + 2; s++) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (!BATCH) {
            for (int c = 0; c < 3; c++) {
                prefetch_tmap(&mk.h[c]);
                prefetch_tmap(&mk.e[c]);
                prefetch_tmap(&mk.ce[c]);
            }
            if (pk.xypsi)
                for (int c = 0; c < 2; c++) {
                    prefetch_tmap(&mk.xpe[c]);
                    prefetch_tmap(&mk.xph[c]);
                    prefetch_tmap(&mk.ype[c]);
                    prefetch_tmap(&mk.yph[c]);
                }
        }
        s_abort = 0;
    }
    // Per-grid values are read from p at each use: constant-bank operands for a
    // single grid, shared-memory loads of the current grid's copy in a batch
    // (held in registers they would be live across the whole item loop).
    if (!BATCH) stage_tables();

    uint32_t g0 = 0;          // planes this CTA has issued before the current item
    uint32_t gp0 = 0;         // psi ring phases this CTA has used before the current item
    int64_t issued_hi = -1;   // highest plane index (relative) issued in the current item (tid 0)
    int64_t psi_hi = -1;      // highest plane whose psi boxes were issued (tid 0)
    int64_t q_abort = 0, i_start_abort = 0;
    bool aborted = false;
    const uint64_t wlim = (!BATCH && pk.wait_ns) ? pk.wait_ns : WAIT_NS;
    bool first_item = true;
    const int64_t nitems = BATCH ? bd.item_off[bd.nsims] : (int64_t)pk.ntz * pk.nty * pk.nxc;
    int cur_sim = -1;

    // Batched launches take items from a queue (grids ordered with the longest
    // items first, so the short ones fill the tail); a single grid walks its
    // uniform items in a fixed stride.
    __shared__ int s_item;
    int64_t gitem = blockIdx.x;
    if (BATCH) {
        if (tid == 0) s_item = atomicAdd(&bd.queue[0], 1);
        __syncthreads();
        gitem = s_item;
    }
    while (gitem < nitems && !aborted) {
        int64_t item = gitem;
        const TMaps *mp = &mk;
        if (BATCH) {
            // grid of this item: largest s with item_off[s] <= gitem
            int lo = 0, hi = bd.nsims - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (bd.item_off[mid] <= gitem) lo = mid;
                else hi = mid - 1;
            }
            item = gitem - bd.item_off[lo];
            mp = &bd.maps[2 * lo + bd.cur];
            if (lo != cur_sim) {
                __syncthreads();  // every thread is done with the previous grid's parameters
                for (int w = tid; w < (int)(sizeof(Params) / 4); w += blockDim.x)
                    reinterpret_cast<int32_t *>(&s_p)[w] =
                        reinterpret_cast<const int32_t *>(&bd.params[2 * lo + bd.cur])[w];
                __syncthreads();
                if (tid == 0) {
                    s_p.t = bd.t;
                    for (int c = 0; c < 3; c++) {
                        prefetch_tmap(&mp->h[c]);
                        prefetch_tmap(&mp->e[c]);
                        prefetch_tmap(&mp->ce[c]);
                    }
                }
                stage_tables();
                __syncthreads();
                cur_sim = lo;
            }
        }
        const TMaps &maps = *mp;
        const int64_t tzi = item % p.ntz, tyi = (item / p.ntz) % p.nty, xci = item / ((int64_t)p.ntz * p.nty);
        const int64_t k0 = tzi * TZ, j0 = tyi * TY;
        const int64_t x0 = xci * p.x_chunk;
        const int64_t x1 = min(x0 + (int64_t)p.x_chunk, p.nx);
        const int64_t i_start = x0 > 0 ? x0 - 1 : 0;
        const int64_t nplanes = x1 - i_start + 1;  // planes i_start .. x1 (H(x1) feeds E(x1-1))
        // Tile-uniform: no grid edge and no y/z CPML slab inside the tile's E/H region.
        // tile's E (k0-1..k0+TZ-1) or H (k0..k0+TZ-1) columns touch a z slab
        // Tile-uniform: no y CPML slab among the tile's rows.  Grid edges are
        // handled on the plain path by per-lane masks, and the z slab is the
        // band kernels' work, so z-slab tiles are plain here too.
        const bool y_plain = p.P[1] == 0 || ((j0 - 1 > p.P[1] || !((p.faces >> 2) & 1)) && (j0 + TY - 1 < p.ny - p.P[1] - 1 || !((p.faces >> 3) & 1)));

        // y psi by TMA for tiles whose y-slab rows lie on one side (box row r <-> j0-1+r)
        const bool ye_f = ((p.faces >> 2) & 1) && p.P[1] > 0 && j0 - 1 <= p.P[1] && j0 + TY - 1 >= 1;
        const bool ye_b = ((p.faces >> 3) & 1) && p.P[1] > 0 && j0 + TY - 1 >= p.ny - p.P[1] - 1 && j0 - 1 <= p.ny - 2;
        const bool yh_f = ((p.faces >> 2) & 1) && p.P[1] > 0 && j0 <= p.P[1] && j0 + TY - 1 >= 1;
        const bool yh_b = ((p.faces >> 3) & 1) && p.P[1] > 0 && j0 + TY - 1 >= p.ny - p.P[1] && j0 <= p.ny - 1;
        const bool ytile = p.xypsi && (ye_f || ye_b || yh_f || yh_b) && !((ye_f || yh_f) && (ye_b || yh_b));
        // the item's E region (planes i_start..x1-1, rows j0-1.., columns k0-1..) meets the Drude box
        const bool dtile = EXT >= 1 && p.drude && i_start < p.dbox[0] + p.dbox[3] && x1 > p.dbox[0] &&
                           j0 - 1 < p.dbox[1] + p.dbox[4] && j0 + TY > p.dbox[1] &&
                           k0 - 1 < p.dbox[2] + p.dbox[5] && k0 + TZ > p.dbox[2];

        // ---- per-item, per-thread cell description (pair at row j, columns k, k+1) ----
        const int64_t jj = j0 - 1 + er, kk = k0 + eko;
        const bool row_in = jj >= 0 && jj < p.ny;
        const bool in0 = row_in && kk >= 0 && kk < p.nz, in1 = row_in && kk + 1 >= 0 && kk + 1 < p.nz;
        const bool j_lt = jj < p.ny - 1, j_gt = jj > 0;
        const bool k0_lt = kk < p.nz - 1, k1_lt = kk + 1 < p.nz - 1, k0_gt = kk > 0, k1_gt = kk + 1 > 0;
        // lanes with a cell outside an update region (grid edges); the i edges are plane-uniform
        const bool emask = !(j_lt && k0_lt && k1_lt), hmask = !(j_gt && k0_gt && k1_gt);
        const int sye = row_in ? slab_e(jj, p.P[1], p.ny, ((p.faces >> 2) & 1), ((p.faces >> 3) & 1)) : -1;
        const int syh = row_in ? slab_h(jj, p.P[1], p.ny, ((p.faces >> 2) & 1), ((p.faces >> 3) & 1)) : -1;
        // H cells of the z band: left to the band kernel (no psi_h update here)
        const bool hb0 = p.zfix && in_zband_h(kk, p.P[2], p.nz, ((p.faces >> 4) & 1), ((p.faces >> 5) & 1));
        const bool hb1 = p.zfix && in_zband_h(kk + 1, p.P[2], p.nz, ((p.faces >> 4) & 1), ((p.faces >> 5) & 1));

        auto issue = [&](int64_t q) {
            const int64_t plane = i_start + q;
            const int st = (int)((g0 + q) % NS);
            uint64_t *bar = &bars[st], *bare = &bars[NS + st];
            if (!BATCH && first_item && blockIdx.x == 0 && q == pk.test_withhold) return;  // test hook
            issued_hi = q;
            if (plane >= p.nx) {
                // Past the last plane: H(p.nx) only feeds E components that are
                // never updated at i = p.nx-1; complete the phases without a copy.
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bare)) : "memory");
                return;
            }
            mbar_arrive_expect_tx(bar, L::TX_H);
            mbar_arrive_expect_tx(bare, L::TX_E);
            const int kc = (int)(k0 - 4), jc = (int)(j0 - 1), xc = (int)plane;
            for (int c = 0; c < 3; c++) tma_load_3d(sH(st, c), &maps.h[c], bar, kc, jc, xc);
            for (int c = 0; c < 3; c++) tma_load_3d(sE(st, c), &maps.e[c], bare, kc, jc, xc);
            for (int c = 0; c < 3; c++) tma_load_3d(sC(st, c), &maps.ce[c], bare, kc, jc, xc);
        };
        // psi boxes of plane q into ring slot (gp0+q)&1: the x slab's on x-slab
        // planes, else the y slab's in y-slab tiles; otherwise a bare arrive
        auto issue_psi = [&](int64_t q) {
            const uint32_t Gp = gp0 + (uint32_t)q;
            const int sl = (int)(Gp & 1);
            uint64_t *bar = &bars[2 * NS + sl];
            psi_hi = q;
            const int64_t plane = i_start + q;
            const int xse = plane < p.nx ? slab_e(plane, p.P[0], p.nx, (p.faces & 1), ((p.faces >> 1) & 1)) : -1;
            const int xsh = plane < p.nx ? slab_h(plane, p.P[0], p.nx, (p.faces & 1), ((p.faces >> 1) & 1)) : -1;
            const bool xm = p.xypsi && (xse >= 0 || xsh >= 0);
            const bool ym = !xm && ytile && plane < p.nx;
            const bool ye = ye_f || ye_b, yh = yh_f || yh_b;
            const uint32_t nbox = xm ? 2u * (xse >= 0) + 2u * (xsh >= 0) : (ym ? 2u * ye + 2u * yh : 0u);
            if (nbox == 0) {
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
                return;
            }
            mbar_arrive_expect_tx(bar, nbox * L::PSI_TX);
            const int kc = (int)(k0 - 4), jc = (int)(j0 - 1), xc = (int)plane;
            if (xm) {
                if (xse >= 0) {
                    tma_load_3d(sP(sl, 0), &maps.xpe[0], bar, kc, jc, xse);
                    tma_load_3d(sP(sl, 1), &maps.xpe[1], bar, kc, jc, xse);
                }
                if (xsh >= 0) {
                    tma_load_3d(sP(sl, 2), &maps.xph[0], bar, kc, jc, xsh);
                    tma_load_3d(sP(sl, 3), &maps.xph[1], bar, kc, jc, xsh);
                }
            } else {
                if (ye) {
                    const int ys = ye_b ? (int)(p.P[1] + (j0 - 1) - (p.ny - p.P[1] - 1)) : (int)(j0 - 2);
                    tma_load_3d(sP(sl, 0), &maps.ype[0], bar, kc, ys, xc);
                    tma_load_3d(sP(sl, 1), &maps.ype[1], bar, kc, ys, xc);
                }
                if (yh) {
                    const int ys = yh_b ? (int)(p.P[1] + (j0 - 1) - (p.ny - p.P[1])) : (int)(j0 - 2);
                    tma_load_3d(sP(sl, 2), &maps.yph[0], bar, kc, ys, xc);
                    tma_load_3d(sP(sl, 3), &maps.yph[1], bar, kc, ys, xc);
                }
            }
        };

        if (tid == 0) {
            // sources inside the extended region of this work item, in list
            // order (one thread: a warp-wide scan costs the kernel registers)
            int n = 0;
            if (p.t >= 0 && p.t < p.namp) {
                for (int s = 0; s < p.nsrc; s++) {
                    const int64_t si = p.src_ijk[3 * s], sj = p.src_ijk[3 * s + 1], sk = p.src_ijk[3 * s + 2];
                    if (si >= i_start && si < x1 && sj >= j0 - 1 && sj < j0 + TY && sk >= k0 - 1 && sk < k0 + TZ &&
                        !(p.zfix && slab_e(sk, p.P[2], p.nz, ((p.faces >> 4) & 1), ((p.faces >> 5) & 1)) >= 0)) {
                        if (n < MAX_LOCAL_SRC) {
                            // packing: si, sj < 65536 (grid extents) and sk < 2^28 (checked at
                            // plan creation), so neither field overflows
                            s_ls_ij[n] = ((uint32_t)si << 16) | (uint32_t)sj;
                            s_ls_kc[n] = (int)(sk << 2) | p.src_comp[s];
                            s_ls_s[n] = s;
                        }
                        n++;
                    }
                }
                if (n > MAX_LOCAL_SRC) {  // the host rejects such layouts; never drop a source silently
                    atomicExch(p.status, FDTD_ERR_CAPACITY);
                    n = MAX_LOCAL_SRC;
                }
            }
            s_nls = n;
        }
        __syncthreads();  // previous item finished by every thread; source list ready
        if (producer) {
            for (int64_t q = 0; q < NS && q < nplanes; q++) issue(q);
            if (nplanes > 1) issue_psi(0);
        }
        const int nls = s_nls;
        // TFSF faces in this item (E faces at p1-1 and p2, H faces at p1 and p2): the tile's
        // rows and columns meet the box's y/z extent [p1-1, p2], and then either hold a y or
        // z face row/column (all planes of the box's x extent) or, per plane, an x face plane
        const bool t_rows = EXT >= 2 && p.tfsf && j0 - 1 <= p.tp2[1] && j0 + TY - 1 >= p.tp1[1] - 1 &&
                            k0 - 1 <= p.tp2[2] && k0 + TZ - 1 >= p.tp1[2] - 1;
        auto holds = [](int64_t lo, int64_t hi, int64_t v) { return v >= lo && v <= hi; };
        const bool t_yz = t_rows && i_start <= p.tp2[0] && x1 - 1 >= p.tp1[0] - 1 &&
                          (holds(j0 - 1, j0 + TY - 1, p.tp1[1] - 1) || holds(j0 - 1, j0 + TY - 1, p.tp1[1]) ||
                           holds(j0 - 1, j0 + TY - 1, p.tp2[1]) || holds(k0 - 1, k0 + TZ - 1, p.tp1[2] - 1) ||
                           holds(k0 - 1, k0 + TZ - 1, p.tp1[2]) || holds(k0 - 1, k0 + TZ - 1, p.tp2[2]));
        // TFSF face codes of the pair (E, H), zero outside the box's faces
        const uint32_t tcode_e = t_rows ? tfsf_lane_codes(p, 0, jj, kk, in0, in1) : 0u;
        const uint32_t tcode_h = t_rows && h_active ? tfsf_lane_codes(p, 1, jj, kk, in0, in1) : 0u;
        const bool tile_plain = y_plain && nls == 0 && !dtile;

        float2 prev_ey = make_float2(0.f, 0.f), prev_ez = make_float2(0.f, 0.f);
        float2 oex = prev_ey, oey = prev_ey, oez = prev_ey;  // own E_new pair
        for (int64_t q = 0; q + 1 < nplanes; q++) {
            const int64_t i = i_start + q;
            const uint32_t G = g0 + (uint32_t)q;
            const int st = (int)(G % NS), st1 = (int)((G + 1) % NS);
            const uint32_t par = (G / NS) & 1, par1 = ((G + 1) / NS) & 1;
            const uint32_t Gp = gp0 + (uint32_t)q;
            const int psl = (int)(Gp & 1);
            // The producer waits for the copies; the barrier then releases the CTA
            // (its mbarrier acquire plus bar.sync order the TMA writes before
            // every thread's reads).  Plane q+1 is needed for its H only:
            // its E and CE have one more iteration to arrive.
            if (producer &&
                (!mbar_wait_bounded(&bars[st], par, p.status, wlim) ||
                 !mbar_wait_bounded(&bars[st1], par1, p.status, wlim) ||
                 !mbar_wait_bounded(&bars[NS + st], par, p.status, wlim) ||
                 !mbar_wait_bounded(&bars[2 * NS + psl], (Gp >> 1) & 1, p.status, wlim)))
                s_abort = 1;
            __syncthreads();  // (A) H of planes q, q+1, E and CE of q visible; iteration q-1 finished everywhere
            if (s_abort) {
                aborted = true;
                q_abort = q;
                i_start_abort = i_start;
                break;
            }
            if (producer) {
                if (q >= 1 && q - 1 + NS < nplanes) issue(q - 1 + NS);  // reuse plane q-1's stage
                if (q + 2 < nplanes) issue_psi(q + 1);                  // reuse plane q-1's psi slot
            }

            // plane-uniform CPML (x) and masks
            const int sxe = slab_e(i, p.P[0], p.nx, (p.faces & 1), ((p.faces >> 1) & 1)), sxh = slab_h(i, p.P[0], p.nx, (p.faces & 1), ((p.faces >> 1) & 1));
            const bool i_lt = i < p.nx - 1, i_gt = i > 0;
            // plane-uniform: TFSF corrections on this plane
            const bool ttile = t_rows && ((t_yz && i >= p.tp1[0] - 1 && i <= p.tp2[0]) ||
                                          i == p.tp1[0] - 1 || i == p.tp1[0] || i == p.tp2[0]);
            const bool e_plain = tile_plain && i_lt && sxe < 0 && !ttile;
            const bool h_plain = tile_plain && i_gt && sxh < 0 && !ttile;
            // where this plane's x/y psi come from (the choice of issue_psi)
            const bool xm = p.xypsi && (sxe >= 0 || sxh >= 0);
            const bool ym = !xm && ytile;

            // ---- E phase ----
            if (e_active) {
                const int hc = 4 + eko;
                const float *HX = sH(st, 0) + er * HC + hc, *HY = sH(st, 1) + er * HC + hc,
                            *HZ = sH(st, 2) + er * HC + hc;
                const float2 hx = ld2(HX), hy = ld2(HY), hz = ld2(HZ);
                const float2 hxj1 = ld2(HX + HC), hzj1 = ld2(HZ + HC);
                const float2 hxk1 = make_float2(HX[1], HX[2]), hyk1 = make_float2(HY[1], HY[2]);
                const float2 hy1 = ld2(sH(st1, 1) + er * HC + hc), hz1 = ld2(sH(st1, 2) + er * HC + hc);
                const int ei = er * EC + hc;
                const float2 ex0 = ld2(sE(st, 0) + ei), ey0 = ld2(sE(st, 1) + ei), ez0 = ld2(sE(st, 2) + ei);
                const float2 cex = ld2(sC(st, 0) + ei), cey = ld2(sC(st, 1) + ei), cez = ld2(sC(st, 2) + ei);
                float2 ex = add2(ex0, mul2(cex, curl4x2(hzj1, hz, hyk1, hy)));
                float2 ey = add2(ey0, mul2(cey, curl4x2(hxk1, hx, hz1, hz)));
                float2 ez = add2(ez0, mul2(cez, curl4x2(hy1, hy, hxj1, hx)));
                if (!e_plain || emask) {
                    // component masks (cells the reference does not update keep their value)
                    if (!(j_lt && k0_lt)) ex.x = ex0.x;
                    if (!(j_lt && k1_lt)) ex.y = ex0.y;
                    if (!(i_lt && k0_lt)) ey.x = ey0.x;
                    if (!(i_lt && k1_lt)) ey.y = ey0.y;
                    if (!(i_lt && j_lt)) {
                        ez.x = ez0.x;
                        ez.y = ez0.y;
                    }
                }
                if (!e_plain) {
                    const bool own = own_row && i >= x0;
                    if (dtile && i >= p.dbox[0] && i < p.dbox[0] + p.dbox[3] && jj >= p.dbox[1] &&
                        jj < p.dbox[1] + p.dbox[4]) {  // Drude ADE, before the CPML terms
                        const int64_t jb = ((i - p.dbox[0]) * p.dbox[4] + (jj - p.dbox[1])) * p.dbox[5] - p.dbox[2];
#pragma unroll
                        for (int e = 0; e < 2; e++) {
                            const int64_t k = kk + e;
                            if (!(e ? in1 : in0) || k < p.dbox[2] || k >= p.dbox[2] + p.dbox[5]) continue;
                            float jn;
                            set(ex, e, drude_cell(get(ex, e), get(cex, e), p.dj_in[0][jb + k], p.dcja[0][jb + k],
                                                  p.dcjb[0][jb + k], jn));
                            if (own) p.dj_out[0][jb + k] = jn;
                            set(ey, e, drude_cell(get(ey, e), get(cey, e), p.dj_in[1][jb + k], p.dcja[1][jb + k],
                                                  p.dcjb[1][jb + k], jn));
                            if (own) p.dj_out[1][jb + k] = jn;
                            set(ez, e, drude_cell(get(ez, e), get(cez, e), p.dj_in[2][jb + k], p.dcja[2][jb + k],
                                                  p.dcjb[2][jb + k], jn));
                            if (own) p.dj_out[2][jb + k] = jn;
                        }
                    }
                    if (sxe >= 0) {  // x slab: ey -= cey (..dHz/dx..), ez += cez (..dHy/dx..)
                        const Coef c = tab_coef(tabs, 0, 2 * p.P[0], 0, sxe);
                        const int64_t qb = ((int64_t)sxe * p.ny + jj) * p.nz + kk;
#pragma unroll
                        for (int e = 0; e < 2; e++) {
                            if (!(e ? in1 : in0)) continue;
                            if (e ? k1_lt : k0_lt) {
                                float psi = xm ? sP(psl, 0)[er * EC + 4 + eko + e] : (FDTD_IN(qb + e, pext_y(p, 0)) ? p.psi_e_in[0][qb + e] : 0.f);
                                const float tc = corr(psi, c, fsub(get(hz1, e), get(hz, e)));
                                if (own) if (FDTD_IN(qb + e, pext_y(p, 0))) p.psi_e_out[0][qb + e] = psi;
                                set(ey, e, fsub(get(ey, e), fmul(get(cey, e), tc)));
                            }
                            if (j_lt) {
                                float psi = xm ? sP(psl, 1)[er * EC + 4 + eko + e] : (FDTD_IN(qb + e, pext_y(p, 1)) ? p.psi_e_in[1][qb + e] : 0.f);
                                const float tc = corr(psi, c, fsub(get(hy1, e), get(hy, e)));
                                if (own) if (FDTD_IN(qb + e, pext_y(p, 1))) p.psi_e_out[1][qb + e] = psi;
                                set(ez, e, fadd(get(ez, e), fmul(get(cez, e), tc)));
                            }
                        }
                    }
                    if (sye >= 0) {  // y slab: ez -= cez (..dHx/dy..), ex += cex (..dHz/dy..)
                        const Coef cye = tab_coef(tabs, (12 * p.P[0]), 2 * p.P[1], 0, sye);
                        const int64_t qb = (i * 2 * p.P[1] + sye) * p.nz + kk;
#pragma unroll
                        for (int e = 0; e < 2; e++) {
                            if (!(e ? in1 : in0)) continue;
                            if (i_lt) {
                                float psi = ym ? sP(psl, 0)[er * EC + 4 + eko + e] : (FDTD_IN(qb + e, pext_y(p, 2)) ? p.psi_e_in[2][qb + e] : 0.f);
                                const float tc = corr(psi, cye, fsub(get(hxj1, e), get(hx, e)));
                                if (own) if (FDTD_IN(qb + e, pext_y(p, 2))) p.psi_e_out[2][qb + e] = psi;
                                set(ez, e, fsub(get(ez, e), fmul(get(cez, e), tc)));
                            }
                            if (e ? k1_lt : k0_lt) {
                                float psi = ym ? sP(psl, 1)[er * EC + 4 + eko + e] : (FDTD_IN(qb + e, pext_y(p, 3)) ? p.psi_e_in[3][qb + e] : 0.f);
                                const float tc = corr(psi, cye, fsub(get(hzj1, e), get(hz, e)));
                                if (own) if (FDTD_IN(qb + e, pext_y(p, 3))) p.psi_e_out[3][qb + e] = psi;
                                set(ex, e, fadd(get(ex, e), fmul(get(cex, e), tc)));
                            }
                        }
                    }
                    if (ttile && tcode_e) {  // TFSF: E += 0.5 (c * H1d), after the CPML terms, before the sources
                        tfsf_apply(p, 0, tcode_e & 0xfff, i, jj, kk, ex.x, ey.x, ez.x);
                        tfsf_apply(p, 0, tcode_e >> 12, i, jj, kk + 1, ex.y, ey.y, ez.y);
                    }
                    const uint32_t ij_here = ((uint32_t)i << 16) | (uint32_t)jj;
                    for (int s = 0; s < nls; s++) {  // soft sources, list order
                        if (s_ls_ij[s] != ij_here) continue;
                        const int kc = s_ls_kc[s];
                        const int64_t sk = kc >> 2;
                        if (sk != kk && sk != kk + 1) continue;
                        const int e = (int)(sk - kk);
                        const float v = p.src_amp[(int64_t)s_ls_s[s] * p.namp + p.t];
                        const int comp = kc & 3;
                        if (comp == 0) set(ex, e, fadd(get(ex, e), v));
                        else if (comp == 1) set(ey, e, fadd(get(ey, e), v));
                        else set(ez, e, fadd(get(ez, e), v));
                    }
                }
                const int o = er * NCW + 2 + eko;
                st2(Nx + o, ex);
                st2(Ny + o, ey);
                st2(Nz + o, ez);
                oex = ex;
                oey = ey;
                oez = ez;
            }
            __syncthreads();  // (B) E_new of plane i visible

            // ---- H phase: own rows ----
            if (h_active) {
                if (i >= x0) {
                    const int o = er * NCW + 2 + eko;
                    const float2 ez_jm = ld2(Nz + o - NCW), ex_jm = ld2(Nx + o - NCW);
                    const float2 ey_km = make_float2(Ny[o - 1], oey.x), ex_km = make_float2(Nx[o - 1], oex.x);
                    const int hi = er * HC + 4 + eko;
                    const float2 hx0 = ld2(sH(st, 0) + hi), hy0 = ld2(sH(st, 1) + hi), hz0 = ld2(sH(st, 2) + hi);
                    const float2 half = make_float2(0.5f, 0.5f);
                    float2 hx = sub2(hx0, mul2(half, curl4x2(oez, ez_jm, oey, ey_km)));
                    float2 hy = sub2(hy0, mul2(half, curl4x2(oex, ex_km, oez, prev_ez)));
                    float2 hz = sub2(hz0, mul2(half, curl4x2(oey, prev_ey, oex, ex_jm)));
                    if (!h_plain || hmask) {
                        if (!(j_gt && k0_gt)) hx.x = hx0.x;
                        if (!(j_gt && k1_gt)) hx.y = hx0.y;
                        if (!(i_gt && k0_gt)) hy.x = hy0.x;
                        if (!(i_gt && k1_gt)) hy.y = hy0.y;
                        if (!(i_gt && j_gt)) {
                            hz.x = hz0.x;
                            hz.y = hz0.y;
                        }
                    }
                    if (!h_plain) {
                        if (sxh >= 0) {  // x slab: hy += (..dEz/dx..), hz -= (..dEy/dx..)
                            const Coef c = tab_coef(tabs, 0, 2 * p.P[0], 1, sxh);
                            const int64_t qb = ((int64_t)sxh * p.ny + jj) * p.nz + kk;
#pragma unroll
                            for (int e = 0; e < 2; e++) {
                                if (!(e ? in1 : in0) || (e ? hb1 : hb0)) continue;
                                if (e ? k1_gt : k0_gt) {
                                    float psi = xm ? sP(psl, 2)[er * EC + 4 + eko + e] : (FDTD_IN(qb + e, pext_y(p, 0)) ? p.psi_h[0][qb + e] : 0.f);
                                    const float tc = corr(psi, c, fsub(get(oez, e), get(prev_ez, e)));
                                    if (FDTD_IN(qb + e, pext_y(p, 0))) p.psi_h[0][qb + e] = psi;
                                    set(hy, e, fadd(get(hy, e), fmul(0.5f, tc)));
                                }
                                if (j_gt) {
                                    float psi = xm ? sP(psl, 3)[er * EC + 4 + eko + e] : (FDTD_IN(qb + e, pext_y(p, 1)) ? p.psi_h[1][qb + e] : 0.f);
                                    const float tc = corr(psi, c, fsub(get(oey, e), get(prev_ey, e)));
                                    if (FDTD_IN(qb + e, pext_y(p, 1))) p.psi_h[1][qb + e] = psi;
                                    set(hz, e, fsub(get(hz, e), fmul(0.5f, tc)));
                                }
                            }
                        }
                        if (syh >= 0) {  // y slab: hz += (..dEx/dy..), hx -= (..dEz/dy..)
                            const Coef cyh = tab_coef(tabs, (12 * p.P[0]), 2 * p.P[1], 1, syh);
                            const int64_t qb = (i * 2 * p.P[1] + syh) * p.nz + kk;
#pragma unroll
                            for (int e = 0; e < 2; e++) {
                                if (!(e ? in1 : in0) || (e ? hb1 : hb0)) continue;
                                if (i_gt) {
                                    float psi = ym ? sP(psl, 2)[er * EC + 4 + eko + e] : (FDTD_IN(qb + e, pext_y(p, 2)) ? p.psi_h[2][qb + e] : 0.f);
                                    const float tc = corr(psi, cyh, fsub(get(oex, e), get(ex_jm, e)));
                                    if (FDTD_IN(qb + e, pext_y(p, 2))) p.psi_h[2][qb + e] = psi;
                                    set(hz, e, fadd(get(hz, e), fmul(0.5f, tc)));
                                }
                                if (e ? k1_gt : k0_gt) {
                                    float psi = ym ? sP(psl, 3)[er * EC + 4 + eko + e] : (FDTD_IN(qb + e, pext_y(p, 3)) ? p.psi_h[3][qb + e] : 0.f);
                                    const float tc = corr(psi, cyh, fsub(get(oez, e), get(ez_jm, e)));
                                    if (FDTD_IN(qb + e, pext_y(p, 3))) p.psi_h[3][qb + e] = psi;
                                    set(hx, e, fsub(get(hx, e), fmul(0.5f, tc)));
                                }
                            }
                        }
                    }
                    if (ttile && tcode_h) {  // TFSF: H += 0.5 (c * E1d), after the CPML terms
                        tfsf_apply(p, 1, tcode_h & 0xfff, i, jj, kk, hx.x, hy.x, hz.x);
                        tfsf_apply(p, 1, tcode_h >> 12, i, jj, kk + 1, hx.y, hy.y, hz.y);
                    }
                    const int64_t gi = i * p.sx + jj * p.sy + kk;
                    if (in1) {
                        if (FDTD_IN(gi + 1, fext_y(p))) st2(p.out[0] + gi, oex);
                        if (FDTD_IN(gi + 1, fext_y(p))) st2(p.out[1] + gi, oey);
                        if (FDTD_IN(gi + 1, fext_y(p))) st2(p.out[2] + gi, oez);
                        if (FDTD_IN(gi + 1, fext_y(p))) st2(p.out[3] + gi, hx);
                        if (FDTD_IN(gi + 1, fext_y(p))) st2(p.out[4] + gi, hy);
                        if (FDTD_IN(gi + 1, fext_y(p))) st2(p.out[5] + gi, hz);
                    } else if (in0) {
                        if (FDTD_IN(gi, fext_y(p))) p.out[0][gi] = oex.x;
                        if (FDTD_IN(gi, fext_y(p))) p.out[1][gi] = oey.x;
                        if (FDTD_IN(gi, fext_y(p))) p.out[2][gi] = oez.x;
                        if (FDTD_IN(gi, fext_y(p))) p.out[3][gi] = hx.x;
                        if (FDTD_IN(gi, fext_y(p))) p.out[4][gi] = hy.x;
                        if (FDTD_IN(gi, fext_y(p))) p.out[5][gi] = hz.x;
                    }
                }
                prev_ey = oey;
                prev_ez = oez;
            }
        }
        if (aborted) break;
        first_item = false;
        g0 += (uint32_t)nplanes;
        gp0 += (uint32_t)(nplanes - 1);  // one psi phase per iteration
        issued_hi = -1;
        psi_hi = -1;
        if (BATCH) {
            __syncthreads();  // every thread has read s_item
            if (tid == 0) s_item = atomicAdd(&bd.queue[0], 1);
            __syncthreads();
            gitem = s_item;
        } else {
            gitem += gridDim.x;
        }
    }

    if (BATCH && tid == 0) {
        // the last CTA to finish clears the queue for the next launch
        __threadfence();
        if (atomicAdd(&bd.queue[1], 1) == (int)gridDim.x - 1) {
            bd.queue[0] = 0;
            bd.queue[1] = 0;
            __threadfence();
        }
    }
    if (aborted) {
        if (producer) {
            atomicExch(p.status, FDTD_ERR_TIMEOUT);
            // Let the copies still in flight land before the CTA's shared
            // memory is released (each wait bounded).
            for (int64_t q = q_abort; q <= issued_hi; q++) {
                if (i_start_abort + q >= p.nx) continue;
                const uint32_t G = g0 + (uint32_t)q;
                mbar_wait_bounded(&bars[G % NS], (G / NS) & 1, nullptr, wlim);
                mbar_wait_bounded(&bars[NS + G % NS], (G / NS) & 1, nullptr, wlim);
            }
            for (int64_t q = q_abort; q <= psi_hi; q++) {
                const uint32_t Gp = gp0 + (uint32_t)q;
                mbar_wait_bounded(&bars[2 * NS + (Gp & 1)], (Gp >> 1) & 1, nullptr, wlim);
            }
        }
        __syncthreads();
    }
}
#undef FDTD_SB

// ---------------------------------------------------------------------------
// z band kernels (single-grid plans).  The fused kernel treats z-slab tiles
// like interior tiles; these two kernels then finish the band in the same
// operation order as the in-kernel path (and the reference's cpml_e/cpml_h):
//   E: on E z-slab nodes, psi_e(z) update and E correction, then the sources
//      on those cells (list order);
//   H: on k in [1, P+1] and [n-P-1, n-1], H recomputed from the input buffer
//      and the final E with its x, y and z CPML terms (x/y psi_h were left
//      untouched there by the fused kernel).
// One thread per cell; z is the fastest index inside each band.
// ---------------------------------------------------------------------------
__device__ __forceinline__ Coef gcoef(const float *b, const float *a, const float *k, int s) {
    return Coef{b[s], a[s], k[s]};
}

// band cell counts of one grid: E (E z-slab nodes) and H (k in the H band)
__host__ __device__ __forceinline__ int64_t zband_e_cells(const Params &p) {
    const int P = p.P[2], f = (p.faces >> 4) & 1, b = (p.faces >> 5) & 1;
    return p.zfix ? p.nx * p.ny * (int64_t)((f + b) * P) : 0;
}
__host__ __device__ __forceinline__ int64_t zband_h_start(const Params &p) {
    const int P = p.P[2], f = (p.faces >> 4) & 1, b = (p.faces >> 5) & 1;
    const int64_t fend = f ? P + 1 : 0;
    return b ? (p.nz - P - 1 > fend + 1 ? p.nz - P - 1 : fend + 1) : p.nz;
}
__host__ __device__ __forceinline__ int64_t zband_h_cells(const Params &p) {
    const int P = p.P[2], f = (p.faces >> 4) & 1;
    const int64_t fend = f ? P + 1 : 0;
    return p.zfix ? p.nx * p.ny * (fend + p.nz - zband_h_start(p)) : 0;
}

// E band cell number t of grid p at step tstep.  All loads come first, then
// the arithmetic, then the stores: a store could alias a later load as far as
// the compiler knows, so loads placed after stores would not be overlapped.
// E band cells per (i, j) row: the front slab's nodes, then the back slab's
__device__ __forceinline__ int zband_e_row(const Params &p) {
    return (((p.faces >> 4) & 1) ? p.P[2] : 0) + (((p.faces >> 5) & 1) ? p.P[2] : 0);
}

// E band cell kb of row (i, j)
__device__ __forceinline__ void zband_e_at(const Params &p, int64_t tstep, int64_t i, int64_t j, int kb) {
    const int P = p.P[2];
    const int nf = ((p.faces >> 4) & 1) ? P : 0;
    const int64_t k = kb < nf ? 1 + kb : p.nz - P - 1 + (kb - nf);
    const int sz = kb < nf ? kb : P + (kb - nf);
    const int64_t c = i * p.sx + j * p.sy + k, qz = (i * p.ny + j) * 2 * P + sz;
    const Coef cf = gcoef(p.tb_e[2], p.ta_e[2], p.tk_e[2], sz);
    const bool ux = j < p.ny - 1, uy = i < p.nx - 1;  // exz / eyz elements that exist
    float px = 0.f, py = 0.f, hyd = 0.f, hxd = 0.f, ex = 0.f, ey = 0.f, cx = 0.f, cy = 0.f;
    if (ux) {
        px = (FDTD_IN(qz, pext_y(p, 4)) ? p.psi_e_in[4][qz] : 0.f);
        hyd = fsub((FDTD_IN(c + 1, fext_y(p)) ? p.in[4][c + 1] : 0.f), (FDTD_IN(c, fext_y(p)) ? p.in[4][c] : 0.f));
        ex = (FDTD_IN(c, fext_y(p)) ? p.out[0][c] : 0.f);
        cx = (FDTD_IN(c, fext_y(p)) ? p.in_ce[0][c] : 0.f);
    }
    if (uy) {
        py = (FDTD_IN(qz, pext_y(p, 5)) ? p.psi_e_in[5][qz] : 0.f);
        hxd = fsub((FDTD_IN(c + 1, fext_y(p)) ? p.in[3][c + 1] : 0.f), (FDTD_IN(c, fext_y(p)) ? p.in[3][c] : 0.f));
        ey = (FDTD_IN(c, fext_y(p)) ? p.out[1][c] : 0.f);
        cy = (FDTD_IN(c, fext_y(p)) ? p.in_ce[1][c] : 0.f);
    }
    if (ux) {  // ex -= cex (..dHy/dz..)
        const float tc = corr(px, cf, hyd);
        if (FDTD_IN(qz, pext_y(p, 4))) p.psi_e_out[4][qz] = px;
        if (FDTD_IN(c, fext_y(p))) p.out[0][c] = fsub(ex, fmul(cx, tc));
    }
    if (uy) {  // ey += cey (..dHx/dz..)
        const float tc = corr(py, cf, hxd);
        if (FDTD_IN(qz, pext_y(p, 5))) p.psi_e_out[5][qz] = py;
        if (FDTD_IN(c, fext_y(p))) p.out[1][c] = fadd(ey, fmul(cy, tc));
    }
    if (tstep >= 0 && tstep < p.namp) {  // sources on this cell, list order
        const int n = p.nbsrc < 0 ? p.nsrc : p.nbsrc;
        for (int b = 0; b < n; b++) {
            const int s = p.nbsrc < 0 ? b : p.bsrc[b];
            if (p.src_ijk[3 * s] != i || p.src_ijk[3 * s + 1] != j || p.src_ijk[3 * s + 2] != k) continue;
            float *f = p.out[p.src_comp[s]] + c;
            if (FDTD_IN(c, fext_y(p))) *f = fadd(*f, p.src_amp[(int64_t)s * p.namp + tstep]);
        }
    }
}

// E band cell number t of grid p (rows of zband_e_row cells, z fastest)
__device__ __forceinline__ void zband_e_cell(const Params &p, int64_t tstep, int64_t t) {
    const int nk = zband_e_row(p);
    zband_e_at(p, tstep, t / ((int64_t)nk * p.ny), (t / nk) % p.ny, (int)(t % nk));
}

// H band cells per (i, j) row: k = 1 .. P+1 (front), then bstart .. nz-1 (back)
__device__ __forceinline__ int zband_h_row(const Params &p) {
    const int64_t fend = ((p.faces >> 4) & 1) ? p.P[2] + 1 : 0;
    return (int)(fend + (p.nz - zband_h_start(p)));
}

// H band cell kb of row (i, j): H recomputed from the input buffer and the
// final E, with its curl, then the x, y and z CPML terms (in-kernel order)
__device__ __forceinline__ void zband_h_at(const Params &p, int64_t i, int64_t j, int kb) {
    const int P = p.P[2];
    const int front = (p.faces >> 4) & 1, back = (p.faces >> 5) & 1;
    const int64_t nz = p.nz, ny = p.ny, nx = p.nx;
    const int64_t fend = front ? P + 1 : 0;          // front band: k = 1 .. fend
    const int64_t bstart = zband_h_start(p);         // back band: k = bstart .. nz-1
    const int nf = (int)fend;
    const int64_t k = kb < nf ? 1 + kb : bstart + (kb - nf);
    const int64_t c = i * p.sx + j * p.sy + k;
    const int f0 = p.faces & 1, b0 = (p.faces >> 1) & 1, f1 = (p.faces >> 2) & 1, b1 = (p.faces >> 3) & 1;
    const int sxh = slab_h(i, p.P[0], nx, f0, b0), syh = slab_h(j, p.P[1], ny, f1, b1);
    const int szh = slab_h(k, P, nz, front, back);
    const int P1 = p.P[1];
    const bool ux = j > 0 && k > 0, uy = i > 0 && k > 0, uz = i > 0 && j > 0;  // update masks
    // ---- loads
    const float *__restrict__ ex = p.out[0];
    const float *__restrict__ ey = p.out[1];
    const float *__restrict__ ez = p.out[2];
    const float hx0 = (FDTD_IN(c, fext_y(p)) ? p.in[3][c] : 0.f), hy0 = (FDTD_IN(c, fext_y(p)) ? p.in[4][c] : 0.f), hz0 = (FDTD_IN(c, fext_y(p)) ? p.in[5][c] : 0.f);
    const float ex_c = (FDTD_IN(c, fext_y(p)) ? ex[c] : 0.f), ey_c = (FDTD_IN(c, fext_y(p)) ? ey[c] : 0.f), ez_c = (FDTD_IN(c, fext_y(p)) ? ez[c] : 0.f);
    const float ez_j = j > 0 ? (FDTD_IN(c - p.sy, fext_y(p)) ? ez[c - p.sy] : 0.f) : 0.f, ex_j = j > 0 ? (FDTD_IN(c - p.sy, fext_y(p)) ? ex[c - p.sy] : 0.f) : 0.f;
    const float ey_i = i > 0 ? (FDTD_IN(c - p.sx, fext_y(p)) ? ey[c - p.sx] : 0.f) : 0.f, ez_i = i > 0 ? (FDTD_IN(c - p.sx, fext_y(p)) ? ez[c - p.sx] : 0.f) : 0.f;
    const float ey_k = (FDTD_IN(c - 1, fext_y(p)) ? ey[c - 1] : 0.f), ex_k = (FDTD_IN(c - 1, fext_y(p)) ? ex[c - 1] : 0.f);  // k >= 1 in the band
    const int64_t qy = syh >= 0 ? (i * 2 * P1 + syh) * nz + k : 0;
    const int64_t qx = sxh >= 0 ? ((int64_t)sxh * ny + j) * nz + k : 0;
    const int64_t qz = szh >= 0 ? (i * ny + j) * 2 * P + szh : 0;
    float ps_hxy = 0.f, ps_hxz = 0.f, ps_hyx = 0.f, ps_hyz = 0.f, ps_hzx = 0.f, ps_hzy = 0.f;
    if (syh >= 0) {
        if (ux) ps_hxy = (FDTD_IN(qy, pext_y(p, 3)) ? p.psi_h[3][qy] : 0.f);
        if (uz) ps_hzy = (FDTD_IN(qy, pext_y(p, 2)) ? p.psi_h[2][qy] : 0.f);
    }
    if (sxh >= 0) {
        if (uy) ps_hyx = (FDTD_IN(qx, pext_y(p, 0)) ? p.psi_h[0][qx] : 0.f);
        if (uz) ps_hzx = (FDTD_IN(qx, pext_y(p, 1)) ? p.psi_h[1][qx] : 0.f);
    }
    if (szh >= 0) {
        if (ux) ps_hxz = (FDTD_IN(qz, pext_y(p, 4)) ? p.psi_h[4][qz] : 0.f);
        if (uy) ps_hyz = (FDTD_IN(qz, pext_y(p, 5)) ? p.psi_h[5][qz] : 0.f);
    }
    // ---- arithmetic
    float hx = hx0, hy = hy0, hz = hz0;
    if (ux) {
        hx = fsub(hx, fmul(0.5f, curl4(ez_c, ez_j, ey_c, ey_k)));
        if (syh >= 0)
            hx = fsub(hx, fmul(0.5f, corr(ps_hxy, gcoef(p.tb_h[1], p.ta_h[1], p.tk_h[1], syh), fsub(ez_c, ez_j))));
        if (szh >= 0)
            hx = fadd(hx, fmul(0.5f, corr(ps_hxz, gcoef(p.tb_h[2], p.ta_h[2], p.tk_h[2], szh), fsub(ey_c, ey_k))));
    }
    if (uy) {
        hy = fsub(hy, fmul(0.5f, curl4(ex_c, ex_k, ez_c, ez_i)));
        if (sxh >= 0)
            hy = fadd(hy, fmul(0.5f, corr(ps_hyx, gcoef(p.tb_h[0], p.ta_h[0], p.tk_h[0], sxh), fsub(ez_c, ez_i))));
        if (szh >= 0)
            hy = fsub(hy, fmul(0.5f, corr(ps_hyz, gcoef(p.tb_h[2], p.ta_h[2], p.tk_h[2], szh), fsub(ex_c, ex_k))));
    }
    if (uz) {
        hz = fsub(hz, fmul(0.5f, curl4(ey_c, ey_i, ex_c, ex_j)));
        if (sxh >= 0)
            hz = fsub(hz, fmul(0.5f, corr(ps_hzx, gcoef(p.tb_h[0], p.ta_h[0], p.tk_h[0], sxh), fsub(ey_c, ey_i))));
        if (syh >= 0)
            hz = fadd(hz, fmul(0.5f, corr(ps_hzy, gcoef(p.tb_h[1], p.ta_h[1], p.tk_h[1], syh), fsub(ex_c, ex_j))));
    }
    // ---- stores
    if (FDTD_IN(c, fext_y(p))) p.out[3][c] = hx;
    if (FDTD_IN(c, fext_y(p))) p.out[4][c] = hy;
    if (FDTD_IN(c, fext_y(p))) p.out[5][c] = hz;
    if (syh >= 0) {
        if (ux) if (FDTD_IN(qy, pext_y(p, 3))) p.psi_h[3][qy] = ps_hxy;
        if (uz) if (FDTD_IN(qy, pext_y(p, 2))) p.psi_h[2][qy] = ps_hzy;
    }
    if (sxh >= 0) {
        if (uy) if (FDTD_IN(qx, pext_y(p, 0))) p.psi_h[0][qx] = ps_hyx;
        if (uz) if (FDTD_IN(qx, pext_y(p, 1))) p.psi_h[1][qx] = ps_hzx;
    }
    if (szh >= 0) {
        if (ux) if (FDTD_IN(qz, pext_y(p, 4))) p.psi_h[4][qz] = ps_hxz;
        if (uy) if (FDTD_IN(qz, pext_y(p, 5))) p.psi_h[5][qz] = ps_hyz;
    }
}

// H band cell number t of grid p (rows of zband_h_row cells, z fastest)
__device__ __forceinline__ void zband_h_cell(const Params &p, int64_t t) {
    const int nk = zband_h_row(p);
    zband_h_at(p, t / ((int64_t)nk * p.ny), (t / nk) % p.ny, (int)(t % nk));
}

struct BandBatch {
    int32_t nsims, cur;
    int64_t t;
    const Params *params;   // [2*nsims], as BatchDesc
    const int64_t *off;     // [nsims + 1]
};

__device__ __forceinline__ int band_sim(const BandBatch &d, int64_t t) {
    int lo = 0, hi = d.nsims - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (d.off[mid] <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}


// Host stub of one fused-kernel instantiation (launched through a pointer).
typedef void (*FusedKernel)(const TMaps, const Params, const BatchDesc);

// Tile heights and pipeline depths compiled in: X(TY, NS) for each.
#define FDTD_FUSED_TILES(X) X(4, 3) X(4, 4) X(4, 6) X(8, 3) X(8, 4) X(16, 3)

// Instantiations compiled in separate translation units (the build compiles
// them in parallel): single-grid kernels (EXT 0..2) and batched kernels
// (EXT 0..1).  false when (ty, ns) is not compiled in.
bool single_kernels(int ty, int ns, FusedKernel out[3]);
bool batch_kernels(int ty, int ns, FusedKernel out[2]);

}  // namespace fused
}  // namespace fdtd
