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
//  * A CTA owns a tile of TZ=32 (z) x TY (y) cells for a chunk of x planes
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
#include <cuda.h>

#include "common.cuh"

namespace fdtd {
namespace fused {

constexpr int TZ = 32;
constexpr int HC = TZ + 8;  // H box: k0-4 .. k0+TZ+3 (needs k0-1 .. k0+TZ)
constexpr int EC = TZ + 4;  // E/CE box: k0-4 .. k0+TZ-1 (needs k0-1 .. k0+TZ-1)
constexpr int NS = 4;       // pipeline stages (planes in flight)
constexpr int MAX_LOCAL_SRC = 16;
constexpr uint64_t WAIT_NS = 1000000000ull;  // a wait gives up after 1 s

constexpr int al128(int b) { return (b + 127) / 128 * 128; }

template <int TY>
struct Layout {
    static constexpr int HR = TY + 2, ER = TY + 1;
    static constexpr int HBOX = HR * HC, EBOX = ER * EC;  // floats per component box
    static constexpr int HBOXB = al128(HBOX * 4), EBOXB = al128(EBOX * 4);
    static constexpr int STAGE = 3 * HBOXB + 6 * EBOXB;  // H(3), E(3), CE(3)
    static constexpr uint32_t TX = 3 * HBOX * 4 + 6 * EBOX * 4;
    static constexpr int NR = TY + 1, NC = TZ + 1;
    static constexpr int ENEW = al128(3 * NR * NC * 4);
    static constexpr int SMEM = NS * STAGE + ENEW + 128 /*barriers*/ + 128 /*align slack*/;
};

struct TMaps {
    CUtensorMap h[3];   // hx, hy, hz of the input buffer, box (HC, TY+2, 1)
    CUtensorMap e[3];   // ex, ey, ez of the input buffer, box (EC, TY+1, 1)
    CUtensorMap ce[3];  // cex, cey, cez,                  box (EC, TY+1, 1)
};

struct Params {
    int64_t nx, ny, nz, sx, sy;
    int32_t ntz, nty, x_chunk;
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

// Bounded wait: true on completion; false after WAIT_NS, or early when
// another CTA has already recorded a timeout in the status word (status may
// be null: then only the deadline applies).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, const int32_t *status) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t n = 1;; n++) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((n & 255) == 0) {
            if (globaltimer_ns() - t0 > WAIT_NS) return false;
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

__device__ __forceinline__ float cpml_corr(float &psi, float b, float a, float km1, float d) {
    psi = fadd(fmul(b, psi), fmul(a, d));
    return fadd(fmul(km1, d), psi);
}

template <int TY>
__global__ void __launch_bounds__(TY * 32)
k_yee_fused(const __grid_constant__ TMaps maps, const Params p) {
    using L = Layout<TY>;
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem =
        reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    float *enew = reinterpret_cast<float *>(smem + NS * L::STAGE);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + NS * L::STAGE + L::ENEW);

    __shared__ int s_abort;
    __shared__ int s_nls;
    __shared__ int s_ls_i[MAX_LOCAL_SRC], s_ls_r[MAX_LOCAL_SRC], s_ls_c[MAX_LOCAL_SRC];
    __shared__ int s_ls_comp[MAX_LOCAL_SRC], s_ls_s[MAX_LOCAL_SRC];

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int item = blockIdx.x;
    const int tzi = item % p.ntz, tyi = (item / p.ntz) % p.nty, xci = item / (p.ntz * p.nty);
    const int64_t k0 = (int64_t)tzi * TZ, j0 = (int64_t)tyi * TY;
    const int64_t x0 = (int64_t)xci * p.x_chunk;
    const int64_t x1 = min(x0 + (int64_t)p.x_chunk, p.nx);
    const int64_t i_start = x0 > 0 ? x0 - 1 : 0;
    const int64_t last_plane = x1;  // H(x1) feeds E(x1-1); beyond nx the box is zero-filled

    auto stage_ptr = [&](int st) { return smem + st * L::STAGE; };
    auto sH = [&](int st, int c) { return reinterpret_cast<float *>(stage_ptr(st) + c * L::HBOXB); };
    auto sE = [&](int st, int c) { return reinterpret_cast<float *>(stage_ptr(st) + 3 * L::HBOXB + c * L::EBOXB); };
    auto sC = [&](int st, int c) {
        return reinterpret_cast<float *>(stage_ptr(st) + 3 * L::HBOXB + (3 + c) * L::EBOXB);
    };

    int64_t issued[NS];  // plane last issued into each stage (meaningful on tid 0)
    for (int s = 0; s < NS; s++) issued[s] = -1;
    auto issue = [&](int64_t plane, int st) {
        uint64_t *bar = &bars[st];
        issued[st] = plane;
        if (plane >= p.nx) {
            // Past the last plane: H(nx) only feeds E components that are never
            // updated at i = nx-1, so the stage content is irrelevant; complete
            // the phase without a copy.
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
            return;
        }
        mbar_arrive_expect_tx(bar, L::TX);
        const int kc = (int)(k0 - 4), jc = (int)(j0 - 1), xc = (int)plane;
        for (int c = 0; c < 3; c++) tma_load_3d(sH(st, c), &maps.h[c], bar, kc, jc, xc);
        for (int c = 0; c < 3; c++) tma_load_3d(sE(st, c), &maps.e[c], bar, kc, jc, xc);
        for (int c = 0; c < 3; c++) tma_load_3d(sC(st, c), &maps.ce[c], bar, kc, jc, xc);
    };

    if (tid == 0) {
        for (int s = 0; s < NS; s++) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        for (int c = 0; c < 3; c++) {
            prefetch_tmap(&maps.h[c]);
            prefetch_tmap(&maps.e[c]);
            prefetch_tmap(&maps.ce[c]);
        }
        s_abort = 0;
        // sources touching the extended region of this work item
        int n = 0;
        if (p.t >= 0 && p.t < p.namp) {
            for (int s = 0; s < p.nsrc; s++) {
                const int64_t si = p.src_ijk[3 * s], sj = p.src_ijk[3 * s + 1], sk = p.src_ijk[3 * s + 2];
                if (si >= i_start && si < x1 && sj >= j0 - 1 && sj < j0 + TY && sk >= k0 - 1 && sk < k0 + TZ) {
                    if (n < MAX_LOCAL_SRC) {
                        s_ls_i[n] = (int)si;
                        s_ls_r[n] = (int)(sj - j0 + 1);
                        s_ls_c[n] = (int)(sk - k0 + 1);
                        s_ls_comp[n] = p.src_comp[s];
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
    __syncthreads();
    if (tid == 0)
        for (int r = 0; r < NS; r++)
            if (i_start + r <= last_plane) issue(i_start + r, r);

    const int64_t nx = p.nx, ny = p.ny, nz = p.nz;
    const int front0 = p.faces & 1, back0 = (p.faces >> 1) & 1;
    const int front1 = (p.faces >> 2) & 1, back1 = (p.faces >> 3) & 1;
    const int front2 = (p.faces >> 4) & 1, back2 = (p.faces >> 5) & 1;
    const float *amp = p.src_amp;

    float prev_ey = 0.f, prev_ez = 0.f;

    // E_new of one cell at smem row r (j = j0-1+r) and column c (k = k0-1+c).
    // own: the cell belongs to this tile (psi_e_out is written only then).
    auto compute_e = [&](int st, int st1, int64_t i, int r, int c, bool own, float &oex, float &oey, float &oez) {
        const int64_t j = j0 - 1 + r, k = k0 - 1 + c;
        const int hr = r, hc = c + 3;
        const float *hx = sH(st, 0), *hy = sH(st, 1), *hz = sH(st, 2);
        const float *hy1 = sH(st1, 1), *hz1 = sH(st1, 2);
        const int hi = hr * HC + hc, ei = r * EC + hc;
        const float hx0 = hx[hi], hy0 = hy[hi], hz0 = hz[hi];
        float ex = sE(st, 0)[ei], ey = sE(st, 1)[ei], ez = sE(st, 2)[ei];
        const float cex = sC(st, 0)[ei], cey = sC(st, 1)[ei], cez = sC(st, 2)[ei];
        const bool in = j >= 0 && k >= 0 && j < ny && k < nz;
        if (in) {
            if (j < ny - 1 && k < nz - 1) ex = fadd(ex, fmul(cex, curl4(hz[hi + HC], hz0, hy[hi + 1], hy0)));
            if (i < nx - 1 && k < nz - 1) ey = fadd(ey, fmul(cey, curl4(hx[hi + 1], hx0, hz1[hi], hz0)));
            if (i < nx - 1 && j < ny - 1) ez = fadd(ez, fmul(cez, curl4(hy1[hi], hy0, hx[hi + HC], hx0)));
            // CPML, x axis (plane-uniform branch)
            const int sxs = slab_e(i, p.P[0], nx, front0, back0);
            if (sxs >= 0) {
                const float b = __ldg(&p.tb_e[0][sxs]), a = __ldg(&p.ta_e[0][sxs]), km = __ldg(&p.tk_e[0][sxs]);
                const int64_t q = ((int64_t)sxs * ny + j) * nz + k;
                if (k < nz - 1) {
                    float psi = p.psi_e_in[0][q];
                    const float tcorr = cpml_corr(psi, b, a, km, fsub(hz1[hi], hz0));
                    if (own) p.psi_e_out[0][q] = psi;
                    ey = fsub(ey, fmul(cey, tcorr));
                }
                if (j < ny - 1) {
                    float psi = p.psi_e_in[1][q];
                    const float tcorr = cpml_corr(psi, b, a, km, fsub(hy1[hi], hy0));
                    if (own) p.psi_e_out[1][q] = psi;
                    ez = fadd(ez, fmul(cez, tcorr));
                }
            }
            const int sys = slab_e(j, p.P[1], ny, front1, back1);
            if (sys >= 0) {
                const float b = __ldg(&p.tb_e[1][sys]), a = __ldg(&p.ta_e[1][sys]), km = __ldg(&p.tk_e[1][sys]);
                const int64_t q = (i * 2 * p.P[1] + sys) * nz + k;
                if (i < nx - 1) {
                    float psi = p.psi_e_in[2][q];
                    const float tcorr = cpml_corr(psi, b, a, km, fsub(hx[hi + HC], hx0));
                    if (own) p.psi_e_out[2][q] = psi;
                    ez = fsub(ez, fmul(cez, tcorr));
                }
                if (k < nz - 1) {
                    float psi = p.psi_e_in[3][q];
                    const float tcorr = cpml_corr(psi, b, a, km, fsub(hz[hi + HC], hz0));
                    if (own) p.psi_e_out[3][q] = psi;
                    ex = fadd(ex, fmul(cex, tcorr));
                }
            }
            const int szs = slab_e(k, p.P[2], nz, front2, back2);
            if (szs >= 0) {
                const float b = __ldg(&p.tb_e[2][szs]), a = __ldg(&p.ta_e[2][szs]), km = __ldg(&p.tk_e[2][szs]);
                const int64_t q = (i * ny + j) * 2 * p.P[2] + szs;
                if (j < ny - 1) {
                    float psi = p.psi_e_in[4][q];
                    const float tcorr = cpml_corr(psi, b, a, km, fsub(hy[hi + 1], hy0));
                    if (own) p.psi_e_out[4][q] = psi;
                    ex = fsub(ex, fmul(cex, tcorr));
                }
                if (i < nx - 1) {
                    float psi = p.psi_e_in[5][q];
                    const float tcorr = cpml_corr(psi, b, a, km, fsub(hx[hi + 1], hx0));
                    if (own) p.psi_e_out[5][q] = psi;
                    ey = fadd(ey, fmul(cey, tcorr));
                }
            }
            for (int q = 0; q < s_nls; q++) {
                if (s_ls_i[q] == i && s_ls_r[q] == r && s_ls_c[q] == c) {
                    const float v = amp[(int64_t)s_ls_s[q] * p.namp + p.t];
                    if (s_ls_comp[q] == 0) ex = fadd(ex, v);
                    else if (s_ls_comp[q] == 1) ey = fadd(ey, v);
                    else ez = fadd(ez, v);
                }
            }
        }
        oex = ex;
        oey = ey;
        oez = ez;
    };

    constexpr int NRC = L::NR * L::NC;
    for (int64_t i = i_start; i < x1; i++) {
        const int64_t rel = i - i_start;
        const int st = (int)(rel % NS), st1 = (int)((rel + 1) % NS);
        const uint32_t par = (uint32_t)((rel / NS) & 1), par1 = (uint32_t)(((rel + 1) / NS) & 1);
        if (!mbar_wait_bounded(&bars[st], par, p.status) || !mbar_wait_bounded(&bars[st1], par1, p.status))
            s_abort = 1;
        __syncthreads();
        if (s_abort) break;

        // ---- E_new on the tile (own cells) and the j0-1 / k0-1 halo ----
        float ex_o, ey_o, ez_o;
        compute_e(st, st1, i, w + 1, lane + 1, i >= x0, ex_o, ey_o, ez_o);
        {
            const int o = (w + 1) * L::NC + lane + 1;
            enew[o] = ex_o;
            enew[NRC + o] = ey_o;
            enew[2 * NRC + o] = ez_o;
        }
        for (int x = tid; x < TZ + TY + 1; x += TY * 32) {
            const int r = x < TZ ? 0 : x - TZ, c = x < TZ ? x + 1 : 0;
            float a, b, d;
            compute_e(st, st1, i, r, c, false, a, b, d);
            const int o = r * L::NC + c;
            enew[o] = a;
            enew[NRC + o] = b;
            enew[2 * NRC + o] = d;
        }
        __syncthreads();

        const int64_t j = j0 + w, k = k0 + lane;
        if (i >= x0 && j < ny && k < nz) {
            const int o = (w + 1) * L::NC + lane + 1;
            const float *Ex = enew, *Ey = enew + NRC, *Ez = enew + 2 * NRC;
            const int hi = (w + 1) * HC + lane + 4;
            float hx = sH(st, 0)[hi], hy = sH(st, 1)[hi], hz = sH(st, 2)[hi];
            if (j > 0 && k > 0) hx = fsub(hx, fmul(0.5f, curl4(ez_o, Ez[o - L::NC], ey_o, Ey[o - 1])));
            if (i > 0 && k > 0) hy = fsub(hy, fmul(0.5f, curl4(ex_o, Ex[o - 1], ez_o, prev_ez)));
            if (i > 0 && j > 0) hz = fsub(hz, fmul(0.5f, curl4(ey_o, prev_ey, ex_o, Ex[o - L::NC])));
            const int sxs = slab_h(i, p.P[0], nx, front0, back0);
            if (sxs >= 0) {
                const float b = __ldg(&p.tb_h[0][sxs]), a = __ldg(&p.ta_h[0][sxs]), km = __ldg(&p.tk_h[0][sxs]);
                const int64_t q = ((int64_t)sxs * ny + j) * nz + k;
                if (k > 0) {
                    float psi = p.psi_h[0][q];
                    const float tcorr = cpml_corr(psi, b, a, km, fsub(ez_o, prev_ez));
                    p.psi_h[0][q] = psi;
                    hy = fadd(hy, fmul(0.5f, tcorr));
                }
                if (j > 0) {
                    float psi = p.psi_h[1][q];
                    const float tcorr = cpml_corr(psi, b, a, km, fsub(ey_o, prev_ey));
                    p.psi_h[1][q] = psi;
                    hz = fsub(hz, fmul(0.5f, tcorr));
                }
            }
            const int sys = slab_h(j, p.P[1], ny, front1, back1);
            if (sys >= 0) {
                const float b = __ldg(&p.tb_h[1][sys]), a = __ldg(&p.ta_h[1][sys]), km = __ldg(&p.tk_h[1][sys]);
                const int64_t q = (i * 2 * p.P[1] + sys) * nz + k;
                if (i > 0) {
                    float psi = p.psi_h[2][q];
                    const float tcorr = cpml_corr(psi, b, a, km, fsub(ex_o, Ex[o - L::NC]));
                    p.psi_h[2][q] = psi;
                    hz = fadd(hz, fmul(0.5f, tcorr));
                }
                if (k > 0) {
                    float psi = p.psi_h[3][q];
                    const float tcorr = cpml_corr(psi, b, a, km, fsub(ez_o, Ez[o - L::NC]));
                    p.psi_h[3][q] = psi;
                    hx = fsub(hx, fmul(0.5f, tcorr));
                }
            }
            const int szs = slab_h(k, p.P[2], nz, front2, back2);
            if (szs >= 0) {
                const float b = __ldg(&p.tb_h[2][szs]), a = __ldg(&p.ta_h[2][szs]), km = __ldg(&p.tk_h[2][szs]);
                const int64_t q = (i * ny + j) * 2 * p.P[2] + szs;
                if (j > 0) {
                    float psi = p.psi_h[4][q];
                    const float tcorr = cpml_corr(psi, b, a, km, fsub(ey_o, Ey[o - 1]));
                    p.psi_h[4][q] = psi;
                    hx = fadd(hx, fmul(0.5f, tcorr));
                }
                if (i > 0) {
                    float psi = p.psi_h[5][q];
                    const float tcorr = cpml_corr(psi, b, a, km, fsub(ex_o, Ex[o - 1]));
                    p.psi_h[5][q] = psi;
                    hy = fsub(hy, fmul(0.5f, tcorr));
                }
            }
            const int64_t g = i * p.sx + j * p.sy + k;
            p.out[0][g] = ex_o;
            p.out[1][g] = ey_o;
            p.out[2][g] = ez_o;
            p.out[3][g] = hx;
            p.out[4][g] = hy;
            p.out[5][g] = hz;
        }
        prev_ey = ey_o;
        prev_ez = ez_o;
        __syncthreads();  // stage st and enew are free again
        if (tid == 0 && i + NS <= last_plane) issue(i + NS, st);
    }

    if (s_abort) {
        if (tid == 0) {
            atomicExch(p.status, FDTD_ERR_TIMEOUT);
            // Let the copies still in flight land before the CTA's shared
            // memory is released (each wait bounded).
            for (int s = 0; s < NS; s++) {
                if (issued[s] < 0 || issued[s] >= p.nx) continue;
                const int64_t rel = issued[s] - i_start;
                mbar_wait_bounded(&bars[s], (uint32_t)((rel / NS) & 1), nullptr);
            }
        }
        __syncthreads();
    }
}

}  // namespace fused
}  // namespace fdtd

// ---------------------------------------------------------------------------
// Host side: plan = encoded tensor maps + launch configuration.
// ---------------------------------------------------------------------------
using namespace fdtd;
using namespace fdtd::fused;

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn get_encode_fn() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        fn = reinterpret_cast<EncodeTiledFn>(ptr);
    }
    return fn;
}

struct fdtd_yee_plan {
    Grid g;
    int ty;
    int x_chunk;
    int nitems;
    int smem;
    int cur;
    TMaps maps[2];
    Params base;
    float *f[2][6];
    float *psi_e[2][6];
};

static int encode_map(EncodeTiledFn enc, CUtensorMap *m, const float *ptr, const Grid &g, int box_z, int box_y) {
    cuuint64_t dims[3] = {(cuuint64_t)g.nz, (cuuint64_t)g.ny, (cuuint64_t)g.nx};
    cuuint64_t strides[2] = {(cuuint64_t)g.sy * 4, (cuuint64_t)g.sx * 4};
    cuuint32_t box[3] = {(cuuint32_t)box_z, (cuuint32_t)box_y, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(ptr), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? FDTD_OK : FDTD_ERR_CUDA;
}

template <int TY>
static int configure(fdtd_yee_plan *pl) {
    pl->smem = Layout<TY>::SMEM;
    cudaError_t e = cudaFuncSetAttribute(k_yee_fused<TY>, cudaFuncAttributeMaxDynamicSharedMemorySize, pl->smem);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return FDTD_ERR_CUDA;
    }
    return FDTD_OK;
}

template <int TY>
static int launch(const fdtd_yee_plan *pl, const TMaps &m, const Params &p, cudaStream_t st) {
    k_yee_fused<TY><<<pl->nitems, TY * 32, pl->smem, st>>>(m, p);
    return check_launch();
}

static bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

extern "C" {

int fdtd_yee_plan_create(fdtd_yee_plan **out, const fdtd_grid *gp, const fdtd_yee_state *s, const fdtd_cpml *c,
                         const fdtd_sources *src, const fdtd_tile *tile, int32_t *status_dev, int32_t cur) {
    if (!out || !s || !status_dev) return FDTD_ERR_ARG;
    *out = nullptr;
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (g.nx < 2 || g.ny < 2 || g.nz < 2) return FDTD_ERR_SHAPE;
    if (g.nx > (1 << 30) || g.ny > (1 << 30) || g.nz > (1 << 30)) return FDTD_ERR_SHAPE;
    if ((g.sx & 3) || (g.sy & 3)) return FDTD_ERR_ALIGN;
    if (cur != 0 && cur != 1) return FDTD_ERR_ARG;
    for (int b = 0; b < 2; b++)
        for (int q = 0; q < 6; q++) {
            if (!s->f[b][q]) return FDTD_ERR_ARG;
            if (!aligned16(s->f[b][q])) return FDTD_ERR_ALIGN;
        }
    for (int q = 0; q < 3; q++) {
        if (!s->ce[q]) return FDTD_ERR_ARG;
        if (!aligned16(s->ce[q])) return FDTD_ERR_ALIGN;
    }
    int ty = tile && tile->tile_y ? tile->tile_y : 8;
    if (ty != 4 && ty != 8 && ty != 16) return FDTD_ERR_UNSUPPORTED;
    int xch = tile && tile->x_chunk ? tile->x_chunk : 64;
    if (xch < 1) return FDTD_ERR_ARG;

    fdtd_yee_plan *pl = new fdtd_yee_plan();
    pl->g = g;
    pl->ty = ty;
    pl->x_chunk = (int)std::min<int64_t>(xch, g.nx);
    pl->cur = cur;
    Params &p = pl->base;
    p = Params{};
    p.nx = g.nx; p.ny = g.ny; p.nz = g.nz; p.sx = g.sx; p.sy = g.sy;
    p.ntz = (int)((g.nz + TZ - 1) / TZ);
    p.nty = (int)((g.ny + ty - 1) / ty);
    p.x_chunk = pl->x_chunk;
    const int64_t nxc = (g.nx + pl->x_chunk - 1) / pl->x_chunk;
    const int64_t nitems = (int64_t)p.ntz * p.nty * nxc;
    if (nitems > 0x7fffffff) { delete pl; return FDTD_ERR_SHAPE; }
    pl->nitems = (int)nitems;
    p.status = status_dev;

    const bool pml = c && (c->npml[0] > 0 || c->npml[1] > 0 || c->npml[2] > 0);
    if (pml) {
        const int64_t n[3] = {g.nx, g.ny, g.nz};
        p.faces = c->faces;
        for (int a = 0; a < 3; a++) {
            p.P[a] = c->npml[a];
            if (c->npml[a] < 0) { delete pl; return FDTD_ERR_ARG; }
            if (c->npml[a] == 0) continue;
            if (n[a] < 2 * (int64_t)c->npml[a] + 2) { delete pl; return FDTD_ERR_SHAPE; }
            if (!all_nonnull(c->b_e[a], c->a_e[a], c->km1_e[a], c->b_h[a], c->a_h[a], c->km1_h[a])) {
                delete pl; return FDTD_ERR_ARG;
            }
            for (int b = 0; b < 2; b++)
                if (!s->psi_e[b][2 * a] || !s->psi_e[b][2 * a + 1]) { delete pl; return FDTD_ERR_ARG; }
            if (!s->psi_h[2 * a] || !s->psi_h[2 * a + 1]) { delete pl; return FDTD_ERR_ARG; }
            p.tb_e[a] = c->b_e[a]; p.ta_e[a] = c->a_e[a]; p.tk_e[a] = c->km1_e[a];
            p.tb_h[a] = c->b_h[a]; p.ta_h[a] = c->a_h[a]; p.tk_h[a] = c->km1_h[a];
        }
        for (int q = 0; q < 6; q++) p.psi_h[q] = s->psi_h[q];
    }
    if (src && src->nsrc > 0) {
        if (!all_nonnull(src->ijk, src->comp, src->amp) || src->namp < 0) { delete pl; return FDTD_ERR_ARG; }
        p.nsrc = src->nsrc; p.src_ijk = src->ijk; p.src_comp = src->comp; p.src_amp = src->amp; p.namp = src->namp;
        // capacity: sources per work item's extended region
        int32_t *hijk = new int32_t[3 * (size_t)src->nsrc];
        if (cudaMemcpy(hijk, src->ijk, sizeof(int32_t) * 3 * src->nsrc, cudaMemcpyDeviceToHost) != cudaSuccess) {
            delete[] hijk; delete pl; return FDTD_ERR_CUDA;
        }
        for (int a = 0; a < src->nsrc; a++) {
            int cnt = 0;
            for (int b = 0; b < src->nsrc; b++) {
                // conservative: same tile neighbourhood (one tile + halo in y/z, one chunk + 1 in x)
                if (std::abs(hijk[3 * a + 1] / ty - hijk[3 * b + 1] / ty) <= 1 &&
                    std::abs(hijk[3 * a + 2] / TZ - hijk[3 * b + 2] / TZ) <= 1 &&
                    std::abs(hijk[3 * a] / pl->x_chunk - hijk[3 * b] / pl->x_chunk) <= 1)
                    cnt++;
            }
            if (cnt > MAX_LOCAL_SRC) { delete[] hijk; delete pl; return FDTD_ERR_CAPACITY; }
            if (hijk[3 * a] < 0 || hijk[3 * a] >= g.nx || hijk[3 * a + 1] < 0 || hijk[3 * a + 1] >= g.ny ||
                hijk[3 * a + 2] < 0 || hijk[3 * a + 2] >= g.nz) {
                delete[] hijk; delete pl; return FDTD_ERR_ARG;
            }
        }
        delete[] hijk;
    }

    EncodeTiledFn enc = get_encode_fn();
    if (!enc) { delete pl; return FDTD_ERR_CUDA; }
    for (int b = 0; b < 2; b++) {
        for (int q = 0; q < 6; q++) {
            pl->f[b][q] = s->f[b][q];
            pl->psi_e[b][q] = s->psi_e[b][q];
        }
        int st = FDTD_OK;
        for (int q = 0; q < 3 && st == FDTD_OK; q++) {
            st = encode_map(enc, &pl->maps[b].h[q], s->f[b][3 + q], g, HC, ty + 2);
            if (st == FDTD_OK) st = encode_map(enc, &pl->maps[b].e[q], s->f[b][q], g, EC, ty + 1);
            if (st == FDTD_OK) st = encode_map(enc, &pl->maps[b].ce[q], s->ce[q], g, EC, ty + 1);
        }
        if (st != FDTD_OK) { delete pl; return st; }
    }
    int st = ty == 4 ? configure<4>(pl) : ty == 8 ? configure<8>(pl) : configure<16>(pl);
    if (st != FDTD_OK) { delete pl; return st; }
    *out = pl;
    return FDTD_OK;
}

int fdtd_yee_plan_run(fdtd_yee_plan *pl, int64_t t0, int64_t nsteps, void *stream) {
    if (!pl || nsteps < 0) return FDTD_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    for (int64_t n = 0; n < nsteps; n++) {
        const int in = pl->cur, outb = 1 - pl->cur;
        Params p = pl->base;
        for (int q = 0; q < 6; q++) {
            p.out[q] = pl->f[outb][q];
            p.psi_e_in[q] = pl->psi_e[in][q];
            p.psi_e_out[q] = pl->psi_e[outb][q];
        }
        p.t = t0 + n;
        int r = pl->ty == 4 ? launch<4>(pl, pl->maps[in], p, st)
                            : pl->ty == 8 ? launch<8>(pl, pl->maps[in], p, st) : launch<16>(pl, pl->maps[in], p, st);
        if (r != FDTD_OK) return r;
        pl->cur = outb;
    }
    return FDTD_OK;
}

int fdtd_yee_plan_current(const fdtd_yee_plan *pl) { return pl ? pl->cur : -1; }

int fdtd_yee_plan_set_current(fdtd_yee_plan *pl, int32_t cur) {
    if (!pl || (cur != 0 && cur != 1)) return FDTD_ERR_ARG;
    pl->cur = cur;
    return FDTD_OK;
}

int fdtd_yee_plan_destroy(fdtd_yee_plan *pl) {
    delete pl;
    return FDTD_OK;
}

}  // extern "C"
