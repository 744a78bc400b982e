// Fused Yee time step: host side (plans, tensor maps, launches) and the
// z-band kernels.  The fused kernel itself is in yee_fused.cuh.
#include <cuda.h>

#include <algorithm>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "yee_fused.cuh"

namespace fdtd {
namespace fused {

// Single-grid band kernels: a warp per (i, j) row (grid (ceil(ny/4), nx),
// 4 warps a block), lanes over the row's band cells -- no index division.
__global__ void __launch_bounds__(128) k_zband_e(const __grid_constant__ Params p) {
    const int64_t j = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5), i = blockIdx.y;
    if (j >= p.ny) return;
    const int nk = zband_e_row(p);
    for (int kb = threadIdx.x & 31; kb < nk; kb += 32) zband_e_at(p, p.t, i, j, kb);
}

__global__ void __launch_bounds__(128) k_zband_h(const __grid_constant__ Params p) {
    const int64_t j = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5), i = blockIdx.y;
    if (j >= p.ny) return;
    const int nk = zband_h_row(p);
    for (int kb = threadIdx.x & 31; kb < nk; kb += 32) zband_h_at(p, i, j, kb);
}

// Batched band kernels: the band cells of all grids numbered consecutively
// (off[s] = first cell of grid s); one launch each for E and H per step.
__global__ void __launch_bounds__(128) k_zband_e_batch(const __grid_constant__ BandBatch d) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.off[d.nsims]) return;
    const int s = band_sim(d, t);
    zband_e_cell(d.params[2 * s + d.cur], d.t, t - d.off[s]);
}

__global__ void __launch_bounds__(128) k_zband_h_batch(const __grid_constant__ BandBatch d) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.off[d.nsims]) return;
    const int s = band_sim(d, t);
    zband_h_cell(d.params[2 * s + d.cur], t - d.off[s]);
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

struct KernelEntry {
    int ty, ns, threads, stage, enew, psiring;
    FusedKernel fn[3];        // single grid, EXT = 0, 1, 2
    FusedKernel fn_batch[2];  // batched, EXT = 0, 1 (batched plans take no plane wave)
};

template <int TY, int NS>
static KernelEntry entry() {
    KernelEntry e{TY, NS, Layout<TY, NS>::THREADS, Layout<TY, NS>::STAGE, Layout<TY, NS>::ENEW,
                  Layout<TY, NS>::PSIRING, {}, {}};
    single_kernels(TY, NS, e.fn);
    batch_kernels(TY, NS, e.fn_batch);
    return e;
}

// Tile heights and pipeline depths compiled in (the autotuner picks among them).
static const KernelEntry *find_kernel(int ty, int ns) {
#define FDTD_ENTRY(TY, NS) entry<TY, NS>(),
    static const KernelEntry table[] = {FDTD_FUSED_TILES(FDTD_ENTRY)};
#undef FDTD_ENTRY
    for (const KernelEntry &e : table)
        if (e.ty == ty && e.ns == ns) return &e;
    return nullptr;
}

struct fdtd_yee_plan {
    Grid g;
    const KernelEntry *k;
    FusedKernel fn;  // the kernel variant launched (with or without the Drude / TFSF code)
    int smem;
    int x_chunk;
    int64_t nitems;
    int nblocks;
    int cur;
    TMaps maps[2];
    Params base;
    float *f[2][6];
    float *psi_e[2][6];
    float *dj[2][3];  // Drude J buffers
    bool has_tfsf;
    fdtd_tfsf tfsf;   // plane-wave source (1-D grid arrays owned by the caller)
};

// 3-D FP32 tensor map: dims (n0 fastest, n1, n2), element strides s1, s2,
// box (b0, b1, 1); out-of-range elements read as zero.
static int encode_map3(EncodeTiledFn enc, CUtensorMap *m, const float *ptr, int64_t n0, int64_t n1, int64_t n2,
                       int64_t s1, int64_t s2, int b0, int b1, CUtensorMapL2promotion promo) {
    cuuint64_t dims[3] = {(cuuint64_t)n0, (cuuint64_t)n1, (cuuint64_t)n2};
    cuuint64_t strides[2] = {(cuuint64_t)s1 * 4, (cuuint64_t)s2 * 4};
    cuuint32_t box[3] = {(cuuint32_t)b0, (cuuint32_t)b1, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(ptr), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, promo,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? FDTD_OK : FDTD_ERR_CUDA;
}

static int encode_map(EncodeTiledFn enc, CUtensorMap *m, const float *ptr, const Grid &g, int box_z, int box_y,
                      CUtensorMapL2promotion promo) {
    return encode_map3(enc, m, ptr, g.nz, g.ny, g.nx, g.sy, g.sx, box_z, box_y, promo);
}

static bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

extern "C" {

// refine: let the default chunk follow the launch-length model below (a plan
// of its own); the batched plan pools every grid's items over one launch and
// keeps the provisional chunk
static int yee_plan_create(fdtd_yee_plan **out, const fdtd_grid *gp, const fdtd_yee_state *s, const fdtd_cpml *c,
                           const fdtd_sources *src, const fdtd_tile *tile, int32_t *status_dev, int32_t cur,
                           void *stream, bool refine) {
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
    const int ty = tile && tile->tile_y ? tile->tile_y : 8;
    const int ns = tile && tile->stages ? tile->stages : 3;
    const KernelEntry *ke = find_kernel(ty, ns);
    if (!ke) return FDTD_ERR_UNSUPPORTED;
    int xch = tile && tile->x_chunk ? tile->x_chunk : 128;
    if (xch < 1) return FDTD_ERR_ARG;
    if (!(tile && tile->x_chunk)) {
        // provisional default chunk: at least ~3 work items per SM so small
        // grids fill the GPU (shorter chunks add pipeline fill and halo planes
        // per item); refined below once the resident CTAs are known
        int dev = 0, nsm = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && nsm > 0) {
            const int64_t tiles = ((g.nz + TZ - 1) / TZ) * ((g.ny + ty - 1) / ty);
            while (xch > 8 && tiles * ((g.nx + xch - 1) / xch) < 3 * (int64_t)nsm) xch /= 2;
        }
    }

    fdtd_yee_plan *pl = new fdtd_yee_plan();
    pl->g = g;
    pl->k = ke;
    pl->x_chunk = (int)std::min<int64_t>(xch, g.nx);
    pl->cur = cur;
    Params &p = pl->base;
    p = Params{};
    p.nx = g.nx; p.ny = g.ny; p.nz = g.nz; p.sx = g.sx; p.sy = g.sy;
    p.ntz = (int)((g.nz + TZ - 1) / TZ);
    p.nty = (int)((g.ny + ty - 1) / ty);
    p.nxc = (int)((g.nx + pl->x_chunk - 1) / pl->x_chunk);
    p.x_chunk = pl->x_chunk;
    pl->nitems = (int64_t)p.ntz * p.nty * p.nxc;
    p.status = status_dev;
    p.wait_ns = 0;         // the 1 s limit
    p.test_withhold = -1;  // every copy issued

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
    for (int q = 0; q < 3; q++) p.in_ce[q] = s->ce[q];
    if (s->drude) {
        const int st = validate_drude(g, s->drude);
        if (st != FDTD_OK) { delete pl; return st; }
        const fdtd_drude &d = *s->drude;
        p.drude = 1;
        const int64_t box[6] = {d.i0, d.j0, d.k0, d.ni, d.nj, d.nk};
        for (int q = 0; q < 6; q++) p.dbox[q] = box[q];
        for (int q = 0; q < 3; q++) {
            if (!d.j2[q]) { delete pl; return FDTD_ERR_ARG; }
            pl->dj[0][q] = d.j[q];
            pl->dj[1][q] = d.j2[q];
            p.dcja[q] = d.cja[q];
            p.dcjb[q] = d.cjb[q];
        }
    }
    if (s->tfsf) {
        const int st = validate_tfsf(g, s->tfsf);
        if (st != FDTD_OK) { delete pl; return st; }
        const fdtd_tfsf &t = *s->tfsf;
        // the box's face cells (p1-1 .. p2) stay clear of the CPML slabs and of the
        // z band, which the band kernels finish after the fused kernel
        const int64_t n3[3] = {g.nx, g.ny, g.nz};
        for (int a = 0; a < 3; a++) {
            const int64_t P = c ? c->npml[a] : 0;
            if (P > 0 && (t.p1[a] - 1 < P + 2 || t.p2[a] + 1 > n3[a] - P - 2)) { delete pl; return FDTD_ERR_UNSUPPORTED; }
        }
        pl->has_tfsf = true;
        pl->tfsf = t;
        p.tfsf = 1;
        p.tfaces = t.faces;
        p.taxis = t.axis;
        for (int a = 0; a < 3; a++) {
            p.tp1[a] = (int32_t)t.p1[a];
            p.tp2[a] = (int32_t)t.p2[a];
        }
        tfsf_table(&t, p.tcoef, p.tix, &p.tvo);
        p.te1d = t.e1d;
        p.th1d = t.h1d;
    }
    // the z slab (when a z face has CPML) is finished by the band kernels
    p.zfix = (p.P[2] > 0 && ((p.faces >> 4) & 3)) ? 1 : 0;
    if (src && src->nsrc > 0) {
        if (!all_nonnull(src->ijk, src->comp, src->amp) || src->namp < 0) { delete pl; return FDTD_ERR_ARG; }
        p.nsrc = src->nsrc; p.src_ijk = src->ijk; p.src_comp = src->comp; p.src_amp = src->amp; p.namp = src->namp;
        // capacity: sources per work item's extended region (checked on the host)
        // read on the caller's stream (after any pending write of the list), then wait for it
        int32_t *hijk = new int32_t[3 * (size_t)src->nsrc];
        cudaError_t ce = cudaMemcpyAsync(hijk, src->ijk, sizeof(int32_t) * 3 * src->nsrc, cudaMemcpyDeviceToHost,
                                         as_stream(stream));
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(as_stream(stream));
        if (ce != cudaSuccess) {
            set_cuda_error(ce);
            delete[] hijk; delete pl; return FDTD_ERR_CUDA;
        }
        // sources on E z-slab nodes: applied by the E band kernel
        if (p.zfix) {
            const int64_t P2 = p.P[2];
            const int f2 = (p.faces >> 4) & 1, b2 = (p.faces >> 5) & 1;
            for (int a = 0; a < src->nsrc; a++) {
                const int64_t sk = hijk[3 * a + 2];
                const bool node = (f2 && sk >= 1 && sk <= P2) || (b2 && sk >= g.nz - P2 - 1 && sk <= g.nz - 2);
                if (!node) continue;
                if (p.nbsrc == MAX_BAND_SRC) {  // too many for the list: the band kernel scans all sources
                    p.nbsrc = -1;
                    break;
                }
                p.bsrc[p.nbsrc++] = a;
            }
        }
        // sources per work item, counted with the kernel's own membership test
        // (x in [i_start, x1), y in [j0-1, j0+TY), z in [k0-1, k0+TZ)); a source
        // lies in at most two chunks/tiles per axis
        std::unordered_map<int64_t, int> per_item;
        const int64_t xc = pl->x_chunk;
        const int64_t ntz = (g.nz + TZ - 1) / TZ, nty = (g.ny + ty - 1) / ty;
        for (int a = 0; a < src->nsrc; a++) {
            const int64_t si = hijk[3 * a], sj = hijk[3 * a + 1], sk = hijk[3 * a + 2];
            if (si < 0 || si >= g.nx || sj < 0 || sj >= g.ny || sk < 0 || sk >= g.nz || sk >= (int64_t(1) << 28)) {
                delete[] hijk; delete pl; return FDTD_ERR_ARG;
            }
            for (int64_t xi = si / xc; xi <= (si + 1) / xc; xi++) {
                const int64_t x0 = xi * xc, x1 = std::min(x0 + xc, (int64_t)g.nx);
                const int64_t is = x0 > 0 ? x0 - 1 : 0;
                if (x0 >= g.nx || si < is || si >= x1) continue;
                for (int64_t yi = sj / ty; yi <= (sj + 1) / ty && yi < nty; yi++) {
                    const int64_t j0 = yi * ty;
                    if (sj < j0 - 1 || sj >= j0 + ty) continue;
                    for (int64_t zi = sk / TZ; zi <= (sk + 1) / TZ && zi < ntz; zi++) {
                        const int64_t k0 = zi * TZ;
                        if (sk < k0 - 1 || sk >= k0 + TZ) continue;
                        if (++per_item[(xi * nty + yi) * ntz + zi] > MAX_LOCAL_SRC) {
                            delete[] hijk; delete pl; return FDTD_ERR_CAPACITY;
                        }
                    }
                }
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
        const int pm = tile ? tile->l2_promotion : 0;
        const CUtensorMapL2promotion promo = pm == 1   ? CU_TENSOR_MAP_L2_PROMOTION_NONE
                                             : pm == 2 ? CU_TENSOR_MAP_L2_PROMOTION_L2_64B
                                             : pm == 3 ? CU_TENSOR_MAP_L2_PROMOTION_L2_128B
                                                       : CU_TENSOR_MAP_L2_PROMOTION_L2_256B;
        int st = FDTD_OK;
        for (int q = 0; q < 3 && st == FDTD_OK; q++) {
            st = encode_map(enc, &pl->maps[b].h[q], s->f[b][3 + q], g, HC, ty + 2, promo);
            if (st == FDTD_OK) st = encode_map(enc, &pl->maps[b].e[q], s->f[b][q], g, EC, ty + 1, promo);
            if (st == FDTD_OK) st = encode_map(enc, &pl->maps[b].ce[q], s->ce[q], g, EC, ty + 1, promo);
        }
        if (st != FDTD_OK) { delete pl; return st; }
    }
    p.stage_bytes = ke->stage;
    // x/y psi slabs through TMA: rows of nz floats must be 16-byte multiples
    {
        const int P0 = p.P[0], P1 = p.P[1];
        bool ok = (P0 > 0 || P1 > 0) && g.nz % 4 == 0;
        for (int q = 0; q < 2 && ok; q++) {
            if (P0 > 0) ok = aligned16(s->psi_e[0][q]) && aligned16(s->psi_e[1][q]) && aligned16(s->psi_h[q]);
            if (ok && P1 > 0)
                ok = aligned16(s->psi_e[0][2 + q]) && aligned16(s->psi_e[1][2 + q]) && aligned16(s->psi_h[2 + q]);
        }
        int st = FDTD_OK;
        const int ec = EC, by = ty + 1;
        for (int b = 0; b < 2 && ok && st == FDTD_OK; b++)
            for (int q = 0; q < 2 && st == FDTD_OK; q++) {
                if (P0 > 0) {
                    st = encode_map3(enc, &pl->maps[b].xpe[q], s->psi_e[b][q], g.nz, g.ny, 2 * P0, g.nz,
                                     g.ny * g.nz, ec, by, CU_TENSOR_MAP_L2_PROMOTION_L2_128B);
                    if (st == FDTD_OK)
                        st = encode_map3(enc, &pl->maps[b].xph[q], s->psi_h[q], g.nz, g.ny, 2 * P0, g.nz,
                                         g.ny * g.nz, ec, by, CU_TENSOR_MAP_L2_PROMOTION_L2_128B);
                }
                if (P1 > 0 && st == FDTD_OK) {
                    st = encode_map3(enc, &pl->maps[b].ype[q], s->psi_e[b][2 + q], g.nz, 2 * P1, g.nx, g.nz,
                                     2 * P1 * g.nz, ec, by, CU_TENSOR_MAP_L2_PROMOTION_L2_128B);
                    if (st == FDTD_OK)
                        st = encode_map3(enc, &pl->maps[b].yph[q], s->psi_h[2 + q], g.nz, 2 * P1, g.nx, g.nz,
                                         2 * P1 * g.nz, ec, by, CU_TENSOR_MAP_L2_PROMOTION_L2_128B);
                }
            }
        if (st != FDTD_OK) { delete pl; return st; }
        p.xypsi = ok ? 1 : 0;
    }
    const int tab_bytes = 6 * 2 * (p.P[0] + p.P[1] + p.P[2]) * 4;
    pl->smem = ns * p.stage_bytes + ke->enew + 128 /*barriers*/ + ke->psiring + tab_bytes + 128 /*align slack*/;
    pl->fn = ke->fn[p.tfsf ? 2 : (p.drude ? 1 : 0)];
    int dev = 0, nsm = 0, occ = 0, optin = 0;
    cudaFuncAttributes fa;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, (const void *)pl->fn);
    if (e != cudaSuccess) { set_cuda_error(e); delete pl; return FDTD_ERR_CUDA; }
    const int max_dyn = optin - (int)fa.sharedSizeBytes;
    if (pl->smem > max_dyn) { delete pl; return FDTD_ERR_UNSUPPORTED; }
    // the attribute is an upper bound; every plan of this kernel fits under it
    e = cudaFuncSetAttribute((const void *)pl->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void *)pl->fn, ke->threads, pl->smem);
    if (e != cudaSuccess) { set_cuda_error(e); delete pl; return FDTD_ERR_CUDA; }
    if (occ < 1) { delete pl; return FDTD_ERR_UNSUPPORTED; }
    if (tile && tile->ctas_per_sm > 0) occ = std::min(occ, (int)tile->ctas_per_sm);
    pl->nblocks = (int)std::min<int64_t>(pl->nitems, (int64_t)nsm * occ);
    if (refine && !pml && !(tile && tile->x_chunk)) {
        // the default chunk of a grid without CPML (items of equal cost), now
        // that the resident CTAs are known: CTA b takes items b, b + CTAs, ...,
        // so a launch lasts ceil(items / CTAs) items of (chunk + 3) plane steps
        // (the pipeline fill and the halo plane of an item); of 128, 96, 64,
        // 48, 32, 24, 16, 12 and 8 planes the chunk with the shortest such
        // launch, the longer one on a tie.  A chunk other than the provisional
        // one re-creates the plan with it (the source capacity per item is
        // checked again).  With CPML the x-slab items cost more and the
        // provisional chunk stays (at 256x256x128 with a 12-cell CPML the
        // model's 64 planes ran the step 7 % slower than 32).
        const int64_t tiles = (int64_t)p.ntz * p.nty, ctas = (int64_t)nsm * occ;
        int best = pl->x_chunk;
        int64_t best_t = -1;
        for (int cand : {128, 96, 64, 48, 32, 24, 16, 12, 8}) {
            const int64_t cc = std::min<int64_t>(cand, g.nx), items = tiles * ((g.nx + cc - 1) / cc);
            const int64_t rounds = (items + std::min(items, ctas) - 1) / std::min(items, ctas);
            const int64_t t = rounds * (cc + 3);
            if (best_t < 0 || t < best_t) {
                best_t = t;
                best = (int)cc;
            }
        }
        if (best != pl->x_chunk) {
            fdtd_tile t2 = tile ? *tile : fdtd_tile{0, 0, 0, 0, 0};
            t2.x_chunk = best;
            fdtd_yee_plan *alt = nullptr;
            if (yee_plan_create(&alt, gp, s, c, src, &t2, status_dev, cur, stream, false) == FDTD_OK) {
                delete pl;
                *out = alt;
                return FDTD_OK;
            }
        }
    }
    *out = pl;
    return FDTD_OK;
}

int fdtd_yee_plan_create(fdtd_yee_plan **out, const fdtd_grid *gp, const fdtd_yee_state *s, const fdtd_cpml *c,
                         const fdtd_sources *src, const fdtd_tile *tile, int32_t *status_dev, int32_t cur,
                         void *stream) {
    return yee_plan_create(out, gp, s, c, src, tile, status_dev, cur, stream, true);
}

int fdtd_yee_plan_run(fdtd_yee_plan *pl, int64_t t0, int64_t nsteps, void *stream) {
    if (!pl || nsteps < 0) return FDTD_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    // TFSF: the 1-D E step of each step runs before its fused kernel (whose E
    // faces read the 1-D H of the previous step, H faces the new 1-D E), the
    // 1-D H step after it
    if (pl->has_tfsf && nsteps > 0) {
        if (t0 + nsteps - 1 >= pl->tfsf.namp || t0 < 0) return FDTD_ERR_ARG;
        FDTD_TRY(tfsf_launch_1d(&pl->tfsf, 0, t0, st));
    }
    for (int64_t n = 0; n < nsteps; n++) {
        NvtxRange nvtx_range("fdtd_yee_step");
        const int in = pl->cur, outb = 1 - pl->cur;
        Params p = pl->base;
        for (int q = 0; q < 6; q++) {
            p.out[q] = pl->f[outb][q];
            p.psi_e_in[q] = pl->psi_e[in][q];
            p.psi_e_out[q] = pl->psi_e[outb][q];
        }
        for (int q = 0; q < 3; q++) {
            p.dj_in[q] = pl->dj[in][q];
            p.dj_out[q] = pl->dj[outb][q];
        }
        p.t = t0 + n;
        BatchDesc bd{};
        pl->fn<<<pl->nblocks, pl->k->threads, pl->smem, st>>>(pl->maps[in], p, bd);
        if (p.zfix) {
            for (int q = 0; q < 6; q++) p.in[q] = pl->f[in][q];
            const dim3 rows((unsigned)((p.ny + 3) / 4), (unsigned)p.nx);
            k_zband_e<<<rows, 128, 0, st>>>(p);
            k_zband_h<<<rows, 128, 0, st>>>(p);
        }
        FDTD_TRY(check_launch());
        if (pl->has_tfsf) FDTD_TRY(tfsf_launch_1d(&pl->tfsf, n + 1 < nsteps ? 2 : 1, t0 + n + 1, st));
        pl->cur = outb;
    }
    return FDTD_OK;
}

int fdtd_yee_plan_current(const fdtd_yee_plan *pl) { return pl ? pl->cur : -1; }

int fdtd_yee_plan_test_timeout(fdtd_yee_plan *pl, int64_t wait_ns, int32_t withhold_plane) {
    if (!pl || wait_ns < 0 || withhold_plane < -1) return FDTD_ERR_ARG;
    pl->base.wait_ns = (uint64_t)wait_ns;
    pl->base.test_withhold = withhold_plane;
    return FDTD_OK;
}

int fdtd_yee_plan_set_current(fdtd_yee_plan *pl, int32_t cur) {
    if (!pl || (cur != 0 && cur != 1)) return FDTD_ERR_ARG;
    pl->cur = cur;
    return FDTD_OK;
}

int fdtd_yee_plan_info(const fdtd_yee_plan *pl, int32_t *info, int32_t n) {
    if (!pl || !info || n < 6) return FDTD_ERR_ARG;
    info[0] = pl->k->ty;
    info[1] = pl->k->ns;
    info[2] = pl->x_chunk;
    info[3] = pl->nblocks;
    info[4] = pl->k->threads;
    info[5] = pl->smem;
    if (n >= 8) {
        info[6] = pl->base.zfix;                  // 1: z slab on the band kernels
        info[7] = (pl->base.zfix ? 3 : 1) + (pl->has_tfsf ? 1 : 0);  // kernel launches per step
    }
    return FDTD_OK;
}

int fdtd_yee_plan_destroy(fdtd_yee_plan *pl) {
    delete pl;
    return FDTD_OK;
}

int fdtd_yee_step_f32(const fdtd_grid *g, const fdtd_yee_state *st, const fdtd_cpml *c, const fdtd_sources *src,
                      int32_t *status_dev, int32_t cur, int64_t t0, int64_t nsteps, int32_t *cur_out,
                      void *stream) {
    if (nsteps < 0) return FDTD_ERR_ARG;
    fdtd_yee_plan *pl = nullptr;
    FDTD_TRY(fdtd_yee_plan_create(&pl, g, st, c, src, nullptr, status_dev, cur, stream));
    const int r = fdtd_yee_plan_run(pl, t0, nsteps, stream);
    if (cur_out) *cur_out = pl->cur;
    fdtd_yee_plan_destroy(pl);  // host-side only: the launches hold copies of everything they use
    return r;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batched plan: many grids, one launch per step.  Every grid gets an ordinary
// plan (validation, tensor maps, parameters); their Params/TMaps and the item
// offsets live in a caller-provided device workspace.
// ---------------------------------------------------------------------------
struct fdtd_batch_plan {
    int32_t nsims;
    const KernelEntry *k;
    FusedKernel fn;  // batched variant launched (with the Drude code when a grid has a Drude box)
    int smem;
    int nblocks;
    int cur;
    int64_t nitems;
    int stage_bytes;
    TMaps *d_maps;
    Params *d_params;
    int64_t *d_off;        // work-item offsets of the fused kernel
    int64_t *d_band_e;     // band cell offsets (E, H) of the band kernels
    int64_t *d_band_h;
    int64_t band_e, band_h;  // band cells in all grids
    int32_t *d_queue;        // work queue of the fused kernel (2 counters)
};

static size_t batch_ws_layout(int32_t nsims, size_t *off_params, size_t *off_items) {
    size_t o = 0;
    o += (size_t)2 * nsims * sizeof(TMaps);
    o = (o + 63) / 64 * 64;
    *off_params = o;
    o += (size_t)2 * nsims * sizeof(Params);
    o = (o + 63) / 64 * 64;
    *off_items = o;  // work-item offsets, then E and H band cell offsets, then the queue
    o += (size_t)3 * (nsims + 1) * sizeof(int64_t);
    o += 64;
    return o;
}

extern "C" {

size_t fdtd_batch_workspace_bytes(int32_t nsims) {
    size_t a, b;
    return nsims > 0 ? batch_ws_layout(nsims, &a, &b) : 0;
}

int fdtd_batch_plan_create(fdtd_batch_plan **out, int32_t nsims, const fdtd_grid *grids, const fdtd_yee_state *states,
                           const fdtd_cpml *cpmls, const fdtd_sources *srcs, const fdtd_tile *tile,
                           int32_t *status_dev, void *workspace, size_t workspace_bytes, int32_t cur,
                           void *stream) {
    if (!out || nsims <= 0 || !grids || !states || !status_dev || !workspace) return FDTD_ERR_ARG;
    *out = nullptr;
    if ((reinterpret_cast<uintptr_t>(workspace) & 63) != 0) return FDTD_ERR_ALIGN;
    size_t off_p, off_i;
    const size_t need = batch_ws_layout(nsims, &off_p, &off_i);
    if (workspace_bytes < need) return FDTD_ERR_CAPACITY;
    std::vector<TMaps> maps((size_t)2 * nsims);
    std::vector<Params> params((size_t)2 * nsims);
    std::vector<int64_t> off((size_t)3 * (nsims + 1), 0);
    int64_t *boff_e = off.data() + (nsims + 1), *boff_h = off.data() + 2 * (nsims + 1);
    const KernelEntry *ke = nullptr;
    int stage_bytes = 0, tab_bytes = 0;
    bool any_drude = false;
    // grids with the longest items (x planes per chunk, then tile rows) come first
    std::vector<int32_t> order((size_t)nsims);
    for (int32_t s = 0; s < nsims; s++) order[s] = s;
    auto item_len = [&](int32_t s) {
        const int64_t xc = tile && tile->x_chunk ? tile->x_chunk : 128;
        return std::min<int64_t>(xc, grids[s].nx) * 65536 + std::min<int64_t>(grids[s].ny, 65535);
    };
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return item_len(a) > item_len(b); });
    for (int32_t s = 0; s < nsims; s++)
        if (states[s].tfsf) return FDTD_ERR_UNSUPPORTED;  // plane waves: single-grid plans only
    for (int32_t s = 0; s < nsims; s++) {
        const int32_t u = order[s];
        fdtd_yee_plan *pl = nullptr;
        const int st = yee_plan_create(&pl, &grids[u], &states[u], cpmls ? &cpmls[u] : nullptr,
                                       srcs ? &srcs[u] : nullptr, tile, status_dev, cur, stream, false);
        if (st != FDTD_OK) return st;
        ke = pl->k;
        stage_bytes = std::max(stage_bytes, pl->base.stage_bytes);
        any_drude = any_drude || pl->base.drude;
        tab_bytes = std::max(tab_bytes, 6 * 2 * (pl->base.P[0] + pl->base.P[1] + pl->base.P[2]) * 4);
        for (int b = 0; b < 2; b++) {
            Params p = pl->base;
            for (int q = 0; q < 6; q++) {
                p.out[q] = pl->f[1 - b][q];
                p.psi_e_in[q] = pl->psi_e[b][q];
                p.psi_e_out[q] = pl->psi_e[1 - b][q];
                p.in[q] = pl->f[b][q];
            }
            for (int q = 0; q < 3; q++) {
                p.dj_in[q] = pl->dj[b][q];
                p.dj_out[q] = pl->dj[1 - b][q];
            }
            params[2 * s + b] = p;
            maps[2 * s + b] = pl->maps[b];
        }
        off[s + 1] = off[s] + pl->nitems;
        boff_e[s + 1] = boff_e[s] + zband_e_cells(pl->base);
        boff_h[s + 1] = boff_h[s] + zband_h_cells(pl->base);
        fdtd_yee_plan_destroy(pl);
    }
    // fill the workspace on the caller's stream (ordered after that stream's
    // earlier launches that may still read it), then wait for the copies: the
    // host-side tables are freed on return
    unsigned char *ws = static_cast<unsigned char *>(workspace);
    cudaStream_t cs = as_stream(stream);
    cudaError_t e = cudaMemcpyAsync(ws, maps.data(), maps.size() * sizeof(TMaps), cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ws + off_p, params.data(), params.size() * sizeof(Params), cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ws + off_i, off.data(), off.size() * sizeof(int64_t), cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess) e = cudaMemsetAsync(ws + off_i + off.size() * sizeof(int64_t), 0, 64, cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    if (e != cudaSuccess) { set_cuda_error(e); return FDTD_ERR_CUDA; }

    fdtd_batch_plan *bp = new fdtd_batch_plan();
    bp->nsims = nsims;
    bp->k = ke;
    bp->stage_bytes = stage_bytes;
    bp->smem = ke->ns * stage_bytes + ke->enew + 128 + ke->psiring + tab_bytes + 128;
    bp->cur = cur;
    bp->nitems = off[nsims];
    bp->d_maps = reinterpret_cast<TMaps *>(ws);
    bp->d_params = reinterpret_cast<Params *>(ws + off_p);
    bp->d_off = reinterpret_cast<int64_t *>(ws + off_i);
    bp->d_band_e = bp->d_off + (nsims + 1);
    bp->d_band_h = bp->d_off + 2 * (nsims + 1);
    bp->band_e = boff_e[nsims];
    bp->band_h = boff_h[nsims];
    bp->d_queue = reinterpret_cast<int32_t *>(ws + off_i + off.size() * sizeof(int64_t));
    int dev = 0, nsm = 0, occ = 0, optin = 0;
    cudaFuncAttributes fa;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    bp->fn = ke->fn_batch[any_drude ? 1 : 0];
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, (const void *)bp->fn);
    if (e != cudaSuccess) { set_cuda_error(e); delete bp; return FDTD_ERR_CUDA; }
    const int max_dyn = optin - (int)fa.sharedSizeBytes;
    if (bp->smem > max_dyn) { delete bp; return FDTD_ERR_UNSUPPORTED; }
    e = cudaFuncSetAttribute((const void *)bp->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void *)bp->fn, ke->threads, bp->smem);
    if (e != cudaSuccess) { set_cuda_error(e); delete bp; return FDTD_ERR_CUDA; }
    if (occ < 1) { delete bp; return FDTD_ERR_UNSUPPORTED; }
    if (tile && tile->ctas_per_sm > 0) occ = std::min(occ, (int)tile->ctas_per_sm);
    bp->nblocks = (int)std::min<int64_t>(bp->nitems, (int64_t)nsm * occ);
    *out = bp;
    return FDTD_OK;
}

int fdtd_batch_plan_run(fdtd_batch_plan *bp, int64_t t0, int64_t nsteps, void *stream) {
    if (!bp || nsteps < 0) return FDTD_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    TMaps dummy_maps;
    memset(&dummy_maps, 0, sizeof(dummy_maps));
    Params dummy{};
    for (int64_t n = 0; n < nsteps; n++) {
        NvtxRange nvtx_range("fdtd_batch_step");
        BatchDesc bd{};
        bd.nsims = bp->nsims;
        bd.cur = bp->cur;
        bd.t = t0 + n;
        bd.params = bp->d_params;
        bd.maps = bp->d_maps;
        bd.item_off = bp->d_off;
        bd.stage_bytes = bp->stage_bytes;
        bd.queue = bp->d_queue;
        bp->fn<<<bp->nblocks, bp->k->threads, bp->smem, st>>>(dummy_maps, dummy, bd);
        if (bp->band_e > 0 || bp->band_h > 0) {
            BandBatch d{bp->nsims, bp->cur, t0 + n, bp->d_params, bp->d_band_e};
            if (bp->band_e > 0) k_zband_e_batch<<<(unsigned)((bp->band_e + 127) / 128), 128, 0, st>>>(d);
            d.off = bp->d_band_h;
            if (bp->band_h > 0) k_zband_h_batch<<<(unsigned)((bp->band_h + 127) / 128), 128, 0, st>>>(d);
        }
        FDTD_TRY(check_launch());
        bp->cur = 1 - bp->cur;
    }
    return FDTD_OK;
}

int fdtd_batch_plan_current(const fdtd_batch_plan *bp) { return bp ? bp->cur : -1; }

int fdtd_batch_plan_set_current(fdtd_batch_plan *bp, int32_t cur) {
    if (!bp || (cur != 0 && cur != 1)) return FDTD_ERR_ARG;
    bp->cur = cur;
    return FDTD_OK;
}

int fdtd_batch_plan_info(const fdtd_batch_plan *bp, int32_t *info, int32_t n) {
    if (!bp || !info || n < 6) return FDTD_ERR_ARG;
    info[0] = bp->k->ty;
    info[1] = bp->k->ns;
    info[2] = (int32_t)std::min<int64_t>(bp->nitems, 0x7fffffff);
    info[3] = bp->nblocks;
    info[4] = bp->k->threads;
    info[5] = bp->smem;
    return FDTD_OK;
}

int fdtd_batch_plan_destroy(fdtd_batch_plan *bp) {
    delete bp;
    return FDTD_OK;
}

int fdtd_batched_run_f32(int32_t nsims, const fdtd_grid *grids, const fdtd_yee_state *states,
                         const fdtd_cpml *cpmls, const fdtd_sources *srcs, int32_t *status_dev, void *workspace,
                         size_t workspace_bytes, int32_t cur, int64_t t0, int64_t nsteps, int32_t *cur_out,
                         void *stream) {
    if (nsteps < 0) return FDTD_ERR_ARG;
    fdtd_batch_plan *bp = nullptr;
    FDTD_TRY(fdtd_batch_plan_create(&bp, nsims, grids, states, cpmls, srcs, nullptr, status_dev, workspace,
                                    workspace_bytes, cur, stream));
    const int r = fdtd_batch_plan_run(bp, t0, nsteps, stream);
    if (cur_out) *cur_out = fdtd_batch_plan_current(bp);
    fdtd_batch_plan_destroy(bp);  // the launches read the caller's workspace, not the plan
    return r;
}

}  // extern "C"
