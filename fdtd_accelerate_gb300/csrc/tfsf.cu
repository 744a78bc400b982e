// Total-field/scattered-field plane wave at normal incidence
// (kuFDTD/v0.2.0/dim3/tfsf.py:14-244).
//
// A 1-D auxiliary grid carries the incident wave along the propagation axis:
//   E[1:-1] -= 0.5 (H[2:] - H[1:-1]);  both ends take the value their
//   neighbour had two E steps earlier;  E[3] = sin(w dt t)     (tfsf.py:26-38)
//   H[1:]   -= 0.5 (E[1:] - E[:-1])                              (tfsf.py:41-42)
// and every enabled face of the total-field box corrects the two tangential
// components of the field just updated by half the incident field:
//   E half: e1 += 0.5 (c * H1d[s]),  H half: h1 += 0.5 (c * E1d[s])
// with the slices of tfsf.py:140-186 and the coefficients c and 1-D slices s
// of tfsf.py:189-231 (1-D index = 3-D index along the axis - p1[axis] + 5).
// The products and sums are rounded in float32 one by one, as NumPy
// evaluates the reference's array expressions.
#include <cmath>
#include <cstring>

#include "common.cuh"

namespace fdtd {

// One (face, component) slice of a half step.
struct TfsfSlice {
    int32_t comp;          // component 0..2 of the updated field
    int32_t vary;          // 1 when the 1-D index follows the propagation axis
    int32_t lo[3], hi[3];  // cell ranges [lo, hi)
    int32_t idx;           // fixed 1-D index (vary = 0) or the offset added to the axis coordinate
    float coef;            // incident coefficient (float32)
};

struct TfsfHalf {
    int32_t n, axis;
    int64_t cells;         // largest slice
    TfsfSlice s[12];
};

// the incident table of tfsf.py:201-206: (ce1, ce2, ch1, ch2, sE1, sE2, sH1, sH2)
// with the 1-D slice ids 1..5 of tfsf.py:195-199
struct IncRow {
    int c[4];    // coefficient selectors: 0 = 0, +/-1 = +/-sin, +/-2 = +/-cos
    int sl[4];
};
static const IncRow kInc[6] = {
    {{-1, 2, 2, 1}, {1, 1, 2, 2}},    // Inc1
    {{1, -2, -2, -1}, {5, 5, 5, 5}},  // Inc2
    {{0, 1, 0, -2}, {4, 3, 3, 4}},    // Inc3
    {{0, -1, 0, 2}, {4, 3, 3, 4}},    // Inc4
    {{-2, 0, -1, 0}, {3, 4, 4, 3}},   // Inc5
    {{2, 0, 1, 0}, {3, 4, 4, 3}},     // Inc6
};
// face f (x front, x back, y front, y back, z front, z back) -> Inc row, per axis (tfsf.py:208-213)
static const int kFaceInc[3][6] = {{0, 1, 2, 3, 4, 5}, {4, 5, 0, 1, 2, 3}, {2, 3, 4, 5, 0, 1}};

int validate_tfsf(const Grid &g, const fdtd_tfsf *t) {
    if (!t) return FDTD_ERR_ARG;
    if (t->axis < 0 || t->axis > 2 || (t->faces & ~0x3F)) return FDTD_ERR_ARG;
    const int64_t n[3] = {g.nx, g.ny, g.nz};
    for (int a = 0; a < 3; a++)
        if (t->p1[a] < 1 || t->p2[a] > n[a] - 1 || t->p2[a] < t->p1[a] + 1) return FDTD_ERR_SHAPE;
    if (!all_nonnull(t->e1d, t->h1d, t->abc, t->amp) || t->namp < 1) return FDTD_ERR_ARG;
    if (n[0] > (1 << 30) || n[1] > (1 << 30) || n[2] > (1 << 30)) return FDTD_ERR_SHAPE;
    return FDTD_OK;
}

int64_t tfsf_n1d(const fdtd_tfsf *t) { return t->p2[t->axis] - t->p1[t->axis] + 11; }

// The slices of one half step (eh = 0: E faces, which read H1d; eh = 1: H
// faces, which read E1d), tfsf.py:140-231.
TfsfHalf tfsf_half(const fdtd_tfsf *t, int eh) {
    TfsfHalf h{};
    h.axis = t->axis;
    const int32_t i1 = (int32_t)t->p1[0], j1 = (int32_t)t->p1[1], k1 = (int32_t)t->p1[2];
    const int32_t i2 = (int32_t)t->p2[0], j2 = (int32_t)t->p2[1], k2 = (int32_t)t->p2[2];
    const int32_t i2d = (int32_t)(t->p2[t->axis] - t->p1[t->axis]) + 5;  // 1-D index of p2
    const float si = (float)std::sin(t->angle), co = (float)std::cos(t->angle);
    auto coef = [&](int sel) -> float {
        switch (sel) {
            case 1: return si;
            case -1: return -si;
            case 2: return co;
            case -2: return -co;
            default: return 0.f;
        }
    };
    // per face: (components of the two E slices, of the two H slices), then the
    // ranges of e1, e2, h1, h2 as {lo_i, hi_i, lo_j, hi_j, lo_k, hi_k}
    for (int f = 0; f < 6; f++) {
        if (!((t->faces >> f) & 1)) continue;
        const int ax = f / 2, back = f & 1;
        int ce[2], ch[2];
        int32_t r[4][6];
        const int32_t xs[2] = {i1, i2}, xsp[2] = {i1, i2 + 1}, ys[2] = {j1, j2}, ysp[2] = {j1, j2 + 1},
                      zs[2] = {k1, k2}, zsp[2] = {k1, k2 + 1};
        if (ax == 0) {
            const int32_t ie = back ? i2 : i1 - 1, ih = back ? i2 : i1;
            ce[0] = 1; ce[1] = 2; ch[0] = 1; ch[1] = 2;   // (ey, ez), (hy, hz)
            const int32_t a[4][6] = {{ie, ie + 1, ysp[0], ysp[1], zs[0], zs[1]},
                                     {ie, ie + 1, ys[0], ys[1], zsp[0], zsp[1]},
                                     {ih, ih + 1, ys[0], ys[1], zsp[0], zsp[1]},
                                     {ih, ih + 1, ysp[0], ysp[1], zs[0], zs[1]}};
            memcpy(r, a, sizeof(r));
        } else if (ax == 1) {
            const int32_t je = back ? j2 : j1 - 1, jh = back ? j2 : j1;
            ce[0] = 2; ce[1] = 0; ch[0] = 2; ch[1] = 0;   // (ez, ex), (hz, hx)
            const int32_t a[4][6] = {{xs[0], xs[1], je, je + 1, zsp[0], zsp[1]},
                                     {xsp[0], xsp[1], je, je + 1, zs[0], zs[1]},
                                     {xsp[0], xsp[1], jh, jh + 1, zs[0], zs[1]},
                                     {xs[0], xs[1], jh, jh + 1, zsp[0], zsp[1]}};
            memcpy(r, a, sizeof(r));
        } else {
            const int32_t ke = back ? k2 : k1 - 1, kh = back ? k2 : k1;
            ce[0] = 0; ce[1] = 1; ch[0] = 0; ch[1] = 1;   // (ex, ey), (hx, hy)
            const int32_t a[4][6] = {{xsp[0], xsp[1], ys[0], ys[1], ke, ke + 1},
                                     {xs[0], xs[1], ysp[0], ysp[1], ke, ke + 1},
                                     {xs[0], xs[1], ysp[0], ysp[1], kh, kh + 1},
                                     {xsp[0], xsp[1], ys[0], ys[1], kh, kh + 1}};
            memcpy(r, a, sizeof(r));
        }
        const IncRow &inc = kInc[kFaceInc[t->axis][f]];
        for (int q = 0; q < 2; q++) {
            TfsfSlice &s = h.s[h.n++];
            const int row = eh == 0 ? q : 2 + q;  // e1, e2 or h1, h2
            s.comp = eh == 0 ? ce[q] : ch[q];
            for (int a = 0; a < 3; a++) {
                s.lo[a] = r[row][2 * a];
                s.hi[a] = r[row][2 * a + 1];
            }
            // E faces read H1d with (ch1, sH1), (ch2, sH2); H faces E1d with (ce1, sE1), (ce2, sE2)
            const int ci = eh == 0 ? 2 + q : q, sid = inc.sl[eh == 0 ? 2 + q : q];
            s.coef = coef(inc.c[ci]);
            if (sid == 3 || sid == 4) {
                s.vary = 1;
                s.idx = 5 - (int32_t)t->p1[t->axis];
            } else {
                s.vary = 0;
                s.idx = sid == 1 ? 4 : (sid == 2 ? 5 : i2d);
            }
            const int64_t cells = (int64_t)(s.hi[0] - s.lo[0]) * (s.hi[1] - s.lo[1]) * (s.hi[2] - s.lo[2]);
            h.cells = cells > h.cells ? cells : h.cells;
        }
    }
    return h;
}

constexpr int kTfsfBlock = 256;

// 1-D E step of step t (one block): interior, then the end values, then the hard source.
__global__ void __launch_bounds__(kTfsfBlock)
k_tfsf_e1d(float *e, const float *h, float *abc, int64_t n, const float *amp, int64_t t) {
    for (int64_t i = 1 + threadIdx.x; i < n - 1; i += blockDim.x) e[i] = fsub(e[i], fmul(0.5f, fsub(h[i + 1], h[i])));
    __syncthreads();
    if (threadIdx.x == 0) {
        e[0] = abc[0];
        abc[0] = abc[1];
        abc[1] = e[1];
        e[n - 1] = abc[2];
        abc[2] = abc[3];
        abc[3] = e[n - 2];
        e[3] = amp[t];
    }
}

__global__ void __launch_bounds__(kTfsfBlock) k_tfsf_h1d(float *h, const float *e, int64_t n) {
    for (int64_t i = 1 + threadIdx.x; i < n; i += blockDim.x) h[i] = fsub(h[i], fmul(0.5f, fsub(e[i], e[i - 1])));
}

// The 1-D H step of step t followed by the 1-D E step of step t+1 (one block;
// between two fused steps).
__global__ void __launch_bounds__(kTfsfBlock)
k_tfsf_he1d(float *e, float *h, float *abc, int64_t n, const float *amp, int64_t t_next) {
    for (int64_t i = 1 + threadIdx.x; i < n; i += blockDim.x) h[i] = fsub(h[i], fmul(0.5f, fsub(e[i], e[i - 1])));
    __syncthreads();
    for (int64_t i = 1 + threadIdx.x; i < n - 1; i += blockDim.x) e[i] = fsub(e[i], fmul(0.5f, fsub(h[i + 1], h[i])));
    __syncthreads();
    if (threadIdx.x == 0) {
        e[0] = abc[0];
        abc[0] = abc[1];
        abc[1] = e[1];
        e[n - 1] = abc[2];
        abc[2] = abc[3];
        abc[3] = e[n - 2];
        e[3] = amp[t_next];
    }
}

// Fused-step form: coefficient and 1-D index of every (half, face, slot) and
// the offset of the varying index (tfsf.py:189-231).
void tfsf_table(const fdtd_tfsf *t, float coef[2][6][2], int32_t ix[2][6][2], int32_t *vo) {
    for (int eh = 0; eh < 2; eh++) {
        const TfsfHalf h = tfsf_half(t, eh);
        int n = 0;
        for (int f = 0; f < 6; f++)
            for (int q = 0; q < 2; q++) {
                coef[eh][f][q] = 0.f;
                ix[eh][f][q] = 0;
                if (!((t->faces >> f) & 1)) continue;
                const TfsfSlice &s = h.s[n++];
                coef[eh][f][q] = s.coef;
                ix[eh][f][q] = s.vary ? -1 : s.idx;
            }
    }
    *vo = 5 - (int32_t)t->p1[t->axis];
}

// which: 0 = 1-D E step of step t, 1 = 1-D H step, 2 = H step then E step of step t
int tfsf_launch_1d(const fdtd_tfsf *t, int which, int64_t step, cudaStream_t st) {
    if (which != 1 && (step < 0 || step >= t->namp)) return FDTD_ERR_ARG;
    const int64_t n = tfsf_n1d(t);
    if (which == 0) k_tfsf_e1d<<<1, kTfsfBlock, 0, st>>>(t->e1d, t->h1d, t->abc, n, t->amp, step);
    else if (which == 1) k_tfsf_h1d<<<1, kTfsfBlock, 0, st>>>(t->h1d, t->e1d, n);
    else k_tfsf_he1d<<<1, kTfsfBlock, 0, st>>>(t->e1d, t->h1d, t->abc, n, t->amp, step);
    return check_launch();
}

// face corrections of slices first, first+1 (one face: two components);
// blockIdx.y picks the slice, threads run over its cells
__global__ void __launch_bounds__(kTfsfBlock)
k_tfsf_faces(Grid g, TfsfHalf half, int first, const float *inc1d, float *f0, float *f1, float *f2) {
    const TfsfSlice &s = half.s[first + blockIdx.y];
    const int64_t ni = s.hi[0] - s.lo[0], nj = s.hi[1] - s.lo[1], nk = s.hi[2] - s.lo[2];
    const int64_t t = (int64_t)blockIdx.x * kTfsfBlock + threadIdx.x;
    if (t >= ni * nj * nk) return;
    const int64_t k = s.lo[2] + t % nk, j = s.lo[1] + (t / nk) % nj, i = s.lo[0] + t / (nk * nj);
    const int64_t ax = half.axis == 0 ? i : (half.axis == 1 ? j : k);
    const float v = inc1d[s.vary ? ax + s.idx : s.idx];
    float *f = s.comp == 0 ? f0 : (s.comp == 1 ? f1 : f2);
    const int64_t c = i * g.sx + j * g.sy + k;
    f[c] = fadd(f[c], fmul(0.5f, fmul(s.coef, v)));
}

// One launch per face, in face order: faces share the cells of the box's
// edges (e.g. hz on the line (p1x, p1y, k) belongs to the x-front and the
// y-front face), which the reference updates one face after the other.
static int launch_tfsf_faces(const Grid &g, const TfsfHalf &h, const float *inc1d, float *f0, float *f1, float *f2,
                             cudaStream_t st) {
    for (int first = 0; first < h.n; first += 2) {
        dim3 grid((unsigned)((h.cells + kTfsfBlock - 1) / kTfsfBlock), 2);
        k_tfsf_faces<<<grid, kTfsfBlock, 0, st>>>(g, h, first, inc1d, f0, f1, f2);
        FDTD_TRY(check_launch());
    }
    return FDTD_OK;
}

}  // namespace fdtd

using namespace fdtd;

extern "C" {

int fdtd_tfsf_update_e_f32(const fdtd_grid *gp, const fdtd_tfsf *t, int64_t tstep, float *ex, float *ey, float *ez,
                           void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!all_nonnull(ex, ey, ez)) return FDTD_ERR_ARG;
    FDTD_TRY(validate_tfsf(g, t));
    if (tstep < 0 || tstep >= t->namp) return FDTD_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    k_tfsf_e1d<<<1, kTfsfBlock, 0, st>>>(t->e1d, t->h1d, t->abc, tfsf_n1d(t), t->amp, tstep);
    FDTD_TRY(check_launch());
    return launch_tfsf_faces(g, tfsf_half(t, 0), t->h1d, ex, ey, ez, st);
}

int fdtd_tfsf_update_h_f32(const fdtd_grid *gp, const fdtd_tfsf *t, float *hx, float *hy, float *hz, void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!all_nonnull(hx, hy, hz)) return FDTD_ERR_ARG;
    FDTD_TRY(validate_tfsf(g, t));
    cudaStream_t st = as_stream(stream);
    k_tfsf_h1d<<<1, kTfsfBlock, 0, st>>>(t->h1d, t->e1d, tfsf_n1d(t));
    FDTD_TRY(check_launch());
    return launch_tfsf_faces(g, tfsf_half(t, 1), t->e1d, hx, hy, hz, st);
}

}  // extern "C"
