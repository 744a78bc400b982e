// Field output on a region (kuFDTD/v0.2.0/dim3/output.py:14-212): the fields
// averaged to the cell centres (E over its two nodes along its own axis, H
// over its four nodes in the plane across it), optionally combined into the
// Poynting vector, then a component, its square, the squared magnitude or the
// magnitude, sampled every `step` cells.  Float32 arithmetic in the order
// NumPy evaluates the reference's expressions:
//   E: 0.5 * (E[c] + E[c+1]),  H: 0.25 * (((H[c] + H[c+a]) + H[c+b]) + H[c+a+b])
//   S: e1*h1 - e2*h2,  sum of squares ((0 + d0^2) + d1^2) + d2^2,  sqrt.
#include "common.cuh"

namespace fdtd {

struct OutArgs {
    int32_t family, kind, comp;  // family 0 E, 1 H, 2 S; kind 0 |v|, 1 |v|^2, 2 v_comp, 3 v_comp^2
    int64_t p1[3], n[3], step[3];
};

__device__ __forceinline__ float cen_e(const Grid &g, const float *const f[6], int q, int64_t c) {
    const int64_t st = q == 0 ? g.sx : (q == 1 ? g.sy : 1);
    return fmul(0.5f, fadd(f[q][c], f[q][c + st]));
}

__device__ __forceinline__ float cen_h(const Grid &g, const float *const f[6], int q, int64_t c) {
    // the two axes across component q, in the order of output.py:124-135
    const int64_t a = q == 0 ? g.sy : g.sx, b = q == 2 ? g.sy : 1;
    const float *h = f[3 + q];
    return fmul(0.25f, fadd(fadd(fadd(h[c], h[c + a]), h[c + b]), h[c + a + b]));
}

__global__ void __launch_bounds__(256) k_output(Grid g, OutArgs o, const float *ex, const float *ey, const float *ez,
                                                const float *hx, const float *hy, const float *hz, float *out) {
    const int64_t t = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (t >= o.n[0] * o.n[1] * o.n[2]) return;
    const int64_t k = o.p1[2] + (t % o.n[2]) * o.step[2];
    const int64_t j = o.p1[1] + ((t / o.n[2]) % o.n[1]) * o.step[1];
    const int64_t i = o.p1[0] + (t / (o.n[2] * o.n[1])) * o.step[0];
    const int64_t c = i * g.sx + j * g.sy + k;
    const float *const f[6] = {ex, ey, ez, hx, hy, hz};
    float v[3];
    int nv;
    if (o.family < 2) {
        if (o.kind >= 2) {
            v[0] = o.family == 0 ? cen_e(g, f, o.comp, c) : cen_h(g, f, o.comp, c);
            nv = 1;
        } else {
            for (int q = 0; q < 3; q++) v[q] = o.family == 0 ? cen_e(g, f, q, c) : cen_h(g, f, q, c);
            nv = 3;
        }
    } else {
        // Poynting: output.py:205-211 (all three) and 198-201 (one component)
        const float cx = cen_e(g, f, 0, c), cy = cen_e(g, f, 1, c), cz = cen_e(g, f, 2, c);
        const float hxc = cen_h(g, f, 0, c), hyc = cen_h(g, f, 1, c), hzc = cen_h(g, f, 2, c);
        const float sx = fsub(fmul(cy, hzc), fmul(cz, hyc));
        const float sy = fsub(fmul(cz, hxc), fmul(cx, hzc));
        const float sz = fsub(fmul(cx, hyc), fmul(cy, hxc));
        if (o.kind >= 2) {
            v[0] = o.comp == 0 ? sx : (o.comp == 1 ? sy : sz);
            nv = 1;
        } else {
            v[0] = sx;
            v[1] = sy;
            v[2] = sz;
            nv = 3;
        }
    }
    float r;
    if (o.kind == 2) {
        r = v[0];
    } else if (o.kind == 3) {
        r = fmul(v[0], v[0]);
    } else {
        r = fmul(v[0], v[0]);  // 0 + v0^2 == v0^2 (squares are not -0)
        for (int q = 1; q < nv; q++) r = fadd(r, fmul(v[q], v[q]));
        if (o.kind == 0) r = __fsqrt_rn(r);
    }
    out[t] = r;
}

}  // namespace fdtd

using namespace fdtd;

extern "C" {

int fdtd_output_f32(const fdtd_grid *gp, const fdtd_output *o, const float *const f[6], float *out, int64_t out_len,
                    void *stream) {
    Grid g;
    FDTD_TRY(validate_grid(gp, &g));
    if (!o || !f || !out) return FDTD_ERR_ARG;
    for (int q = 0; q < 6; q++)
        if (!f[q]) return FDTD_ERR_ARG;
    OutArgs a;
    a.family = o->form >> 4;
    a.kind = (o->form >> 2) & 3;
    a.comp = o->form & 3;
    if (a.family > 2 || a.comp > 2 || (o->form & ~0x3F)) return FDTD_ERR_ARG;
    const int64_t n3[3] = {g.nx, g.ny, g.nz};
    int64_t total = 1;
    for (int ax = 0; ax < 3; ax++) {
        // every averaged node lies inside the grid: p2 + 1 <= n - 1
        if (o->p1[ax] < 0 || o->p2[ax] < o->p1[ax] || o->p2[ax] + 1 > n3[ax] - 1) return FDTD_ERR_SHAPE;
        if (o->step[ax] < 1) return FDTD_ERR_ARG;
        a.p1[ax] = o->p1[ax];
        a.step[ax] = o->step[ax];
        a.n[ax] = (o->p2[ax] - o->p1[ax]) / o->step[ax] + 1;
        total *= a.n[ax];
    }
    if (out_len < total) return FDTD_ERR_CAPACITY;
    k_output<<<(unsigned)((total + 255) / 256), 256, 0, as_stream(stream)>>>(g, a, f[0], f[1], f[2], f[3], f[4], f[5],
                                                                             out);
    return check_launch();
}

}  // extern "C"
