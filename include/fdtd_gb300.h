/*
 * fdtd_gb300.h -- C ABI of the GB300 (sm_103a) Yee time-step engine.
 *
 * Plain C: pointers, sizes, an opaque stream handle.  All field pointers
 * are DEVICE pointers to float32 arrays of logical shape (nx, ny, nz),
 * z fastest, with element strides sx (x) and sy (y) and unit z stride --
 * the memory layout of the reference's C-order NumPy field arrays (and of
 * KEMP's z-padded arrays).  Every entry point that launches work is
 * stream-ordered on its `stream` and does not synchronise the host, except
 * plan creation: fdtd_yee_plan_create (when the grid has sources) and
 * fdtd_batch_plan_create read or write device memory on the given stream
 * and wait for that stream once before they return, so they belong
 * outside stream capture; the plans' run calls are stream-ordered and
 * capturable.  No entry point allocates device memory, none exits the
 * process, and each returns an fdtd_status.  `stream` is a cudaStream_t
 * (NULL = legacy default stream).
 *
 * Reference interfaces replaced (paths inside wbkifun/fdtd_accelerate):
 *   fdtd_update_e_f32      2nd_order-Yee/Numpy/fdtd3d.py:10-13 update_e;
 *                          2nd_order-Yee/python-C/dielectric-sse-omp.c:68-121;
 *                          KEMP/v0.7_pml/fdtd3d/cpu/src/core.c:11 (ctypes
 *                          argtypes KEMP/v0.7_pml/fdtd3d/cpu/core.py:89-105)
 *   fdtd_update_h_f32      2nd_order-Yee/Numpy/fdtd3d.py:4-7 update_h;
 *                          KEMP/v0.7_pml/fdtd3d/cpu/src/core.c:59 (ch arrays
 *                          of coeff_use='h', naive/core.py:37-47)
 *   fdtd_update_pbc_{e,h}  2nd_order-Yee/Numpy/fdtd3d.py:16-37
 *   fdtd_cpml_{e,h}_f32    kuFDTD/v0.2.0/dim3/cpu/core/cpml_non_kappa.c:14-429
 *                          update_{x,y,z}_{e,h} (one call covers all axes and
 *                          faces), with the kappa term of
 *                          kuFDTD/before_CUDA/v0.3.0/boundary/core/cpml_core.c:238-263
 *   fdtd_add_sources_f32   2nd_order-Yee/CUDA/fdtd3d_201_250x250x320cell_15npml_100000tstep.cu:352-363
 *                          updateSrc; KEMP/v0.7_pml/fdtd3d/naive/incident_direct.py:52-70
 *   fdtd_drude_update_e_f32  kuFDTD/v0.2.0/dim3/cpu/core/drude_ade.c:14-93
 *                          drude_ade.update_e (Ncore, Nx, Ny, Nz, idx0,
 *                          spaceNyz, spaceNz, Ex..CEz, Jx..CJBz): the box and
 *                          strides travel in fdtd_drude / fdtd_grid
 *   fdtd_tfsf_update_{e,h}_f32  kuFDTD/v0.2.0/dim3/tfsf.py Tfsf.updateE(tstep) /
 *                          updateH() (Fdtd1d + TfsfFace + TfsfIncNormal)
 *   fdtd_output_f32        kuFDTD/v0.2.0/dim3/output.py Output.get_data()
 *                          (centred fields, Poynting vector, square/sum/sqrt)
 *   fdtd_step_unfused_f32  one time step in the order of
 *                          fdtd3d_201_..._100000tstep.cu:718-742
 *   fdtd_yee_plan_*, fdtd_yee_step_f32  the same step, fused into one pass per
 *                          step (the step function as one call, or a plan)
 *                          (no reference counterpart as one call; replaces
 *                          the >= 15 launches per step of the loop above)
 *   fdtd_symplectic_{h,e}_f32  4th_order-Symplectic/PyCUDA/100-base.py:10-44
 *                          update_h / update_e (stage coefficient argument);
 *                          4th_order-Symplectic/Python-C/dielectric.c:5-96
 *   fdtd_symplectic_stage_f32  one stage of PyCUDA/100-base.py:124-141 with
 *                          its CPML slabs in the same launch
 */
#ifndef FDTD_GB300_H
#define FDTD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    FDTD_OK = 0,
    FDTD_ERR_ARG = 1,         /* null pointer or invalid scalar argument   */
    FDTD_ERR_SHAPE = 2,       /* extents / strides inconsistent            */
    FDTD_ERR_ALIGN = 3,       /* pointer or stride alignment requirement   */
    FDTD_ERR_CUDA = 4,        /* CUDA runtime/driver error (see fdtd_last_cuda_error) */
    FDTD_ERR_TIMEOUT = 5,     /* a bounded device-side wait expired        */
    FDTD_ERR_UNSUPPORTED = 6, /* configuration not supported by this path  */
    FDTD_ERR_CAPACITY = 7     /* request exceeds a fixed capacity          */
} fdtd_status;

/* Grid: logical extents and element strides (z stride is 1). */
typedef struct {
    int64_t nx, ny, nz;
    int64_t sx, sy;
} fdtd_grid;

/* CPML: slab thickness per axis (0 = none), enabled faces (bit 2a = front,
 * bit 2a+1 = back face of axis a), and device tables of 2*npml[a] entries:
 * b, a and km1 = 1/kappa - 1, for E nodes and H nodes.  Slab index s < P is
 * the front slab at node s+1; s >= P the back slab at node n-P-1+(s-P)
 * (E) or n-P+(s-P) (H). */
typedef struct {
    int32_t npml[3];
    int32_t faces;
    const float *b_e[3], *a_e[3], *km1_e[3];
    const float *b_h[3], *a_h[3], *km1_h[3];
} fdtd_cpml;

/* psi slabs, dense: x (2P, ny, nz), y (nx, 2P, nz), z (nx, ny, 2P).
 * e: eyx, ezx, ezy, exy, exz, eyz     h: hyx, hzx, hzy, hxy, hxz, hyz
 * (NULL allowed for an axis without PML). */
typedef struct {
    float *e[6];
    float *h[6];
} fdtd_psi;

/* Soft sources: F[i,j,k] += amp[s*namp + t] for step t (0 <= t < namp),
 * applied after the E update and its CPML correction, in list order.
 * comp: 0..2 = ex, ey, ez.  All arrays are device arrays. */
typedef struct {
    int32_t nsrc;
    const int32_t *ijk;   /* 3*nsrc */
    const int32_t *comp;  /* nsrc   */
    const float *amp;     /* nsrc*namp */
    int64_t namp;
} fdtd_sources;

/* Drude dispersive region (auxiliary differential equation): a sub-box of
 * ni x nj x nk cells starting at cell (i0, j0, k0) of the E arrays, with
 * dense (ni, nj, nk) device arrays per component: j = polarisation current
 * (state, updated in place), cja and cjb = its coefficients.  After the E
 * update and before its CPML correction, per cell and component:
 *   e' = e - ce*J;  e = e';  J = cja*J + cjb*e'
 * Replaces kuFDTD DrudeAde (kuFDTD/v0.2.0/dim3/cpu/matter.py:222-314,
 * kuFDTD/v0.2.0/dim3/cpu/core/drude_ade.c:14-93).  j2: a second J buffer for
 * the fused step, which reads J from buffer `cur` (j when cur = 0, j2 when
 * cur = 1, as the fields) and writes the other (neighbouring tiles recompute
 * halo cells from the old J); unused by fdtd_drude_update_e_f32 (in place
 * on j). */
typedef struct {
    int64_t i0, j0, k0, ni, nj, nk;
    float *j[3];
    const float *cja[3], *cjb[3];
    float *j2[3];
} fdtd_drude;

/* Total-field/scattered-field plane wave at normal incidence (kuFDTD Tfsf,
 * kuFDTD/v0.2.0/dim3/tfsf.py:14-244).  p1, p2: corners of the total-field
 * box as set_space leaves them (p2 = the given pt2 + 1); faces: bit f on for
 * face f = x front, x back, y front, y back, z front, z back; axis: the
 * propagation axis 0..2; angle: polarisation angle (radians).  The 1-D
 * auxiliary grid lives in device arrays e1d, h1d of n1d = p2[axis] -
 * p1[axis] + 11 floats and abc[4] (two-step delay of both ends), zeroed by
 * the caller; amp[t] (t < namp) = sin(w dt t) is the hard source written
 * to e1d[3] in step t. */
typedef struct {
    int64_t p1[3], p2[3];
    int32_t faces, axis;
    double angle;
    float *e1d, *h1d, *abc;
    const float *amp;
    int64_t namp;
} fdtd_tfsf;

/* Field output on the region p1..p2 (inclusive) sampled every step cells
 * (kuFDTD Output, kuFDTD/v0.2.0/dim3/output.py:14-212): the fields averaged
 * to the cell centres, then per form = family*16 + kind*4 + comp with family
 * 0 E, 1 H, 2 Poynting S and kind 0 |v|, 1 |v|^2, 2 v[comp], 3 v[comp]^2
 * (dataforms 'e', 'e2', 'ex', 'ex2', 'h', ..., 's', 's2', 'sx', 'sx2'). */
typedef struct {
    int32_t form;
    int64_t p1[3], p2[3], step[3];
} fdtd_output;

const char *fdtd_status_string(int status);
int fdtd_last_cuda_error(void);
/* Bounds-checked debug build (the library compiled with -DFDTD_CHECK,
 * libfdtd_gb300_check.so; no reference counterpart: the reference has no
 * checked build): kernels compare each wrapped global index with its array's
 * extent and skip an access outside it.  Writes the first miss recorded since
 * the last call, (1 << 63) | (source line << 40) | (index & (2^40 - 1)), or 0,
 * and clears the record; waits for the device.  The product build returns
 * FDTD_ERR_UNSUPPORTED. */
int fdtd_debug_check(uint64_t *first_bad);

/* ---- reference-shaped kernels (in place) ---------------------------- */
int fdtd_update_e_f32(const fdtd_grid *g, float *ex, float *ey, float *ez,
                      const float *hx, const float *hy, const float *hz,
                      const float *cex, const float *cey, const float *cez, void *stream);
/* ch pointers may be NULL: constant 0.5 (fdtd3d.py / KEMP coeff_use='') */
int fdtd_update_h_f32(const fdtd_grid *g, const float *ex, const float *ey, const float *ez,
                      float *hx, float *hy, float *hz,
                      const float *chx, const float *chy, const float *chz, void *stream);
/* axes: bit 0 = x, 1 = y, 2 = z */
int fdtd_update_pbc_e_f32(const fdtd_grid *g, int32_t axes, float *ex, float *ey, float *ez, void *stream);
int fdtd_update_pbc_h_f32(const fdtd_grid *g, int32_t axes, float *hx, float *hy, float *hz, void *stream);
int fdtd_cpml_e_f32(const fdtd_grid *g, const fdtd_cpml *c,
                    float *ex, float *ey, float *ez,
                    const float *hx, const float *hy, const float *hz,
                    const float *cex, const float *cey, const float *cez,
                    const fdtd_psi *psi, void *stream);
int fdtd_cpml_h_f32(const fdtd_grid *g, const fdtd_cpml *c,
                    const float *ex, const float *ey, const float *ez,
                    float *hx, float *hy, float *hz,
                    const float *chx, const float *chy, const float *chz,
                    const fdtd_psi *psi, void *stream);
int fdtd_add_sources_f32(const fdtd_grid *g, const fdtd_sources *src, int64_t t,
                         float *ex, float *ey, float *ez, void *stream);
/* TFSF: the 1-D E step (tfsf.py:26-38) of step t, then E += 0.5 * incident H
 * on every enabled face (tfsf.py:234-237); call it after fdtd_cpml_e_f32.
 * The H form: the 1-D H step, then H += 0.5 * incident E (tfsf.py:240-244);
 * call it after fdtd_cpml_h_f32.  The box must lie inside the grid with one
 * cell to spare on each side (the E faces sit at p1-1 and p2). */
int fdtd_tfsf_update_e_f32(const fdtd_grid *g, const fdtd_tfsf *t, int64_t tstep, float *ex, float *ey, float *ez,
                           void *stream);
int fdtd_tfsf_update_h_f32(const fdtd_grid *g, const fdtd_tfsf *t, float *hx, float *hy, float *hz, void *stream);
/* Output of o into out (C order, n[a] = (p2[a]-p1[a])/step[a] + 1 per axis,
 * out_len >= their product); the region needs p2 + 1 <= n - 1 on every axis
 * (the averages read the next node). */
int fdtd_output_f32(const fdtd_grid *g, const fdtd_output *o, const float *const f[6], float *out, int64_t out_len,
                    void *stream);
/* Drude ADE on the box of d (in place on E and d->j); call it between
 * fdtd_update_e_f32 and fdtd_cpml_e_f32. */
int fdtd_drude_update_e_f32(const fdtd_grid *g, const fdtd_drude *d, float *ex, float *ey, float *ez,
                            const float *cex, const float *cey, const float *cez, void *stream);

/* One whole step, unfused (update_e, cpml_e, sources, update_h, cpml_h),
 * in place.  c and src may be NULL. */
int fdtd_step_unfused_f32(const fdtd_grid *g, float *const f[6], const float *const ce[3],
                          const float *const ch[3], const fdtd_cpml *c, const fdtd_psi *psi,
                          const fdtd_sources *src, int64_t t, void *stream);

/* ---- fused Yee step (one HBM pass per step) --------------------------- */
/* State in two buffers (ping-pong): f[b] = ex,ey,ez,hx,hy,hz of buffer b,
 * psi_e[b] the E-psi slabs of buffer b; psi_h is updated in place.
 * Requirements: sx, sy multiples of 4 and 16-byte aligned base pointers;
 * nx, ny, nz >= 2.  ch is the constant 0.5 on this path. */
typedef struct {
    float *f[2][6];
    float *psi_e[2][6];
    float *psi_h[6];
    const float *ce[3];
    const fdtd_drude *drude;  /* NULL: no dispersive region */
    const fdtd_tfsf *tfsf;    /* NULL: no plane wave; else the fused step applies it (box
                                 faces at least P+2 cells away from every CPML slab) */
} fdtd_yee_state;

/* Launch shape of the fused kernel (0 = default): tile height in y (4, 8
 * or 16 cells; the tile is 64 cells wide in z), x planes per work item,
 * resident CTAs per SM (persistent grid), pipeline stages (planes staged in
 * shared memory), L2 promotion of the tile loads (0 = 256 B, 1 = none,
 * 2 = 64 B, 3 = 128 B).  x_chunk 0 picks a chunk that gives every SM
 * about three work items, and for a grid without CPML (work items of equal
 * cost) the chunk of 128 .. 8 planes whose persistent launch is shortest
 * (ceil(items / CTAs) items of chunk + 3 plane steps). */
typedef struct {
    int32_t tile_y;
    int32_t x_chunk;
    int32_t ctas_per_sm;
    int32_t stages;
    int32_t l2_promotion;
} fdtd_tile;

typedef struct fdtd_yee_plan fdtd_yee_plan;

/* status_dev: device int32 the kernel sets non-zero when a bounded wait
 * expires (may be NULL). cur: index of the buffer holding the state now.
 * stream: the source positions (device array src->ijk) are read on this
 * stream, after any work queued on it, and the call waits for that read
 * (host-side capacity checks need them). */
int fdtd_yee_plan_create(fdtd_yee_plan **plan, const fdtd_grid *g, const fdtd_yee_state *st,
                         const fdtd_cpml *c, const fdtd_sources *src, const fdtd_tile *tile,
                         int32_t *status_dev, int32_t cur, void *stream);
int fdtd_yee_plan_run(fdtd_yee_plan *plan, int64_t t0, int64_t nsteps, void *stream);
int fdtd_yee_plan_current(const fdtd_yee_plan *plan);
int fdtd_yee_plan_set_current(fdtd_yee_plan *plan, int32_t cur);
/* Test hook for the bounded device waits (no reference counterpart: the
 * reference's kernels never wait on a copy).  wait_ns > 0 replaces the 1 s
 * limit of every mbarrier wait of the plan's fused kernel (0 restores it);
 * withhold_plane >= 0 makes CTA 0 skip the copies of that plane of its first
 * work item, so that its wait runs out with no copy in flight, the kernel
 * writes FDTD_ERR_TIMEOUT to status_dev and every CTA returns; -1 issues
 * every copy.  The aborted step leaves the output buffer partly written. */
int fdtd_yee_plan_test_timeout(fdtd_yee_plan *plan, int64_t wait_ns, int32_t withhold_plane);
/* info[0..5] = tile_y, stages, x_chunk, CTAs launched, threads/CTA, shared bytes/CTA;
 * with n >= 8 also info[6] = 1 when the z slab runs on the band kernels and
 * info[7] = kernel launches per step */
int fdtd_yee_plan_info(const fdtd_yee_plan *plan, int32_t *info, int32_t n);
int fdtd_yee_plan_destroy(fdtd_yee_plan *plan);

/* nsteps fused steps in one call: fdtd_yee_plan_create (default launch
 * shape), fdtd_yee_plan_run, fdtd_yee_plan_destroy, all on `stream`.  The
 * plan's host set-up (tensor-map encoding, occupancy query, the read of the
 * source positions on `stream`: the call waits for that stream once before
 * it launches) is paid on every call; keep a plan for repeated short runs.  cur: buffer holding
 * the state now; *cur_out
 * (may be NULL) receives the buffer holding it after the steps.  Replaces
 * the time loop of fdtd3d_201_250x250x320cell_15npml_100000tstep.cu:718-742
 * (update_e, CPML-E, source, update_h, CPML-H per step) as one call. */
int fdtd_yee_step_f32(const fdtd_grid *g, const fdtd_yee_state *st, const fdtd_cpml *c,
                      const fdtd_sources *src, int32_t *status_dev, int32_t cur,
                      int64_t t0, int64_t nsteps, int32_t *cur_out, void *stream);

/* ---- fused 4th-order stage pair (one HBM pass per H+E stage pair) ------- */
/* State in two buffers (ping-pong): f[b] = ex,ey,ez,hx,hy,hz of buffer b,
 * psi_h[b] the H psi slabs of buffer b (layouts of fdtd_psi); the E psi
 * slabs psi_e are updated in place.  Requirements: C-order arrays with
 * 16-byte aligned bases and rows (nz a multiple of 4 floats), fewer than
 * 2^31 elements each, nx, ny, nz >= 4, a uniform ch. */
typedef struct {
    float *f[2][6];
    float *psi_e[6];
    float *psi_h[2][6];
    const float *ce[3];
} fdtd_symp_state;

typedef struct fdtd_symp_plan fdtd_symp_plan;

/* x_chunk: x planes per work item (0: the plan picks it per tiling, from a model of the
 * work-queue schedule); cur: buffer holding the state;
 * status_dev: device int32 set non-zero when a bounded wait expires;
 * queue_dev: device int32[2], zero at plan creation, the work queue the
 * CTAs draw items from (the kernel leaves it zero after each run; runs of
 * plans sharing it must not overlap); the source positions are read on
 * `stream` (the call waits for it once). */
int fdtd_symp_pair_plan_create(fdtd_symp_plan **plan, const fdtd_grid *g, const fdtd_symp_state *st,
                               const fdtd_sources *src, int32_t x_chunk, int32_t cur,
                               int32_t *status_dev, int32_t *queue_dev, void *stream);
/* One pass: the H stage cl_a (with two_h = 1, then the H stage cl_b), the E
 * stage dl, then the sources at amplitude index src_t, reading buffer cur and
 * writing the other.  Each stage's CPML tables come from its fdtd_cpml (the
 * H tables of h_a / h_b, the E tables of e; NULL: no CPML); ch is uniform.
 * Bit-identical to fdtd_symplectic_stage_f32 for each stage in turn and
 * fdtd_add_sources_f32.  Replaces one (update_h, update_e) pair of the
 * stage loop of 4th_order-Symplectic/PyCUDA/100-base.py:124-141. */
int fdtd_symp_pair_run(fdtd_symp_plan *plan, const fdtd_cpml *h_a, const fdtd_cpml *h_b,
                       const fdtd_cpml *e, float cl_a, float cl_b, int32_t two_h, float dl,
                       float ch, int64_t src_t, void *stream);
int fdtd_symp_pair_plan_current(const fdtd_symp_plan *plan);
int fdtd_symp_pair_plan_set_current(fdtd_symp_plan *plan, int32_t cur);
int fdtd_symp_pair_plan_destroy(fdtd_symp_plan *plan);

/* ---- batched fused step: many independent grids, one launch per step --- */
/* Every grid keeps its own state, CPML and sources (arrays as for
 * fdtd_yee_plan_create); all grids advance together (same buffer index,
 * same step number).  The per-grid launch parameters and TMA descriptors
 * live in a caller-provided device workspace of
 * fdtd_batch_workspace_bytes(nsims) bytes, 64-byte aligned (the plan
 * allocates no device memory).  Each grid's result equals its own
 * fdtd_yee_plan_run bit for bit.  No reference counterpart as one call:
 * replaces one reference time loop per simulation. */
typedef struct fdtd_batch_plan fdtd_batch_plan;
size_t fdtd_batch_workspace_bytes(int32_t nsims);
/* stream: the workspace is filled on this stream, after the work queued on
 * it (earlier launches that may still read the workspace), and the call
 * waits for the copies before it returns. */
int fdtd_batch_plan_create(fdtd_batch_plan **plan, int32_t nsims, const fdtd_grid *grids,
                           const fdtd_yee_state *states, const fdtd_cpml *cpmls,
                           const fdtd_sources *srcs, const fdtd_tile *tile, int32_t *status_dev,
                           void *workspace, size_t workspace_bytes, int32_t cur, void *stream);
int fdtd_batch_plan_run(fdtd_batch_plan *plan, int64_t t0, int64_t nsteps, void *stream);
int fdtd_batch_plan_current(const fdtd_batch_plan *plan);
int fdtd_batch_plan_set_current(fdtd_batch_plan *plan, int32_t cur);
/* info[0..5] = tile_y, stages, work items, CTAs launched, threads/CTA, shared bytes/CTA */
int fdtd_batch_plan_info(const fdtd_batch_plan *plan, int32_t *info, int32_t n);
int fdtd_batch_plan_destroy(fdtd_batch_plan *plan);

/* The batched form in one call: fdtd_batch_plan_create (default launch
 * shape), fdtd_batch_plan_run, fdtd_batch_plan_destroy, all on `stream`;
 * workspace as for fdtd_batch_plan_create (whose copies into the workspace
 * make the call wait for that stream once before it launches).  *cur_out (may be
 * NULL) receives the buffer holding every grid's state after the steps. */
int fdtd_batched_run_f32(int32_t nsims, const fdtd_grid *grids, const fdtd_yee_state *states,
                         const fdtd_cpml *cpmls, const fdtd_sources *srcs, int32_t *status_dev,
                         void *workspace, size_t workspace_bytes, int32_t cur,
                         int64_t t0, int64_t nsteps, int32_t *cur_out, void *stream);

/* ---- adjoint (reverse-time) step -------------------------------------- */
/* Point lists: comp 0..5 = ex, ey, ez, hx, hy, hz at (i, j, k); device arrays. */
typedef struct {
    int32_t n;
    const int32_t *ijk;   /* 3*n */
    const int32_t *comp;  /* n   */
} fdtd_points;

typedef struct {
    float *f[6];
} fdtd_fields6;

/* Adjoint state of the fused/unfused 2nd-order step (ch = 0.5).  lf: adjoint
 * fields (grid layout); lpsi_e/lpsi_h: adjoint psi (layouts of fdtd_psi);
 * w_e/w_h: scratch of the same layouts; grad_ce: dL/dCE accumulators (grid
 * layout).  psi entries may be NULL on axes without PML. */
typedef struct {
    float *lf[6];
    float *lpsi_e[6], *lpsi_h[6];
    float *w_e[6], *w_h[6];
    float *grad_ce[3];
} fdtd_adjoint_state;

/* One reverse step n: first adds mon_grad[p] to the adjoint of monitor
 * point p (the monitors read the state at the end of step n), then applies
 * the transpose of step n (cpml_h, update_h, cpml_e, update_e) and adds
 * lE * (E increment / CE) to grad_ce.  h_prev: forward H entering step n;
 * psi_e_cur: forward E-psi after step n.  mon may be NULL.  No reference
 * counterpart: the reference has no gradient path. */
int fdtd_adjoint_step_f32(const fdtd_grid *g, const fdtd_cpml *c, const fdtd_adjoint_state *s,
                          const float *const h_prev[3], const float *const psi_e_cur[6],
                          const float *const ce[3], const fdtd_points *mon, const float *mon_grad,
                          void *stream);
/* fdtd_adjoint_step_f32 with dL/dCE accumulated only on the cells of the box
 * grad_box = {i0, j0, k0, ni, nj, nk} (a design region; grad_ce is left
 * untouched outside it).  The adjoint fields lf / lpsi evolve exactly as in
 * fdtd_adjoint_step_f32; cells outside the box skip the forward-H reads and
 * the accumulator's read and write.  A box outside the grid: FDTD_ERR_SHAPE.
 * No reference counterpart. */
int fdtd_adjoint_step_region_f32(const fdtd_grid *g, const fdtd_cpml *c, const fdtd_adjoint_state *s,
                                 const float *const h_prev[3], const float *const psi_e_cur[6],
                                 const float *const ce[3], const fdtd_points *mon, const float *mon_grad,
                                 const int64_t grad_box[6], void *stream);
/* fdtd_adjoint_step_f32 without caller scratch: s->w_e / s->w_h are ignored
 * and a device array of 4 Mi floats (16 MiB) inside the library is used
 * instead, for callers that cannot allocate device memory.  A CPML layer
 * whose 12 w arrays (4*(2Px*ny*nz + nx*2Py*nz + nx*ny*2Pz) floats plus
 * alignment) do not fit returns FDTD_ERR_CAPACITY.  The first call on a
 * device sets it up and should come before any stream capture; calls that
 * overlap in time on one device race on the shared scratch.  No counterpart
 * in the reference. */
int fdtd_adjoint_step_noalloc_f32(const fdtd_grid *g, const fdtd_cpml *c, const fdtd_adjoint_state *s,
                                  const float *const h_prev[3], const float *const psi_e_cur[6],
                                  const float *const ce[3], const fdtd_points *mon, const float *mon_grad,
                                  void *stream);
/* out[p] = f[comp[p]][i, j, k] (NaN for a point outside the grid) */
int fdtd_gather_points_f32(const fdtd_grid *g, const fdtd_points *pts, const float *const f[6],
                           float *out, void *stream);
/* f[comp[p]][i, j, k] += vals[p], in list order (points outside the grid skipped) */
int fdtd_add_points_f32(const fdtd_grid *g, const fdtd_points *pts, float *const f[6],
                        const float *vals, void *stream);

/* ---- FP64 step (accuracy checks) --------------------------------------- */
/* One whole step in FP64, unfused and in place, with the FP32 step's
 * operation order (update_e, cpml_e, sources, update_h, cpml_h; ch = 0.5).
 * The CPML tables (fdtd_cpml) and source amplitudes stay FP32 and are widened.
 * psi arrays: the layouts of fdtd_psi, in double.  No reference counterpart as
 * one call: the reference's NumPy step run in float64. */
int fdtd_step_unfused_f64(const fdtd_grid *g, double *const f[6], const double *const ce[3],
                          const fdtd_cpml *c, double *const psi_e[6], double *const psi_h[6],
                          const fdtd_sources *src, int64_t t, void *stream);
/* out[p] = f[comp[p]][i, j, k] in double (NaN for a point outside the grid) */
int fdtd_gather_points_f64(const fdtd_grid *g, const fdtd_points *pts, const double *const f[6],
                           double *out, void *stream);
/* The soft sources of fdtd_add_sources_f32 on double arrays (FP32 amplitudes
 * widened), list order. */
int fdtd_add_sources_f64(const fdtd_grid *g, const fdtd_sources *src, int64_t t,
                         double *ex, double *ey, double *ez, void *stream);
/* One 4th-order stage with its stage-wise CPML in FP64, in place: the
 * arithmetic of fdtd_symplectic_stage_f32 in double (4th_order-Symplectic/
 * PyCUDA/100-base.py:10-44 run in float64).  coef, ch_scalar and cf are the
 * FP32 path's values widened; the CPML tables stay FP32 and are widened; psi:
 * the stage's six psi arrays (E stage: E psi, H stage: H psi) in double. */
int fdtd_symplectic_stage_f64(const fdtd_grid *g, const fdtd_cpml *c, int32_t e_or_h, double coef,
                              double ch_scalar, double *const f[6], const double *const cf[3],
                              double *const psi[6], void *stream);

/* ---- 4th-order symplectic stages (in place) --------------------------- */
int fdtd_symplectic_h_f32(const fdtd_grid *g, float cl,
                          const float *ex, const float *ey, const float *ez,
                          float *hx, float *hy, float *hz,
                          const float *chx, const float *chy, const float *chz, void *stream);
int fdtd_symplectic_e_f32(const fdtd_grid *g, float dl,
                          float *ex, float *ey, float *ez,
                          const float *hx, const float *hy, const float *hz,
                          const float *cex, const float *cey, const float *cez, void *stream);

/* H stage with a uniform ch (4th-order workload: ch = S/24); same update as
 * fdtd_symplectic_h_f32 with ch arrays filled with `ch`. */
int fdtd_symplectic_h_scalar_f32(const fdtd_grid *g, float cl, float ch,
                                 const float *ex, const float *ey, const float *ez,
                                 float *hx, float *hy, float *hz, void *stream);
/* 4th-order CPML stage corrections (no reference counterpart: the
 * reference's 4th-order programs have no absorbing boundary).  c holds the
 * stage's b/a tables (b = exp(-(sigma/kappa+alpha)*coef*S)) and km1; slab
 * geometry and psi layout as fdtd_cpml_{e,h}_f32.  Call after the stage's
 * main update.  ch arrays may be NULL: uniform ch. */
int fdtd_symplectic_cpml_e_f32(const fdtd_grid *g, const fdtd_cpml *c, float dl,
                               float *ex, float *ey, float *ez,
                               const float *hx, const float *hy, const float *hz,
                               const float *cex, const float *cey, const float *cez,
                               const fdtd_psi *psi, void *stream);
int fdtd_symplectic_cpml_h_f32(const fdtd_grid *g, const fdtd_cpml *c, float cl, float ch,
                               const float *ex, const float *ey, const float *ez,
                               float *hx, float *hy, float *hz,
                               const float *chx, const float *chy, const float *chz,
                               const fdtd_psi *psi, void *stream);

/* One whole stage in one launch: the stage update of fdtd_symplectic_h_f32 /
 * fdtd_symplectic_h_scalar_f32 (e_or_h = 0, coef = cl) or
 * fdtd_symplectic_e_f32 (e_or_h = 1, coef = dl) followed, on the slabs of
 * the enabled faces, by the corrections of fdtd_symplectic_cpml_{h,e}_f32 in
 * their order (x, y, z), with the same arithmetic (bit-identical results).
 * f = ex, ey, ez, hx, hy, hz; c = the updated field's coefficient arrays
 * (ce for E; ch for H, or NULL with ch_scalar).  c (the CPML tables of this
 * stage) and psi may be NULL: no absorbing slabs.  Replaces the stage loop
 * body of 4th_order-Symplectic/PyCUDA/100-base.py:124-141 (one kernel per
 * stage there as well). */
int fdtd_symplectic_stage_f32(const fdtd_grid *g, const fdtd_cpml *c, int32_t e_or_h, float coef,
                              float ch_scalar, float *const f[6], const float *const cf[3],
                              const fdtd_psi *psi, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* FDTD_GB300_H */
