"""GPU parity of the 4th-order symplectic path (stages, CPML, whole steps)."""
import os

import numpy as np
import pytest
import torch

import oracle
from tests.conftest import cuda_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not cuda_available(), reason="needs a CUDA GPU")]

NAMES = ("ex", "ey", "ez", "hx", "hy", "hz")


@pytest.fixture(scope="module")
def S():
    import fdtd_accelerate_gb300 as F
    F.build()
    from fdtd_accelerate_gb300 import symplectic
    return symplectic


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _host(t):
    return t.detach().cpu().numpy()


def test_golden_reference_c_stages_through_gpu(S, golden_dir):
    """4th_order-Symplectic/Python-C/dielectric.c outputs, reproduced through
    the reference signature update_h(nx, ny, nz, cl, ...)."""
    g = np.load(os.path.join(golden_dir, "symp_c.npz"))
    for n in range(int(g["ncases"])):
        t = "c%d_" % n
        which = int(g[t + "meta"][0])
        f = [_dev(g[t + "in_" + k]) for k in NAMES]
        c = [_dev(g[t + "in_" + k]) for k in ("c0", "c1", "c2")]
        coef = float(g[t + "coef"][()])
        nx, ny, nz = f[0].shape
        if which == 0:
            S.update_h(nx, ny, nz, coef, *f, *c)
            comps = range(3, 6)
        else:
            S.update_e(nx, ny, nz, coef, *f, *c)
            comps = range(0, 3)
        torch.cuda.synchronize()
        for q in comps:
            np.testing.assert_array_equal(_host(f[q])[:-1, :-1, :-1], g[t + "out_" + NAMES[q]][:-1, :-1, :-1],
                                          err_msg="case %d %s" % (n, NAMES[q]))


@pytest.mark.parametrize("shape", [(12, 13, 14), (20, 9, 33)])
def test_stages_bit_exact_vs_oracle(S, shape):
    rng = np.random.default_rng(2)
    f = {k: rng.standard_normal(shape).astype(np.float32) for k in NAMES}
    c = [rng.random(shape, dtype=np.float32) for _ in range(3)]
    d = {k: _dev(v) for k, v in f.items()}
    dc = [_dev(x) for x in c]
    nx, ny, nz = shape
    ch = np.float32(S.COURANT / 24)
    for cl, dl in zip(S.CL[:4], S.DL[:4]):
        oracle.symp_h(np.float32(cl), *(f[k] for k in NAMES), *c)
        S.update_h(nx, ny, nz, cl, *(d[k] for k in NAMES), *dc)
        oracle.symp_h_scalar(np.float32(cl), ch, *(f[k] for k in NAMES))
        S.update_h(nx, ny, nz, cl, *(d[k] for k in NAMES), float(ch))
        oracle.symp_e(np.float32(dl), *(f[k] for k in NAMES), *c)
        S.update_e(nx, ny, nz, dl, *(d[k] for k in NAMES), *dc)
    torch.cuda.synchronize()
    for k in NAMES:
        np.testing.assert_array_equal(_host(d[k]), f[k], err_msg=k)


class OracleSymplectic:
    """The symplectic step of SymplecticSolver restated with oracle calls."""

    def __init__(self, S, shape, ce, ch, npml, faces, sources, dtype=np.float32):
        self.S, self.shape, self.dtype = S, shape, dtype
        self.f = {k: np.zeros(shape, dtype) for k in NAMES}
        self.ce = [np.asarray(c, dtype) for c in ce]
        self.ch = dtype(ch)
        self.npml, self.faces = npml, faces
        self.tables = {}
        for coef in set(S.CL) | set(S.DL[:4]):
            t = [oracle.symp_stage_tables(p, coef, S.COURANT) if p else None for p in npml]
            self.tables[coef] = {k: [x[k] if x is not None else None for x in t]
                                 for k in ("b_e", "a_e", "km1_e", "b_h", "a_h", "km1_h")}
        nx, ny, nz = shape
        ps = [(2 * npml[0], ny, nz), (nx, 2 * npml[1], nz), (nx, ny, 2 * npml[2])]
        self.psi_e = [np.zeros(ps[a], dtype) if npml[a] else None for a in range(3) for _ in range(2)]
        self.psi_h = [np.zeros(ps[a], dtype) if npml[a] else None for a in range(3) for _ in range(2)]
        self.sources = sources
        self.tstep = 1

    def _h(self, cl):
        f = self.f
        oracle.symp_h_scalar(self.dtype(cl), self.ch, *(f[k] for k in NAMES))
        if any(self.npml):
            oracle.symp_cpml_h(self.npml, self.faces, self.dtype(cl), self.ch, self.tables[cl],
                               *(f[k] for k in NAMES), self.psi_h)

    def step(self, n):
        f, S = self.f, self.S
        for _ in range(n):
            tn = self.tstep
            for sn in range(4):
                self._h(S.CL[sn])
                oracle.symp_e(self.dtype(S.DL[sn]), *(f[k] for k in NAMES), *self.ce)
                if any(self.npml):
                    oracle.symp_cpml_e(self.npml, self.faces, self.dtype(S.DL[sn]), self.tables[S.DL[sn]],
                                       *(f[k] for k in NAMES), *self.ce, self.psi_e)
                for comp, (i, j, k), amp in self.sources:
                    f[comp][i, j, k] = f[comp][i, j, k] + self.dtype(np.float32(amp(tn + sn / 5.0)))
            self._h(S.CL[4])
            self.tstep += 1


@pytest.mark.parametrize("shape,npml,faces", [((30, 26, 34), 5, 0x3F), ((24, 28, 20), 4, 0x15),
                                              ((22, 22, 40), 0, 0x3F)])
def test_symplectic_steps_bit_exact_vs_oracle(S, shape, npml, faces):
    from fdtd_accelerate_gb300 import configs
    rng = np.random.default_rng(4)
    spheres = configs.random_spheres(rng, shape, 5, 2, 5, 1.0, 4.0)
    ce = [(c.numpy() * np.float32(S.COURANT / 24 / 0.5)).astype(np.float32)
          for c in configs.ce_from_spheres(shape, spheres)]
    src = [("ez", (shape[0] // 2, shape[1] // 2, shape[2] // 2),
            lambda t: np.sin(0.3 * t) * np.exp(-0.5 * ((t - 4.0) / 2.0) ** 2))]
    solver = S.SymplecticSolver(shape, ce=ce, npml=npml, faces=faces, sources=src, max_steps=8)
    orc = OracleSymplectic(S, shape, ce, S.COURANT / 24, solver.cpml.npml, solver.cpml.faces, src)
    solver.step(6)
    orc.step(6)
    torch.cuda.synchronize()
    for k in NAMES:
        np.testing.assert_array_equal(_host(solver.fields[k]), orc.f[k], err_msg=k)
    for q in range(6):
        if orc.psi_e[q] is not None:
            np.testing.assert_array_equal(_host(solver.cpml.psi_e[q]), orc.psi_e[q], err_msg="psi_e%d" % q)
            np.testing.assert_array_equal(_host(solver.cpml.psi_h[q]), orc.psi_h[q], err_msg="psi_h%d" % q)


@pytest.mark.parametrize("shape,npml,faces,ch_arrays", [((30, 26, 34), 5, 0x3F, False),
                                                        ((24, 28, 20), 4, 0x15, True),
                                                        ((26, 22, 30), 3, 0x2A, False),
                                                        ((22, 22, 40), 0, 0x3F, True),
                                                        ((50, 20, 36), 4, 0x3F, False)])
def test_symplectic_fused_stages_equal_per_call_path(S, shape, npml, faces, ch_arrays):
    """One launch per stage (stage update and CPML slabs together) equals the
    reference-shaped calls (update_h / update_e, then the per-axis CPML
    corrections) bit for bit, with uniform ch and with ch arrays."""
    rng = np.random.default_rng(9)
    ce = [(S.COURANT / 24 / rng.uniform(1.0, 4.0, shape)).astype(np.float32) for _ in range(3)]
    ch = [(S.COURANT / 24 * rng.uniform(0.8, 1.0, shape)).astype(np.float32) for _ in range(3)] if ch_arrays else None
    src = [("ez", (shape[0] // 2, shape[1] // 2, shape[2] // 2),
            lambda t: np.sin(0.3 * t) * np.exp(-0.5 * ((t - 4.0) / 2.0) ** 2))]
    init = {k: (0.1 * rng.standard_normal(shape)).astype(np.float32) for k in NAMES}
    runs = []
    for fused in (True, False):
        s = S.SymplecticSolver(shape, ce=ce, ch=ch, npml=npml, faces=faces, sources=src, max_steps=8)
        s.set_fields(**init)
        (s.step if fused else s.step_unfused)(5)
        runs.append(s)
    torch.cuda.synchronize()
    a, b = runs
    for k in NAMES:
        np.testing.assert_array_equal(_host(a.fields[k]), _host(b.fields[k]), err_msg=k)
    if a.cpml.active:
        for q in range(6):
            if a.cpml.psi_e[q] is not None:
                np.testing.assert_array_equal(_host(a.cpml.psi_e[q]), _host(b.cpml.psi_e[q]), err_msg="psi_e%d" % q)
                np.testing.assert_array_equal(_host(a.cpml.psi_h[q]), _host(b.cpml.psi_h[q]), err_msg="psi_h%d" % q)


def test_symplectic_cpml_absorbs(S):
    """A pulse launched in a CPML box leaves: field energy falls well below the
    PEC box's energy, which stays bounded (the scheme is stable)."""
    shape = (48, 48, 48)
    # derivative of a Gaussian: no DC part, so no static field stays behind
    src = [("ez", (24, 24, 24), lambda t: -(t - 20.0) / 16.0 * np.exp(-0.5 * ((t - 20.0) / 4.0) ** 2))]
    energies = {}
    for npml in (0, 8):
        s = S.SymplecticSolver(shape, npml=npml, sources=src, max_steps=300)
        s.step(300)
        torch.cuda.synchronize()
        energies[npml] = sum(float((t.double() ** 2).sum()) for t in s.f)
        assert np.isfinite(energies[npml])
    assert energies[8] < 0.05 * energies[0], energies


@pytest.mark.parametrize("shape,npml,faces,x_chunk,steps", [
    ((40, 36, 68), 5, 0x3F, 0, 3),        # one x chunk, ragged y and z tiles
    ((44, 34, 72), 6, 0x3F, 8, 4),        # several x chunks: halo planes recomputed at chunk starts
    ((30, 40, 64), 4, 0x15, 5, 2),        # front faces only, odd chunk length
    ((28, 20, 36), 3, 0x2A, 7, 3),        # back faces only
    ((36, 18, 40), 0, 0x3F, 9, 3),        # no CPML
    ((24, 50, 100), 6, 0x3F, 0, 1),       # one step: no merged H stages
    # grids with tiles clear of the y/z slabs (the pair kernel) and an edge shell
    ((40, 60, 132), 5, 0x3F, 0, 3),       # merged H stages on both parts
    ((33, 64, 100), 4, 0x15, 7, 2),       # front faces only
    ((36, 70, 164), 6, 0x30, 0, 2),       # z faces only: no y edge rows
    ((30, 80, 68), 3, 0x0C, 9, 2),        # y faces only
])
def test_stage_pairs_equal_stage_kernels(S, shape, npml, faces, x_chunk, steps):
    """The fused stage pairs (one pass per H+E stage pair, the closing and
    opening H stages of consecutive steps merged) equal the one-launch-per-stage
    path bit for bit: fields, E psi and H psi, with sources on tile edges in y
    and z and on a chunk edge in x, spheres, random initial state."""
    from fdtd_accelerate_gb300 import configs
    rng = np.random.default_rng(12)
    spheres = configs.random_spheres(rng, shape, 5, 2, 5, 1.0, 4.0)
    ce = [(c.numpy() * np.float32(S.COURANT / 24 / 0.5)).astype(np.float32)
          for c in configs.ce_from_spheres(shape, spheres)]
    amp = lambda t: np.sin(0.3 * t) * np.exp(-0.5 * ((t - 4.0) / 2.0) ** 2)
    nx, ny, nz = shape
    src = [("ez", (nx // 2, ny // 2, nz // 2), amp), ("ex", (max(x_chunk, 3), 15, 31), amp),
           ("ey", (nx // 3, 16, 32), lambda t: 0.5 * amp(t + 1.0)), ("ez", (nx - 4, ny - 3, nz - 2), amp)]
    init = {k: (0.1 * rng.standard_normal(shape)).astype(np.float32) for k in NAMES}
    runs = []
    for fused in (True, False):
        s = S.SymplecticSolver(shape, ce=ce, npml=npml, faces=faces, sources=src, max_steps=steps + 2,
                               fused=fused, x_chunk=x_chunk)
        assert s.pair_path() == fused
        s.set_fields(**init)
        s.step(steps)
        runs.append(s)
    torch.cuda.synchronize()
    a, b = runs
    a.check_status()
    for k in NAMES:
        np.testing.assert_array_equal(_host(a.fields[k]), _host(b.fields[k]), err_msg=k)
    if a.cpml.active:
        for q in range(6):
            if a.cpml.psi_e[q] is not None:
                np.testing.assert_array_equal(_host(a.cpml.psi_e[q]), _host(b.cpml.psi_e[q]), err_msg="psi_e%d" % q)
                np.testing.assert_array_equal(_host(a.cpml.psi_h[q]), _host(b.cpml.psi_h[q]), err_msg="psi_h%d" % q)


def test_stage_pairs_then_stage_kernels_interleave(S):
    """Runs alternating between the stage-pair path and the stage kernels keep
    the state (the current buffer, H psi set, step number) consistent."""
    shape, npml = (32, 34, 44), 4
    rng = np.random.default_rng(3)
    init = {k: (0.1 * rng.standard_normal(shape)).astype(np.float32) for k in NAMES}
    src = [("ez", (16, 17, 22), lambda t: np.sin(0.2 * t))]
    a = S.SymplecticSolver(shape, npml=npml, sources=src, max_steps=10, fused=True)
    b = S.SymplecticSolver(shape, npml=npml, sources=src, max_steps=10, fused=False)
    for s in (a, b):
        s.set_fields(**init)
    assert a.pair_path() and not b.pair_path()
    a.step(2)
    a.step_stages(1)
    a.step(3)
    b.step(6)
    torch.cuda.synchronize()
    for k in NAMES:
        np.testing.assert_array_equal(_host(a.fields[k]), _host(b.fields[k]), err_msg=k)
