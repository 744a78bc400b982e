"""Differentiable FP64 restatement of the 2nd-order Yee step with kappa CPML.

Test infrastructure only (the oracle): it pins the hand-written adjoint
kernels by PyTorch autograd on the same step.  Semantics follow the C oracle
(oracle/fdtd_oracle.c), which restates
  update_e / update_h    2nd_order-Yee/Numpy/fdtd3d.py:4-13
  cpml_e / cpml_h        kuFDTD/before_CUDA/v0.3.0/boundary/core/cpml_core.c:238-263
                         with the slab ranges of kuFDTD/v0.2.0/dim3/cpu/core/cpml_non_kappa.c
  step order             update_e, cpml_e, sources, update_h, cpml_h
                         (2nd_order-Yee/CUDA/fdtd3d_201_250x250x320cell_15npml_100000tstep.cu:718-742)
Every operation is out of place so autograd sees the whole map; ch = 0.5.
"""
import torch
import torch.nn.functional as Fn

__all__ = ["TorchYee"]


def _nodes(P, n, front, back, kind):
    """Slab node indices (2P) and the enabled mask per slab index."""
    if kind == "e":
        idx = list(range(1, P + 1)) + [n - P - 1 + s for s in range(P)]
    else:
        idx = list(range(1, P + 1)) + [n - P + s for s in range(P)]
    on = [bool(front)] * P + [bool(back)] * P
    return torch.tensor(idx), torch.tensor(on)


class TorchYee:
    """shape, npml (Px, Py, Pz), faces bitmask, tables: per-axis dicts of
    b_e, a_e, km1_e, b_h, a_h, km1_h (tensors or arrays, length 2P)."""

    def __init__(self, shape, npml=(0, 0, 0), faces=0x3F, tables=None, dtype=torch.float64):
        self.shape = tuple(shape)
        self.npml = tuple(int(p) for p in npml)
        self.faces = faces
        self.dtype = dtype
        self.ax = []
        for a in range(3):
            P = self.npml[a]
            if P == 0:
                self.ax.append(None)
                continue
            n = self.shape[a]
            front, back = (faces >> (2 * a)) & 1, (faces >> (2 * a + 1)) & 1
            ie, on = _nodes(P, n, front, back, "e")
            ih, _ = _nodes(P, n, front, back, "h")
            t = {k: torch.as_tensor(tables[a][k]).to(dtype) for k in ("b_e", "a_e", "km1_e", "b_h", "a_h", "km1_h")}
            self.ax.append(dict(P=P, ie=ie, ih=ih, on=on, **t))

    def zero_state(self):
        z = lambda s: torch.zeros(s, dtype=self.dtype)
        nx, ny, nz = self.shape
        ps = [(2 * self.npml[0], ny, nz), (nx, 2 * self.npml[1], nz), (nx, ny, 2 * self.npml[2])]
        E = [z(self.shape) for _ in range(3)]
        H = [z(self.shape) for _ in range(3)]
        pe = [z(ps[a]) if self.npml[a] else None for a in range(3) for _ in range(2)]
        ph = [z(ps[a]) if self.npml[a] else None for a in range(3) for _ in range(2)]
        return E, H, pe, ph

    # broadcasting helpers: table along the slab axis of the psi layout
    @staticmethod
    def _bc(v, axis):
        return v.view(-1, 1, 1) if axis == 0 else v.view(1, -1, 1) if axis == 1 else v.view(1, 1, -1)

    @staticmethod
    def _take(f, idx, axis):
        return f.index_select(axis, idx)

    def _psi_term(self, A, axis, which, psi, d, valid):
        """psi' = b psi + a d on enabled slabs with the element mask; returns
        (psi', km1 d + psi') zeroed where not applied."""
        b = self._bc(A["b_" + which], axis)
        a = self._bc(A["a_" + which], axis)
        k = self._bc(A["km1_" + which], axis)
        on = self._bc(A["on"], axis) & valid
        psi_new = torch.where(on, b * psi + a * d, psi)
        term = torch.where(on, k * d + psi_new, torch.zeros_like(d))
        return psi_new, term

    def step(self, E, H, pe, ph, ce, t=None, sources=()):
        """One step; returns (E, H, pe, ph).  sources: (comp 0..2, (i, j, k), amplitude)."""
        ex, ey, ez = E
        hx, hy, hz = H
        cex, cey, cez = ce
        nx, ny, nz = self.shape
        # ---- update_e
        cx = (hz[:, 1:, :-1] - hz[:, :-1, :-1]) - (hy[:, :-1, 1:] - hy[:, :-1, :-1])
        cy = (hx[:-1, :, 1:] - hx[:-1, :, :-1]) - (hz[1:, :, :-1] - hz[:-1, :, :-1])
        cz = (hy[1:, :-1, :] - hy[:-1, :-1, :]) - (hx[:-1, 1:, :] - hx[:-1, :-1, :])
        ex = ex + cex * Fn.pad(cx, (0, 1, 0, 1, 0, 0))
        ey = ey + cey * Fn.pad(cy, (0, 1, 0, 0, 0, 1))
        ez = ez + cez * Fn.pad(cz, (0, 0, 0, 1, 0, 1))
        # ---- cpml_e
        pe = list(pe)
        kr = lambda n: torch.arange(n)
        if self.ax[0] is not None:
            A = self.ax[0]
            ie = A["ie"]
            d1 = self._take(hz, ie + 1, 0) - self._take(hz, ie, 0)
            d2 = self._take(hy, ie + 1, 0) - self._take(hy, ie, 0)
            v1 = (kr(nz) < nz - 1).view(1, 1, -1)
            v2 = (kr(ny) < ny - 1).view(1, -1, 1)
            pe[0], t1 = self._psi_term(A, 0, "e", pe[0], d1, v1)
            pe[1], t2 = self._psi_term(A, 0, "e", pe[1], d2, v2)
            ey = ey.index_add(0, ie, -(self._take(cey, ie, 0) * t1))
            ez = ez.index_add(0, ie, self._take(cez, ie, 0) * t2)
        if self.ax[1] is not None:
            A = self.ax[1]
            je = A["ie"]
            d1 = self._take(hx, je + 1, 1) - self._take(hx, je, 1)
            d2 = self._take(hz, je + 1, 1) - self._take(hz, je, 1)
            v1 = (kr(nx) < nx - 1).view(-1, 1, 1)
            v2 = (kr(nz) < nz - 1).view(1, 1, -1)
            pe[2], t1 = self._psi_term(A, 1, "e", pe[2], d1, v1)
            pe[3], t2 = self._psi_term(A, 1, "e", pe[3], d2, v2)
            ez = ez.index_add(1, je, -(self._take(cez, je, 1) * t1))
            ex = ex.index_add(1, je, self._take(cex, je, 1) * t2)
        if self.ax[2] is not None:
            A = self.ax[2]
            ke = A["ie"]
            d1 = self._take(hy, ke + 1, 2) - self._take(hy, ke, 2)
            d2 = self._take(hx, ke + 1, 2) - self._take(hx, ke, 2)
            v1 = (kr(ny) < ny - 1).view(1, -1, 1)
            v2 = (kr(nx) < nx - 1).view(-1, 1, 1)
            pe[4], t1 = self._psi_term(A, 2, "e", pe[4], d1, v1)
            pe[5], t2 = self._psi_term(A, 2, "e", pe[5], d2, v2)
            ex = ex.index_add(2, ke, -(self._take(cex, ke, 2) * t1))
            ey = ey.index_add(2, ke, self._take(cey, ke, 2) * t2)
        # ---- sources
        E = [ex, ey, ez]
        for comp, (i, j, k), amp in sources:
            idx = (torch.tensor([i]), torch.tensor([j]), torch.tensor([k]))
            E[comp] = E[comp].index_put(idx, torch.tensor([float(amp)], dtype=self.dtype), accumulate=True)
        ex, ey, ez = E
        # ---- update_h
        sx = (ez[:, 1:, 1:] - ez[:, :-1, 1:]) - (ey[:, 1:, 1:] - ey[:, 1:, :-1])
        sy = (ex[1:, :, 1:] - ex[1:, :, :-1]) - (ez[1:, :, 1:] - ez[:-1, :, 1:])
        sz = (ey[1:, 1:, :] - ey[:-1, 1:, :]) - (ex[1:, 1:, :] - ex[1:, :-1, :])
        hx = hx - 0.5 * Fn.pad(sx, (1, 0, 1, 0, 0, 0))
        hy = hy - 0.5 * Fn.pad(sy, (1, 0, 0, 0, 1, 0))
        hz = hz - 0.5 * Fn.pad(sz, (0, 0, 1, 0, 1, 0))
        # ---- cpml_h
        ph = list(ph)
        if self.ax[0] is not None:
            A = self.ax[0]
            ih = A["ih"]
            d1 = self._take(ez, ih, 0) - self._take(ez, ih - 1, 0)
            d2 = self._take(ey, ih, 0) - self._take(ey, ih - 1, 0)
            v1 = (kr(nz) > 0).view(1, 1, -1)
            v2 = (kr(ny) > 0).view(1, -1, 1)
            ph[0], t1 = self._psi_term(A, 0, "h", ph[0], d1, v1)
            ph[1], t2 = self._psi_term(A, 0, "h", ph[1], d2, v2)
            hy = hy.index_add(0, ih, 0.5 * t1)
            hz = hz.index_add(0, ih, -(0.5 * t2))
        if self.ax[1] is not None:
            A = self.ax[1]
            jh = A["ih"]
            d1 = self._take(ex, jh, 1) - self._take(ex, jh - 1, 1)
            d2 = self._take(ez, jh, 1) - self._take(ez, jh - 1, 1)
            v1 = (kr(nx) > 0).view(-1, 1, 1)
            v2 = (kr(nz) > 0).view(1, 1, -1)
            ph[2], t1 = self._psi_term(A, 1, "h", ph[2], d1, v1)
            ph[3], t2 = self._psi_term(A, 1, "h", ph[3], d2, v2)
            hz = hz.index_add(1, jh, 0.5 * t1)
            hx = hx.index_add(1, jh, -(0.5 * t2))
        if self.ax[2] is not None:
            A = self.ax[2]
            kh = A["ih"]
            d1 = self._take(ey, kh, 2) - self._take(ey, kh - 1, 2)
            d2 = self._take(ex, kh, 2) - self._take(ex, kh - 1, 2)
            v1 = (kr(ny) > 0).view(1, -1, 1)
            v2 = (kr(nx) > 0).view(-1, 1, 1)
            ph[4], t1 = self._psi_term(A, 2, "h", ph[4], d1, v1)
            ph[5], t2 = self._psi_term(A, 2, "h", ph[5], d2, v2)
            hx = hx.index_add(2, kh, 0.5 * t1)
            hy = hy.index_add(2, kh, -(0.5 * t2))
        return [ex, ey, ez], [hx, hy, hz], pe, ph

    def run(self, ce, nsteps, sources=(), monitors=(), checkpoint_every=0):
        """Monitor series (nsteps, nmon) and final fields from a zero state.
        sources: (comp, ijk, table indexed by step number); monitors:
        (comp 0..5, ijk).  checkpoint_every > 0 recomputes segments in
        backward (torch.utils.checkpoint) to bound host memory."""
        E, H, pe, ph = self.zero_state()
        rows = []

        def seg(t0, n, *flat):
            E, H = list(flat[0:3]), list(flat[3:6])
            k = 6
            pe_, ph_ = [], []
            for lst in (pe_, ph_):
                for q in range(6):
                    lst.append(flat[k] if flat[k].numel() else None)
                    k += 1
            out_rows = []
            for s in range(n):
                t = t0 + s + 1
                srcs = [(c, ijk, tab[t]) for c, ijk, tab in sources]
                E, H, pe_, ph_ = self.step(E, H, pe_, ph_, ce, t, srcs)
                f6 = E + H
                out_rows.append(torch.stack([f6[c][i, j, k] for c, (i, j, k) in monitors])
                                if monitors else torch.zeros(0, dtype=self.dtype))
            empty = torch.zeros(0, dtype=self.dtype)
            return (torch.stack(out_rows), *E, *H, *[p if p is not None else empty for p in pe_ + ph_])

        empty = torch.zeros(0, dtype=self.dtype)
        flat = (*E, *H, *[p if p is not None else empty for p in pe + ph])
        K = checkpoint_every if checkpoint_every > 0 else nsteps
        t0 = 0
        while t0 < nsteps:
            n = min(K, nsteps - t0)
            if checkpoint_every > 0:
                from torch.utils.checkpoint import checkpoint
                out = checkpoint(seg, t0, n, *flat, use_reentrant=False)
            else:
                out = seg(t0, n, *flat)
            rows.append(out[0])
            flat = out[1:]
            t0 += n
        return torch.cat(rows), list(flat[0:6])
