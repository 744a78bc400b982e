"""Soft (additive) point sources with precomputed amplitude tables.

F[i, j, k] += amp(t) after the E update and its CPML correction, as
updateSrc does in 2nd_order-Yee/CUDA/fdtd3d_201_250x250x320cell_15npml_100000tstep.cu:352-363
and KEMP/v0.7_pml/fdtd3d/naive/incident_direct.py:52-70 (is_overwrite=False).
Amplitudes are evaluated in FP64 on the host and rounded once to FP32.
"""
import ctypes as C
import math

import numpy as np
import torch

from . import _native as N

__all__ = ["gaussian_sine", "PointSources", "COMPONENTS"]

COMPONENTS = {"ex": 0, "ey": 1, "ez": 2}


def gaussian_sine(n, t0=150.0, width=30.0, freq=0.05):
    """sin(2 pi freq n) exp(-((n - t0)/width)^2 / 2), FP64, n = step number
    (pulse of 2nd_order-Yee/Numpy/new_pml_test/gaussian.py:7-8,27)."""
    n = np.asarray(n, dtype=np.float64)
    return np.sin(2.0 * math.pi * freq * n) * np.exp(-0.5 * ((n - t0) / width) ** 2)


class PointSources:
    """A list of (component, (i, j, k), amplitude table) soft sources.

    The table of source s is indexed by the step number t (0-based index
    into the array; entries past its end add nothing).
    """

    def __init__(self, shape, sources, device="cuda"):
        nx, ny, nz = shape
        self.shape = tuple(shape)
        self.device = torch.device(device)
        srcs = list(sources)
        namp = max([len(a) for _, _, a in srcs], default=0)
        ijk = np.zeros((len(srcs), 3), np.int32)
        comp = np.zeros(len(srcs), np.int32)
        amp = np.zeros((len(srcs), namp), np.float64)
        for s, (c, (i, j, k), a) in enumerate(srcs):
            if c not in COMPONENTS:
                raise ValueError("source component must be one of ex, ey, ez : %r" % (c,))
            if not (0 <= i < nx and 0 <= j < ny and 0 <= k < nz):
                raise ValueError("source point %s outside grid %s" % ((i, j, k), self.shape))
            ijk[s] = (i, j, k)
            comp[s] = COMPONENTS[c]
            amp[s, :len(a)] = a
        self.sources = srcs
        self.namp = namp
        self.ijk_host = ijk
        self.comp_host = comp
        self.amp_host = amp.astype(np.float32)
        self.ijk = torch.tensor(ijk.reshape(-1), device=self.device)
        self.comp = torch.tensor(comp, device=self.device)
        self.amp = torch.tensor(self.amp_host.reshape(-1), device=self.device)

    def __len__(self):
        return len(self.sources)

    def struct(self):
        s = N.Sources()
        s.nsrc = len(self.sources)
        s.ijk = self.ijk.data_ptr() if len(self) else None
        s.comp = self.comp.data_ptr() if len(self) else None
        s.amp = self.amp.data_ptr() if len(self) and self.namp else None
        s.namp = self.namp
        return s

    def apply(self, t, ex, ey, ez):
        """Add the step-t amplitudes to E (reference order: list order)."""
        from .api import check_field_tensors, grid_of, stream_of
        ref = check_field_tensors(("ex", "ey", "ez"), (ex, ey, ez))
        g = grid_of(ref)
        st = self.struct()
        with torch.cuda.device(ref.device):
            N.call("fdtd_add_sources_f32", C.byref(g), C.byref(st), int(t),
                   *[C.c_void_p(x.data_ptr()) for x in (ex, ey, ez)], stream_of(ref))
