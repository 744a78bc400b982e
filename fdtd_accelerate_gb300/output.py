"""Field output on a region: centred fields, Poynting vector, snapshots.

Mirrors kuFDTD's Output (kuFDTD/v0.2.0/dim3/output.py:14-212): a dataform
('e', 'e2', 'ex', 'ey', 'ez', 'ex2', ..., 'h'..., 's', 's2', 'sx', ..., 'sz2'),
the region pt1..pt2 (None: 1 and n-2, as set_space) and a spatial step.
get_data() averages the fields to the cell centres (E over its two nodes, H
over its four), forms the Poynting vector for the 's' forms, and returns the
component, its square, the squared magnitude or the magnitude as a float32
CUDA tensor; axes where pt1 == pt2 are dropped, as the reference's
data_slice does.  `save(path)` writes the array as .npy (the reference's
HDF5 output needs h5py, which this environment does not have).
"""
import ctypes as C

import numpy as np
import torch

from . import _native as N

__all__ = ["Output", "DATAFORMS"]

DATAFORMS = ("e", "e2", "ex", "ey", "ez", "ex2", "ey2", "ez2",
             "h", "h2", "hx", "hy", "hz", "hx2", "hy2", "hz2",
             "s", "s2", "sx", "sy", "sz", "sx2", "sy2", "sz2")


def form_code(dataform):
    d = dataform.lower()
    if d not in DATAFORMS:
        raise ValueError("The dataform is not one of %s" % (DATAFORMS,))
    family = "ehs".index(d[0])
    if len(d) == 1:
        kind, comp = 0, 0
    elif d == d[0] + "2":
        kind, comp = 1, 0
    elif len(d) == 2:
        kind, comp = 2, "xyz".index(d[1])
    else:
        kind, comp = 3, "xyz".index(d[1])
    return family * 16 + kind * 4 + comp


class Output:
    def __init__(self, dataform, pt1, pt2, spatial_step=(1, 1, 1)):
        self.dataform = dataform.lower()
        self.form = form_code(self.dataform)
        self.pt1, self.pt2 = list(pt1), list(pt2)
        self.spatial_step = tuple(int(v) for v in spatial_step)
        self.space = None

    def set_space(self, space):
        """space: a YeeSolver (its current fields) or a dict of six (nx, ny, nz)
        CUDA float32 tensors ex..hz of one layout."""
        self.space = space
        fields = self._fields()
        n = list(fields[0].shape)
        self.p1 = [1 if v is None else int(v) for v in self.pt1]
        self.p2 = [n[a] - 2 if v is None else int(v) for a, v in enumerate(self.pt2)]
        for a in range(3):
            if self.p1[a] < 0 or self.p2[a] < self.p1[a] or self.p2[a] + 1 > n[a] - 1:
                raise ValueError("output region %s..%s does not fit the %s grid" % (self.p1, self.p2, tuple(n)))
        self.shape = tuple((self.p2[a] - self.p1[a]) // self.spatial_step[a] + 1 for a in range(3))
        self.squeeze = tuple(a for a in range(3) if self.p2[a] == self.p1[a])

    def _fields(self):
        from .api import check_field_tensors
        sp = self.space
        if hasattr(sp, "fields"):
            sp = sp.fields
        ts = [sp[k] for k in ("ex", "ey", "ez", "hx", "hy", "hz")]
        check_field_tensors(("ex", "ey", "ez", "hx", "hy", "hz"), ts)
        return ts

    def get_data(self, out=None):
        from .api import grid_of, stream_of
        if self.space is None:
            raise ValueError("set_space first")
        ts = self._fields()
        if out is None:
            out = torch.empty(self.shape, dtype=torch.float32, device=ts[0].device)
        o = N.Output(self.form)
        for a in range(3):
            o.p1[a], o.p2[a], o.step[a] = self.p1[a], self.p2[a], self.spatial_step[a]
        f = (C.c_void_p * 6)(*[t.data_ptr() for t in ts])
        with torch.cuda.device(ts[0].device):
            N.call("fdtd_output_f32", C.byref(grid_of(ts[0])), C.byref(o), f, C.c_void_p(out.data_ptr()),
                   out.numel(), stream_of(ts[0]))
        for a in reversed(self.squeeze):
            out = out.select(a, 0)
        return out

    def save(self, path):
        """Snapshot of get_data() as a .npy file (host copy)."""
        np.save(path, self.get_data().cpu().numpy())
