"""KEMP-style object API on the GPU (drop-in for KEMP/v0.7_pml/fdtd3d/{cpu,gpu}).

    fields = Fields(nx, ny, nz, coeff_use='e')          # cpu/fields.py:8-145
    Core(fields)                                         # cpu/core.py:8-123
    Pml(fields, ('+-', '+-', '+-'), npml=12)             # naive/pml.py:8-190 (kappa CPML)
    IncidentDirect(fields, 'ez', pt0, pt1, tfunc)        # cpu/incident_direct.py:9-85
    getf = GetFields(fields, 'ez', pt0, pt1)             # cpu/get_set_fields.py:7-63
    for t in range(n): fields.update_e(); fields.update_h()

Instances run in KEMP's priority order core < current < pml < incident < pbc
(util/common.py:383-397).  Field arrays are z-padded CUDA float32 tensors
(KEMP pads nz to a 16-byte pitch, cpu/fields.py:27-31); `fields.get(name)`
returns the (nx, ny, nz) view.  Argument checks raise TypeError/ValueError
as util/common.py:6-53 does.
"""
import types

import numpy as np
import torch

from . import api
from .cpml import CpmlLayer

__all__ = ["Fields", "Core", "Pml", "IncidentDirect", "GetFields", "SetFields", "Pbc",
           "check_type", "check_value", "slices_two_points", "shape_two_points", "convert_indices"]

_PRIORITY = {"core": 0, "current": 1, "pml": 2, "incident": 3, "pbc": 4, "mpi": 5, "exchange": 6}
_EH = ("ex", "ey", "ez", "hx", "hy", "hz")


def check_type(arg_name, arg, arg_type, element_type=None):
    if not isinstance(arg, arg_type):
        raise TypeError("argument '%s' type must be a %s : %s is given" % (arg_name, repr(arg_type), type(arg)))
    if isinstance(arg, (list, tuple)):
        if element_type is None:
            raise TypeError("argument '%s': element_type must be given for a list or tuple" % arg_name)
        for element in arg:
            if not isinstance(element, element_type):
                raise TypeError("argument '%s's element type must be a %s : %s is given"
                                % (arg_name, repr(element_type), type(element)))


def check_value(arg_name, arg, values):
    values = tuple(values) if isinstance(values, (list, tuple, range)) else (values,)
    if arg not in values:
        raise ValueError("argument '%s' value must be one of %s : %s is given"
                         % (arg_name, repr(values if len(values) < 8 else values[:2] + ('...',) + values[-2:]),
                            repr(arg)))


def convert_indices(ns, pt):
    """Negative ints count from the end, floats are fractions of n (util/common.py:219-262)."""
    out = []
    for n, p in zip(ns, pt):
        if isinstance(p, (bool, np.bool_)):
            raise TypeError("point coordinates must be int or float")
        if isinstance(p, (int, np.integer)):
            out.append(int(p) if p >= 0 else int(n + p))
        elif isinstance(p, float):
            out.append(int(n * p))
        else:
            raise TypeError("point coordinates must be int or float : %s is given" % type(p))
    return tuple(out)


def slices_two_points(pt0, pt1):
    return tuple(slice(p0, p1 + 1) if p0 != p1 else p0 for p0, p1 in zip(pt0, pt1))


def shape_two_points(pt0, pt1, mul_x=1, is_dummy=False):
    shape = []
    for p0, p1 in zip(pt0, pt1):
        v = abs(p1 - p0) + 1
        if v != 1 or is_dummy:
            shape.append(v)
    if not shape:
        return (mul_x,)
    shape[0] *= mul_x
    return tuple(shape)


class Fields:
    def __init__(self, nx, ny, nz, coeff_use="e", precision_float="single", device="cuda", segment_nbytes=16):
        check_type("nx", nx, int)
        check_type("ny", ny, int)
        check_type("nz", nz, int)
        check_value("coeff_use", coeff_use, ("", "e", "h", "eh"))
        check_value("precision_float", precision_float, ("single",))
        check_type("segment_nbytes", segment_nbytes, int)
        self.dtype = np.float32
        self.align_size = max(1, segment_nbytes // 4)
        self.pad = int(np.ceil(nz / self.align_size) * self.align_size) - nz
        self.nx, self.ny, self.nz = nx, ny, nz
        self.ns = [nx, ny, nz]
        self.ns_pitch = [nx, ny, nz + self.pad]
        self.ns_pad = [nx, ny, self.pad]
        self.slice_z = slice(None, None) if self.pad == 0 else slice(None, -self.pad)
        self.device = torch.device(device)
        self.precision_float = precision_float
        self.coeff_use = coeff_use
        self.ce_on = "e" in coeff_use
        self.ch_on = "h" in coeff_use
        z = lambda v: torch.full(self.ns_pitch, v, dtype=torch.float32, device=self.device)
        self._store = {k: z(0.0) for k in _EH}
        # KEMP initialises coefficients to 0.5 (cpu/fields.py:50-54); without
        # 'e' the E update uses 0.5 arrays too (the kernels take arrays)
        for k in ("cex", "cey", "cez"):
            self._store[k] = z(0.5)
        if self.ch_on:
            for k in ("chx", "chy", "chz"):
                self._store[k] = z(0.5)
        self.ehs = [self.get(k) for k in _EH]
        self.ex, self.ey, self.ez, self.hx, self.hy, self.hz = self.ehs
        self.ces = [self.get(k) for k in ("cex", "cey", "cez")]
        self.cex, self.cey, self.cez = self.ces
        self.chs = [self.get(k) for k in ("chx", "chy", "chz")] if self.ch_on else None
        if self.ch_on:
            self.chx, self.chy, self.chz = self.chs
        self.instance_list = []

    def append_instance(self, instance):
        new = _PRIORITY[instance.priority_type]
        idx = len(self.instance_list)
        for i, inst in enumerate(self.instance_list):
            if new < _PRIORITY[inst.priority_type]:
                idx = i
                break
        self.instance_list.insert(idx, instance)

    def get(self, str_f):
        valid = list(_EH) + ["cex", "cey", "cez"] + (["chx", "chy", "chz"] if self.ch_on else [])
        check_value("str_f", str_f, valid)
        return self._store[str_f][:, :, :self.nz]

    def _set(self, names, arrays):
        for name, a in zip(names, arrays):
            if not isinstance(a, (np.ndarray, torch.Tensor)):
                raise TypeError("argument '%s' type must be a numpy.ndarray or torch.Tensor : %s is given"
                                % (name, type(a)))
            self.get(name).copy_(torch.as_tensor(np.asarray(a) if isinstance(a, np.ndarray) else a,
                                                 dtype=torch.float32))

    def set_ehs(self, ex, ey, ez, hx, hy, hz):
        self._set(_EH, (ex, ey, ez, hx, hy, hz))

    def set_ces(self, cex, cey, cez):
        self._set(("cex", "cey", "cez"), (cex, cey, cez))

    def set_chs(self, chx, chy, chz):
        if not self.ch_on:
            raise AttributeError("The Fields instance has no ch arrays. You should add 'h' in the option 'coeff_use'")
        self._set(("chx", "chy", "chz"), (chx, chy, chz))

    def update_e(self):
        for inst in self.instance_list:
            inst.update_e()

    def update_h(self):
        for inst in self.instance_list:
            inst.update_h()

    def enqueue_barrier(self):
        torch.cuda.synchronize(self.device)


class Core:
    """E/H curl updates (KEMP cpu/core.py:118-123 -> the sm_103a kernels)."""

    priority_type = "core"

    def __init__(self, fields):
        check_type("fields", fields, Fields)
        self.mainf = fields
        fields.append_instance(self)

    def update_e(self):
        f = self.mainf
        api.update_e(*f.ehs, *f.ces)

    def update_h(self):
        f = self.mainf
        if f.ch_on:
            api.update_h(*f.ehs, *f.chs)
        else:
            api.update_h(*f.ehs)


class Pml:
    """Kappa CPML on the faces named per axis ('+', '-', '+-', ''), KEMP's
    Pml(fields, directions, npml, sigma_max, kappa_max, alpha_max, m_sigma, m_alpha)
    (naive/pml.py:8-45) with sigma_max derived from the reflection R."""

    priority_type = "pml"

    def __init__(self, fields, directions, npml=12, R=1e-8, kappa_max=5.0, alpha_max=0.05, m_sigma=4, m_alpha=1,
                 dt=0.5):
        check_type("fields", fields, Fields)
        check_type("directions", directions, (list, tuple), str)
        if len(directions) != 3:
            raise ValueError("directions must have 3 entries")
        for d in directions:
            check_value("direction", d, ("+", "-", "+-", "-+", ""))
        self.mainf = fields
        self.layer = CpmlLayer(fields.ns, npml, tuple(directions), m=m_sigma, R=R, kappa_max=kappa_max,
                               alpha_max=alpha_max, m_alpha=m_alpha, dt=dt, device=fields.device)
        fields.append_instance(self)

    def update_e(self):
        f = self.mainf
        self.layer.update_e(*f.ehs, *f.ces)

    def update_h(self):
        f = self.mainf
        if f.ch_on:
            self.layer.update_h(*f.ehs, *f.chs)
        else:
            self.layer.update_h(*f.ehs)


class Pbc:
    """Periodic planes along the given axes (2nd_order-Yee/Numpy/fdtd3d.py:16-37)."""

    priority_type = "pbc"

    def __init__(self, fields, axes):
        check_type("fields", fields, Fields)
        check_type("axes", axes, str)
        for a in axes:
            check_value("axes", a, ("x", "y", "z"))
        self.mainf, self.axes = fields, axes
        fields.append_instance(self)

    def update_e(self):
        f = self.mainf
        api.update_pbc_e(self.axes, f.ex, f.ey, f.ez)

    def update_h(self):
        f = self.mainf
        api.update_pbc_h(self.axes, f.hx, f.hy, f.hz)


def _check_points(fields, pt0, pt1):
    check_type("pt0", pt0, (list, tuple), (int, float))
    check_type("pt1", pt1, (list, tuple), (int, float))
    pt0 = list(convert_indices(fields.ns, pt0))
    pt1 = list(convert_indices(fields.ns, pt1))
    for axis, n, p0, p1 in zip("xyz", fields.ns, pt0, pt1):
        check_value("pt0 %s" % axis, p0, range(n))
        check_value("pt1 %s" % axis, p1, range(n))
    return pt0, pt1


class GetFields:
    """Asynchronous copy of a region to pinned host memory (cpu/get_set_fields.py:7-63)."""

    def __init__(self, fields, str_f, pt0, pt1):
        check_type("fields", fields, Fields)
        check_type("str_f", str_f, (str, list, tuple), str)
        pt0, pt1 = _check_points(fields, pt0, pt1)
        self.str_fs = (str_f,) if isinstance(str_f, str) else tuple(str_f)
        for s in self.str_fs:
            check_value("str_f", s, _EH)
        self.mainf = fields
        self.slices = slices_two_points(pt0, pt1)
        shape = shape_two_points(pt0, pt1, len(self.str_fs))
        self.host_array = torch.zeros(shape, dtype=torch.float32).pin_memory()
        self.split = dict(zip(self.str_fs, torch.chunk(self.host_array, len(self.str_fs))))

    def get_event(self):
        for s in self.str_fs:
            self.split[s].copy_(self.mainf.get(s)[self.slices].reshape(self.split[s].shape), non_blocking=True)
        evt = torch.cuda.Event()
        evt.record()
        return evt

    def get_fields(self, str_f=""):
        if str_f == "":
            return self.host_array.numpy()
        return self.split[str_f].numpy()


class SetFields:
    """Region overwrite / add of a scalar or array (cpu/get_set_fields.py:67-127)."""

    def __init__(self, fields, str_f, pt0, pt1, is_array=False, is_overwrite=True):
        check_type("fields", fields, Fields)
        check_type("str_f", str_f, (str, list, tuple), str)
        check_type("is_array", is_array, bool)
        check_type("is_overwrite", is_overwrite, bool)
        pt0, pt1 = _check_points(fields, pt0, pt1)
        self.str_fs = (str_f,) if isinstance(str_f, str) else tuple(str_f)
        for s in self.str_fs:
            check_value("str_f", s, _EH)
        self.mainf = fields
        self.slices = slices_two_points(pt0, pt1)
        self.shape = shape_two_points(pt0, pt1, len(self.str_fs))
        self.is_array, self.is_overwrite = is_array, is_overwrite

    def set_fields(self, values):
        f = self.mainf
        if self.is_array:
            v = torch.as_tensor(values)
            if v.dtype != torch.float32:
                raise ValueError("argument 'value.dtype' value must be float32 : %s is given" % v.dtype)
            if tuple(v.shape) != self.shape:
                raise ValueError("argument 'value.shape' value must be %s : %s is given" % (self.shape, tuple(v.shape)))
            parts = torch.chunk(v.to(f.device), len(self.str_fs))
            for s, part in zip(self.str_fs, parts):
                view = f.get(s)[self.slices]
                part = part.reshape(view.shape)
                if self.is_overwrite:
                    view.copy_(part)
                else:
                    view.add_(part)
        else:
            val = float(np.float32(values))
            for s in self.str_fs:
                view = f.get(s)[self.slices]
                if self.is_overwrite:
                    view.fill_(val)
                else:
                    view.add_(val)


class IncidentDirect:
    """Region source F[region] (+)= f32(tfunc(tstep)) * spatial_value after the
    E (or H) update (naive/incident_direct.py:9-70, cpu/incident_direct.py:9-85)."""

    priority_type = "incident"

    def __init__(self, fields, str_f, pt0, pt1, tfunc, spatial_value=1.0, is_overwrite=False):
        check_type("fields", fields, Fields)
        check_value("str_f", str_f, _EH)
        check_type("tfunc", tfunc, types.FunctionType)
        check_type("spatial_value", spatial_value, (np.ndarray, np.number, float, int))
        check_type("is_overwrite", is_overwrite, bool)
        pt0, pt1 = _check_points(fields, pt0, pt1)
        self.mainf, self.tfunc = fields, tfunc
        self.e_or_h = str_f[0]
        is_array = isinstance(spatial_value, np.ndarray)
        if is_array:
            shape = shape_two_points(pt0, pt1)
            if shape != spatial_value.shape:
                raise ValueError("shape mismatch : %s, %s" % (shape, spatial_value.shape))
            if spatial_value.dtype != np.float32:
                raise ValueError("dtype mismatch : float32, %s" % spatial_value.dtype)
            self.svalue = torch.as_tensor(spatial_value).to(fields.device)
        else:
            self.svalue = np.float32(spatial_value)
        self.str_f = str_f
        self.slices = slices_two_points(pt0, pt1)
        self.is_overwrite = is_overwrite
        self.tstep = 1
        fields.append_instance(self)

    def update(self):
        amp = np.float32(self.tfunc(self.tstep))
        view = self.mainf.get(self.str_f)[self.slices]
        if isinstance(self.svalue, np.float32):
            v = float(np.float32(amp * self.svalue))
            if self.is_overwrite:
                view.fill_(v)
            else:
                view.add_(v)
        else:
            v = (self.svalue * float(amp)).reshape(view.shape)
            if self.is_overwrite:
                view.copy_(v)
            else:
                view.add_(v)
        self.tstep += 1

    def update_e(self):
        if self.e_or_h == "e":
            self.update()

    def update_h(self):
        if self.e_or_h == "h":
            self.update()
