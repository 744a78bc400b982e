"""Many independent Yee grids advanced by one launch per step.

The reference runs one simulation per process and time loop (e.g.
2nd_order-Yee/CUDA/fdtd3d_201_250x250x320cell_15npml_100000tstep.cu:718-742).
BatchSolver keeps a list of YeeSolver grids of any (uneven) sizes and
advances all of them with the batched fused kernel: the work items of every
grid (z tile x y tile x x chunk) form one list that the persistent CTAs walk,
so small grids that would leave most SMs idle on their own fill the GPU
together.  Each grid's result is bit-identical to its own YeeSolver.step.

A run of n steps can be captured into one CUDA graph (``run_graph``) so the
n launches go to the GPU as a single submission; the launch shape comes from
``autotune`` (timed candidates, cached in a JSON file).
"""
import ctypes as C
import json
import os

import torch

from . import _native as N
from .solver import YeeSolver

__all__ = ["BatchSolver", "TILE_CANDIDATES", "tune_cache_path"]

# (tile_y, x_chunk, ctas_per_sm, stages) candidates for the autotuner
TILE_CANDIDATES = ((8, 128, 0, 3), (8, 64, 0, 3), (8, 32, 0, 3), (8, 16, 0, 3), (4, 64, 0, 4), (4, 32, 0, 4),
                   (16, 128, 0, 3), (16, 64, 0, 3), (16, 32, 0, 3), (16, 16, 0, 3), (8, 64, 0, 4))


def tune_cache_path():
    return os.environ.get("FDTD_TUNE_CACHE",
                          os.path.join(os.path.dirname(os.path.abspath(__file__)), "_tune_cache.json"))


class BatchSolver:
    """solvers: YeeSolver instances on one device, all at the same step."""

    def __init__(self, solvers, tile=None):
        self.solvers = list(solvers)
        if not self.solvers:
            raise ValueError("BatchSolver needs at least one grid")
        s0 = self.solvers[0]
        self.device = s0.device
        for s in self.solvers:
            if s.device != self.device:
                raise ValueError("all grids must live on one device")
            if s.tstep != s0.tstep or s.cur != s0.cur:
                raise ValueError("all grids must be at the same step")
        self.tile = tile
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device)
        nbytes = N.lib().fdtd_batch_workspace_bytes(len(self.solvers))
        # 64-byte aligned by the caching allocator (it hands out 512-byte blocks)
        self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        self._plan = None
        self._graphs = {}

    @classmethod
    def from_workloads(cls, works, tile=None, device="cuda"):
        from . import configs
        solvers = []
        for w in works:
            ce = configs.ce_from_spheres(w.shape, w.spheres, device=device)
            solvers.append(YeeSolver(w.shape, ce=ce, npml=w.npml, sources=w.source_list(), device=device))
        return cls(solvers, tile=tile)

    @property
    def tstep(self):
        return self.solvers[0].tstep

    @property
    def cur(self):
        return self.solvers[0].cur

    @property
    def cells(self):
        return sum(s.shape[0] * s.shape[1] * s.shape[2] for s in self.solvers)

    # ------------------------------------------------------------------ plan
    def plan(self):
        if self._plan is None:
            n = len(self.solvers)
            grids = (N.Grid * n)(*[s.grid() for s in self.solvers])
            states = (N.YeeState * n)(*[s._state_struct() for s in self.solvers])
            cpmls = (N.Cpml * n)(*[s.cpml.struct() for s in self.solvers])
            srcs = (N.Sources * n)(*[s.sources.struct() for s in self.solvers])
            tile = N.Tile(*(tuple(self.tile or ()) + (0, 0, 0, 0, 0))[:5])
            h = C.c_void_p()
            # the workspace is rewritten on the current stream, after the launches
            # queued on it that may still read it
            with torch.cuda.device(self.device):
                stream = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
                N.call("fdtd_batch_plan_create", C.byref(h), n, grids, states, cpmls, srcs, C.byref(tile),
                       C.c_void_p(self.status.data_ptr()), C.c_void_p(self.workspace.data_ptr()),
                       self.workspace.numel(), self.cur, stream)
            self._plan = h
        return self._plan

    def plan_info(self):
        info = (C.c_int32 * 6)()
        N.call("fdtd_batch_plan_info", self.plan(), info, 6)
        return dict(zip(("tile_y", "stages", "items", "ctas", "threads", "smem_bytes"), list(info)))

    def _advance(self, n):
        for s in self.solvers:
            s.tstep += n
            if n % 2:
                s.cur = 1 - s.cur

    def step(self, n=1):
        """Advance every grid n steps (n launches on the current stream)."""
        plan = self.plan()
        L = N.lib()
        L.fdtd_batch_plan_set_current(plan, self.cur)
        with torch.cuda.device(self.device):
            stream = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
            N.call("fdtd_batch_plan_run", plan, int(self.tstep), int(n), stream)
        self._advance(n)

    def capture(self, n):
        """A CUDA graph of n steps starting at the current step and buffer.
        Replaying it repeats steps tstep..tstep+n-1 (source times included)."""
        plan = self.plan()
        key = (self.tstep, self.cur, n)
        g = self._graphs.get(key)
        if g is None:
            L = N.lib()
            side = torch.cuda.Stream(self.device)
            side.wait_stream(torch.cuda.current_stream(self.device))
            g = torch.cuda.CUDAGraph()
            with torch.cuda.device(self.device), torch.cuda.stream(side):
                L.fdtd_batch_plan_set_current(plan, self.cur)
                with torch.cuda.graph(g, stream=side):
                    N.call("fdtd_batch_plan_run", plan, int(self.tstep), int(n),
                           C.c_void_p(side.cuda_stream))
            torch.cuda.current_stream(self.device).wait_stream(side)
            self._graphs[key] = g
        return g

    def run_graph(self, n):
        """Advance n steps as one graph launch (captured on first use)."""
        g = self.capture(n)
        g.replay()
        self._advance(n)

    def check_status(self):
        v = int(self.status.item())
        if v:
            self.status.zero_()
            N.check(v, "fdtd_batch_plan_run (device status)")

    # --------------------------------------------------------------- autotune
    def signature(self):
        dev = torch.cuda.get_device_name(self.device)
        shapes = ";".join("%dx%dx%d/%d" % (s.shape + (max(s.cpml.npml),)) for s in self.solvers)
        return "%s|%s" % (dev, shapes)

    def _snapshot(self):
        out = []
        for s in self.solvers:
            t = [s._state.clone()]
            t += [p.clone() if p is not None else None for b in range(2) for p in s.cpml.psi_e[b]]
            t += [p.clone() if p is not None else None for p in s.cpml.psi_h]
            out.append((t, s.tstep, s.cur))
        return out

    def _restore(self, snap):
        for s, (t, tstep, cur) in zip(self.solvers, snap):
            s._state.copy_(t[0])
            k = 1
            for b in range(2):
                for q in range(6):
                    if t[k] is not None:
                        s.cpml.psi_e[b][q].copy_(t[k])
                    k += 1
            for q in range(6):
                if t[k] is not None:
                    s.cpml.psi_h[q].copy_(t[k])
                k += 1
            s.tstep, s.cur = tstep, cur

    def autotune(self, candidates=TILE_CANDIDATES, steps=6, use_cache=True):
        """Time each candidate launch shape on this batch and keep the fastest.
        Grid state is saved before and restored after; results are cached per
        device name and grid set."""
        path = tune_cache_path()
        key = self.signature()
        cache = {}
        if use_cache and os.path.exists(path):
            try:
                with open(path) as fh:
                    cache = json.load(fh)
            except (OSError, ValueError):
                cache = {}
        if use_cache and key in cache:
            self._set_tile(tuple(cache[key]["tile"]))
            return cache[key]
        snap = self._snapshot()
        results = []
        stream = torch.cuda.current_stream(self.device)
        for cand in candidates:
            try:
                self._set_tile(tuple(cand))
                self.plan()
            except (ValueError, NotImplementedError, N.FdtdError):
                continue
            self.step(2)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            self.step(steps)
            b.record(stream)
            b.synchronize()
            results.append((a.elapsed_time(b) / steps, tuple(cand)))
        self._restore(snap)
        torch.cuda.synchronize(self.device)
        self.check_status()
        if not results:
            raise RuntimeError("no launch shape could be planned for this batch")
        best_ms, best = min(results)
        self._set_tile(best)
        entry = {"tile": list(best), "ms_per_step": best_ms,
                 "tried": [[list(c), ms] for ms, c in results]}
        if use_cache:
            cache[key] = entry
            try:
                with open(path, "w") as fh:
                    json.dump(cache, fh, indent=1)
            except OSError:
                pass
        return entry

    def _set_tile(self, tile):
        tile = tuple(tile) if tile else None
        if tile != (tuple(self.tile) if self.tile else None):
            self.close()
            self.tile = tile

    def close(self):
        if self._plan is not None:
            N.lib().fdtd_batch_plan_destroy(self._plan)
            self._plan = None
        self._graphs = {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
