"""Benchmark: Yee+CPML time step, 1024 x 1024 x 512 cells, 12-cell CPML on
all faces, 200 seeded dielectric spheres, 6 Gaussian dipoles (FP32).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step advances the whole grid by one time step (E + E-CPML + sources +
H + H-CPML): the fused kernel plus the two z-band kernels that finish the
z-slab CPML.  The state (33 GB) is far larger than L2, so no flush is needed
between steps.  Prints one JSON line.

Other workloads (each prints its own line; the default is the headline):
  --workload plain128    128^3 PEC vacuum, 1000 steps, plus the error against
                         the FP64 oracle after those steps
  --workload symp512     4th-order symplectic 512^3, 10-cell CPML, eps U[1,4]
  --workload batched64   64 ragged grids, 500 steps, one graph launch, against
                         64 sequential single-grid solves
  --workload adjoint256  gradient run at 256x256x128, 3000 steps: backward /
                         forward cost and central differences at 32 cells
  --workload drude512    512^3 with a 256^3 Drude (ADE) box, 12-cell CPML,
                         beside the same grid without it
  --workload tfsf512     512^3 with a TFSF plane wave on the box 64..447,
                         12-cell CPML, beside the same grid without it

--impl reference times the reference's CPU path on the host cores: the
reference's own C cannot be built on the benchmark host (SSE intrinsics,
Python-2 extension API), so the C oracle -- a line-by-line restatement of
the reference's CPU arithmetic, OpenMP over all host threads -- stands in
(kind "port"), on the same 1024 x 1024 x 512 workload (W untimed and K timed
steps; a 256-plane slice only when the host lacks memory for the full grid).

N > 1: the path has no exchange step on one GPU per box (replicas only);
each rank runs an independent replica and `value` sums over ranks.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcell-updates/s (Yee+CPML 1024x1024x512, 12-cell CPML, FP32)"
UNIT = "Mcells/s"
SHAPE = (1024, 1024, 512)
NPML = 12
# Measured STREAM-style copy bandwidth of this machine's GB300 (GB/s); read
# from MEASURED_PEAKS.json when present.
FALLBACK_HBM_GBS = 6790.7
# DRAM traffic of one time step (dram__bytes_read.sum + dram__bytes_write.sum),
# from an ncu capture of the same workload scaled to 512x512x256 (three steps,
# the per-launch values agree to 0.2 %), scaled to another size by the units
# each kernel processes: the fused kernel's bytes per grid cell, and the two
# z-band kernels' bytes per band cell (nx * ny * 2P z-slab E nodes).
NCU_FUSED_DRAM_BYTES_PER_CELL = 63.48
NCU_BAND_DRAM_BYTES_PER_BAND_CELL = 193.0
# The plain 128^3 step (one fused launch, no CPML): DRAM bytes of one launch
# after an L2 flush, from an ncu capture of that workload (three launches,
# within 2 %); part of the 50 MB of field writes is still in L2 when the
# launch ends, so the write count is low.
NCU_PLAIN128_DRAM_BYTES = 92.9e6


def step_traffic_bytes(shape, npml):
    nx, ny, nz = shape
    return NCU_FUSED_DRAM_BYTES_PER_CELL * nx * ny * nz + NCU_BAND_DRAM_BYTES_PER_BAND_CELL * nx * ny * 2 * npml


def algorithmic_bytes_per_step(shape, npml):
    """Compulsory FP32 traffic of one step: every field read+written once
    (6 x 8 B), every E coefficient read once (3 x 4 B), every psi value read
    and written once (4 psi arrays per slab cell, 8 B each)."""
    nx, ny, nz = shape
    cells = nx * ny * nz
    slab_cells = 2 * npml * (ny * nz + nx * nz + nx * ny) if npml else 0
    return cells * 60 + slab_cells * 32


def symplectic_pair_bytes_per_step(shape, npml):
    """FP32 traffic of one 4th-order step taken as four fused stage-pair passes
    (each H stage with the E stage after it: fields read and written, E
    coefficients read = 60 B/cell; the closing H stage of a step merged into the
    next pass), plus per pass two E psi and two H psi values read and written
    on every slab cell (32 B x 4)."""
    nx, ny, nz = shape
    cells = nx * ny * nz
    slab_cells = 2 * npml * (ny * nz + nx * nz + nx * ny) if npml else 0
    return cells * 4 * 60 + slab_cells * 4 * 32


def symplectic_bytes_per_step(shape, npml):
    """Algorithmic FP32 traffic of one 4th-order symplectic step taken stage by
    stage (5 H stages: E read, H read+written = 36 B/cell; 4 E stages: H read,
    E read+written, CE read = 48 B/cell; 372 B/cell), plus per stage two psi
    values read and written on every slab cell (16 B x 9 stages)."""
    nx, ny, nz = shape
    cells = nx * ny * nz
    slab_cells = 2 * npml * (ny * nz + nx * nz + nx * ny) if npml else 0
    return cells * (5 * 36 + 4 * 48) + slab_cells * 9 * 16


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json)"
    except Exception:
        return FALLBACK_HBM_GBS, "measured (pool copy bandwidth, 2026-12-03)"


class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sms, maxes, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                maxes.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sms:
            return None
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": max(maxes), "reasons": sorted(reasons),
                "samples": len(sms)}


def _mem_available_bytes():
    try:
        with open("/proc/meminfo") as fh:
            for line in fh:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return None


def _cpu_sample_shape(shape):
    """The workload's own grid when the host has room for the oracle's state
    (9 field and coefficient arrays, psi slabs, a margin); else a 256-plane
    slice of it."""
    need = 10 * 4 * int(np.prod(shape)) * 1.3
    avail = _mem_available_bytes()
    if avail is None or avail >= need:
        return tuple(shape), False
    return (256,) + tuple(shape[1:]), True


def workload_name(shape):
    return ("Yee+CPML %dx%dx%d, 12-cell CPML (m=4, R=1e-8, kappa_max=5, alpha_max=0.05), "
            "200 spheres eps_r U[1,12], 6 Gaussian dipoles" % tuple(shape))


def cpu_oracle_run(shape=SHAPE, seconds=12.0, warmup=1, steps=None):
    """Time the oracle (the reference's CPU arithmetic restated in C, OpenMP
    over all host threads) on the workload: `warmup` untimed steps, then
    `steps` timed steps, or as many as fit in `seconds` when steps is None."""
    import oracle
    from fdtd_accelerate_gb300 import configs
    sample_shape, sliced = _cpu_sample_shape(shape)
    work = configs.cpml1024(steps=4)
    if sample_shape != SHAPE:
        work = configs.scaled(work, sample_shape, steps=4)
    ce = [c.numpy() for c in configs.ce_from_spheres(sample_shape, work.spheres)]
    tables = [oracle.cpml_tables(NPML) for _ in range(3)]
    tab = {k: [t[k] for t in tables] for k in tables[0]}
    f = {k: np.zeros(sample_shape, np.float32) for k in ("ex", "ey", "ez", "hx", "hy", "hz")}
    f.update(cex=ce[0], cey=ce[1], cez=ce[2])
    del ce
    srcs = [(c, ijk, a.astype(np.float32)) for c, ijk, a in work.source_list(4000)]
    sim = oracle.OracleSim(f, (NPML,) * 3, 0x3F, tab, srcs)
    sim.tstep = 150
    sim.step(max(1, warmup))  # warm-up (page faults, thread pool)
    done = 0
    t0 = time.perf_counter()
    while True:
        sim.step(1)
        done += 1
        el = time.perf_counter() - t0
        if (steps is not None and done >= steps) or (steps is None and (el >= seconds or done >= 2000)):
            break
    cells = int(np.prod(sample_shape))
    what = ("the workload itself (%dx%dx%d)" % sample_shape if not sliced else
            "a %dx%dx%d slice of the workload (host memory short of the full grid)" % sample_shape)
    return {"value": cells * done / el / 1e6, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "ms_per_step": el / done * 1e3, "same_config": not sliced,
            "sample": "oracle (C restatement of the reference CPU path, OpenMP %d threads) on %s, %d steps "
                      "after %d warm-up, %.1f s" % (os.cpu_count(), what, done, max(1, warmup), el)}


def accuracy_summary(errs, steps, what):
    """FP32-vs-FP64 distance of a run (fp64.family_errors output) for a JSON line."""
    return {"steps": steps, "vs": what,
            "max_family_rel": max(e["max"] for e in errs.values()),
            "rms_family_rel": max(e["rms"] for e in errs.values()),
            "per_component": {k: {"max": round(e["max"], 9), "rms": round(e["rms"], 9)} for k, e in errs.items()},
            "metric": "per component: max |fp32 - fp64| / max |fp64| over its field family (E or H), and the "
                      "root-mean-square ratio; the line reports the largest over components"}


def cpml1024_accuracy(shape, steps, dev):
    """The workload run from zero for `steps` steps by the fused FP32 path and by
    the FP64 step on the GPU (FP32 coefficients, tables, amplitudes widened)."""
    import torch
    import fdtd_accelerate_gb300 as F
    from fdtd_accelerate_gb300 import configs
    from fdtd_accelerate_gb300.fp64 import YeeRun64, family_errors
    work = configs.cpml1024(steps=steps, npml=NPML)
    if shape != SHAPE:
        work = configs.scaled(work, shape, steps=steps)
    ce = configs.ce_from_spheres(shape, work.spheres, device=dev)
    src = work.source_list(steps + 2)
    s32 = F.YeeSolver(shape, ce=ce, npml=NPML, sources=src, device=dev)
    s32.step(steps)
    s64 = YeeRun64(shape, ce=ce, npml=NPML, sources=src, device=dev)
    del ce
    s64.step(steps)
    torch.cuda.synchronize()
    s32.check_status()
    errs = family_errors(s32.fields, s64.fields)
    s32.close()
    del s32, s64
    torch.cuda.empty_cache()
    return accuracy_summary(errs, steps, "FP64 step on the GPU (fdtd_step_unfused_f64), same inputs")


def max_over_ranks(x, device):
    """The largest x over the ranks of the default process group (x itself
    without one): whole-job times are the slowest rank's."""
    import torch
    dist = torch.distributed
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, rank, world):
    """The reference's CPU path on the host cores, on the same workload and
    grid as our arm: W untimed steps, then K timed steps."""
    if rank != 0:
        return
    base = cpu_oracle_run(shape=args.shape, warmup=args.warmup, steps=args.steps)
    line = {"metric": METRIC, "value": base["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": base["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded spheres and dipoles, normalised units)", "impl": "reference",
            "config": {"workload": workload_name(args.shape), "cells": int(np.prod(args.shape)),
                       "same_config": base["same_config"]},
            "cpu_baseline": {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world):
    import torch
    import fdtd_accelerate_gb300 as F
    from fdtd_accelerate_gb300 import configs

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    shape = args.shape
    work = configs.cpml1024(steps=args.warmup + args.steps + 2, npml=NPML)
    if shape != SHAPE:
        work = configs.scaled(work, shape)
    ce = configs.ce_from_spheres(shape, work.spheres, device=dev)
    sources = work.source_list(args.warmup + 2 * args.steps + 4)
    solver = F.YeeSolver(shape, ce=ce, npml=NPML, sources=sources, device=dev, tile=args.tile)
    del ce
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(dev)
    info = solver.plan_info()

    for _ in range(args.warmup):
        solver.step(1)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()

    sampler = ClockSampler(dev.index)
    sampler.start()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    torch.cuda.synchronize()
    t_all0 = torch.cuda.Event(enable_timing=True)
    t_all1 = torch.cuda.Event(enable_timing=True)
    t_all0.record(stream)
    for s in range(args.steps):
        starts[s].record(stream)
        solver.step(1)
        ends[s].record(stream)
    t_all1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    solver.check_status()
    total_ms = t_all0.elapsed_time(t_all1)
    per_launch_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_ms = max_over_ranks(total_ms, dev)
    cells = int(np.prod(shape))
    value = cells * args.steps * world / (total_ms / 1e3) / 1e6

    # --- e2e: public API with host buffers (pinned), copies inside the timed region
    e2e = None
    if not args.no_e2e:
        host_f = {k: torch.empty(shape, dtype=torch.float32).pin_memory() for k in F.solver.FIELD_NAMES}
        host_ce = [torch.empty(shape, dtype=torch.float32).pin_memory() for _ in range(3)]
        for k, v in solver.fields.items():
            host_f[k].copy_(v)
        for q in range(3):
            host_ce[q].copy_(solver.ce[q])
        # one untimed pass over the same buffers first: the first DMA from
        # freshly pinned pages also pays for mapping them
        solver.load_host(host_f, host_ce)
        solver.step(1)
        solver.store_host(host_f)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        ev[0].record(stream)
        solver.load_host(host_f, host_ce)
        ev[1].record(stream)
        solver.step(args.steps)
        ev[2].record(stream)
        solver.store_host(host_f)
        ev[3].record(stream)
        torch.cuda.synchronize()
        solver.check_status()
        e_ms = max_over_ranks(ev[0].elapsed_time(ev[3]), dev)
        h2d = 9 * cells * 4
        d2h = 6 * cells * 4
        h2d_ms, run_ms, d2h_ms = (ev[q].elapsed_time(ev[q + 1]) for q in range(3))
        e2e = {"value": cells * args.steps * world / (e_ms / 1e3) / 1e6, "unit": UNIT,
               "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
               "h2d_ms": h2d_ms, "steps_ms": run_ms, "d2h_ms": d2h_ms,
               "h2d_GBs": h2d / (h2d_ms / 1e3) / 1e9, "d2h_GBs": d2h / (d2h_ms / 1e3) / 1e9,
               "note": "one public-API run of %d steps: H2D of fields+coefficients from pinned host "
                       "memory, %d fused steps, D2H of the fields (after one untimed pass over the "
                       "same buffers)" % (args.steps, args.steps)}
        del host_f, host_ce

    accuracy = None
    if args.accuracy_steps and world == 1:
        solver.close()
        del solver
        torch.cuda.empty_cache()
        accuracy = cpml1024_accuracy(shape, args.accuracy_steps, dev)

    if rank != 0:
        return
    alg = algorithmic_bytes_per_step(shape, NPML)
    avg_launch_s = statistics.mean(per_launch_ms) / 1e3
    peak, peak_src = measured_peak()
    achieved = alg / avg_launch_s / 1e9
    traffic = step_traffic_bytes(shape, NPML)
    if shape != SHAPE:
        line_note = "scaled workload %dx%dx%d (not the headline size)" % tuple(shape)
    else:
        line_note = None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded spheres and dipoles, normalised units)",
        "config": {"workload": workload_name(shape),
                   "cells": cells, "l2": "state 33 GB >> L2 (no flush needed)",
                   "kernel": "k_yee_fused (TMA 3-D boxes, ping-pong state)" +
                             (" + k_zband_e + k_zband_h (z-slab CPML)" if info["z_band"] else ""),
                   "tile": info,
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "traffic_source": "ncu dram bytes at 512x512x256, scaled per grid cell (fused kernel) "
                                       "and per z-band cell (band kernels)",
                     "alg_bytes_per_launch": alg, "peak_source": peak_src,
                     "avg_launch_ms": avg_launch_s * 1e3,
                     "scope": "one time step (%d launch%s, timed together with CUDA events)"
                              % (info["launches_per_step"], "es" if info["launches_per_step"] > 1 else "")},
        "clocks": clocks,
        "e2e": e2e,
        "gpu_launches": args.steps * info["launches_per_step"],
    }
    if line_note:
        line["config"]["note"] = line_note
    if accuracy is not None:
        line["accuracy"] = accuracy
    if not args.no_cpu_baseline and world == 1:
        base = cpu_oracle_run(shape=shape, seconds=args.cpu_seconds)
        line["cpu_baseline"] = {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# secondary workloads (one JSON line each; not the headline)
# ---------------------------------------------------------------------------
def _flush_l2(buf):
    """Overwrite a buffer larger than L2 (126 MB) so the next step starts cold."""
    buf.add_(1.0)


def _timed_steps(torch, stream, step, nsteps, flush=None):
    """Per-step CUDA-event times (ms); an L2 flush runs outside each timed step."""
    times = []
    for _ in range(nsteps):
        if flush is not None:
            flush()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step()
        b.record(stream)
        times.append((a, b))
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in times]


def _base_line(metric, value, unit, args, ms, dtype, workload, extra=None):
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded)", "config": {"workload": workload}}
    if extra:
        line.update(extra)
    return line


def run_plain128(args):
    """128^3 PEC vacuum, Ez source at the centre (one fused launch per step)."""
    import torch
    import fdtd_accelerate_gb300 as F
    from fdtd_accelerate_gb300 import configs
    dev = torch.device("cuda", 0)
    w = configs.plain128(steps=max(1000, args.warmup + args.steps + 2))
    s = F.YeeSolver(w.shape, sources=w.source_list(), device=dev, tile=args.tile)
    stream = torch.cuda.current_stream(dev)
    flush_buf = torch.zeros(64 << 20, dtype=torch.float32, device=dev)  # 256 MB > L2
    for _ in range(args.warmup):
        s.step(1)
    sampler = ClockSampler(0)
    sampler.start()
    ms = _timed_steps(torch, stream, lambda: s.step(1), args.steps, lambda: _flush_l2(flush_buf))
    clocks = sampler.stop()
    s.check_status()
    cells = w.cells
    avg = statistics.mean(ms)
    alg = algorithmic_bytes_per_step(w.shape, 0)
    peak, src = measured_peak()
    achieved = alg / (avg / 1e3) / 1e9
    info = s.plan_info()
    line = _base_line("Mcell-updates/s (plain Yee 128^3 PEC, FP32)", cells / (avg / 1e3) / 1e6, UNIT, args, avg,
                      "f32", "plain Yee 128x128x128, PEC walls, vacuum, Ez source at the centre (L2 flushed "
                      "before every timed step)",
                      {"roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                    "frac": achieved / peak,
                                    "traffic": NCU_PLAIN128_DRAM_BYTES if w.shape == (128, 128, 128) else None,
                                    "traffic_source": "ncu dram bytes of one launch of this workload",
                                    "alg_bytes_per_launch": alg, "peak_source": src},
                       "clocks": clocks, "gpu_launches": args.steps * info["launches_per_step"],
                       "accuracy": "bit-exact against the FP32 oracle after 1000 steps; FP32-vs-FP64 floor in "
                                   "tests/test_gpu_accuracy.py"})
    line["config"]["tile"] = info
    print(json.dumps(line), flush=True)


def run_symp512(args):
    """4th-order symplectic, 512^3, 10-cell CPML, 60 spheres eps U[1,4], one dipole."""
    import torch
    import fdtd_accelerate_gb300 as F
    from fdtd_accelerate_gb300 import configs, symplectic
    dev = torch.device("cuda", 0)
    shape, npml = tuple(args.symp_shape), 10
    s = configs.symp512_solver(shape, device=dev, max_steps=args.warmup + args.steps + 2, npml=npml,
                               fused=not args.symp_stages)
    stream = torch.cuda.current_stream(dev)
    s.step(args.warmup)
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    # one run of K steps, as a simulation advances (consecutive steps share a
    # pass: the closing H stage of a step merges with the opening one of the next)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    s.step(args.steps)
    b.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    s.check_status()
    avg = a.elapsed_time(b) / args.steps
    cells = int(np.prod(shape))
    alg = symplectic_bytes_per_step(shape, npml)
    alg_pair = symplectic_pair_bytes_per_step(shape, npml)
    alg_fused = algorithmic_bytes_per_step(shape, npml)
    peak, psrc = measured_peak()
    pair = s.pair_path()
    # the roofline of the path that ran: the stage-pair byte count (four passes
    # of 60 B/cell) or the stage-by-stage one (372 B/cell)
    alg_run = alg_pair if pair else alg
    achieved = alg_run / (avg / 1e3) / 1e9
    # launches: per pass the pair kernel and the shell's H and E kernels, and
    # the run's last H stage; or per step 5 H and 4 E stage launches and a
    # source launch after each E stage
    launches = 4 * args.steps * 3 + 1 if pair else args.steps * (5 + 4 * 2)
    accuracy = None
    if args.accuracy_steps:
        from fdtd_accelerate_gb300.fp64 import SympRun64, family_errors
        del s
        torch.cuda.empty_cache()
        s32 = configs.symp512_solver(shape, device=dev, max_steps=args.accuracy_steps + 2, npml=npml)
        r64 = SympRun64(s32)
        s32.step(args.accuracy_steps)
        r64.step(args.accuracy_steps)
        torch.cuda.synchronize()
        accuracy = accuracy_summary(family_errors(s32.fields, r64.fields), args.accuracy_steps,
                                    "FP64 twin of the stage kernels on the GPU (fdtd_symplectic_stage_f64), same inputs")
        del s32, r64
        torch.cuda.empty_cache()
    line = _base_line("Mcell-updates/s (4th-order symplectic %dx%dx%d, 10-cell CPML, FP32)" % shape, cells / (avg / 1e3) / 1e6,
                      UNIT, args, avg, "f32", "4th-order symplectic %dx%dx%d, 10-cell CPML, 60 spheres eps_r " % shape +
                      "U[1,4], Ez dipole; 4 E + 5 H stages per step, " +
                      ("four stage-pair passes per step (k_symp_pair inside, k_edge_* on the y/z CPML shell) "
                       "in one %d-step run" % args.steps
                       if pair else "one launch per stage with its CPML slabs") +
                      " (6 fields + 3 coefficient arrays: %.1f GB >> L2)" % (9 * cells * 4 / 1e9),
                      {"roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                    "frac": achieved / peak, "traffic": None, "peak_source": psrc,
                                    "alg_bytes_per_launch": alg_run,
                                    "scope": ("one time step on the stage-pair byte count (four passes of "
                                              "60 B/cell + 128 B per slab cell)") if pair else
                                             ("one time step on the stage-by-stage byte count of the workload "
                                              "(372 B/cell + 144 B per slab cell)"),
                                    "frac_of_stage_bytes": alg / (avg / 1e3) / 1e9 / peak,
                                    "stage_bytes_per_step": alg,
                                    "frac_of_pair_pass_bytes": alg_pair / (avg / 1e3) / 1e9 / peak,
                                    "pair_pass_bytes_per_step": alg_pair,
                                    "frac_of_fused_step_bytes": alg_fused / (avg / 1e3) / 1e9 / peak},
                       "clocks": clocks, "gpu_launches": launches})
    if accuracy is not None:
        line["accuracy"] = accuracy
    print(json.dumps(line), flush=True)


def run_drude512(args):
    """512^3 vacuum, 12-cell CPML, a centred 256^3 Drude box (gold-like: eps_inf 9.0685,
    wp dt = 0.075, gamma dt = 0.0019, the parameters of kuFDTD/v0.2.0/dim3/cpu/test/
    030-drude-cpml.py in the step's normalised units), one Ez dipole; the same grid without
    the Drude box is timed beside it."""
    import torch
    import fdtd_accelerate_gb300 as F
    dev = torch.device("cuda", 0)
    shape, npml, box0, box = (512, 512, 512), 12, (128, 128, 128), (256, 256, 256)
    dt = 0.5
    eps_inf, wp, gamma = 9.0685, 0.075 / dt, 0.00192 / dt
    t = np.arange(args.warmup + args.steps + 2, dtype=np.float64)
    src = [("ez", (256, 256, 64), np.sin(2 * np.pi * 0.05 * t) * np.exp(-0.5 * ((t - 150.0) / 30.0) ** 2))]
    stream = torch.cuda.current_stream(dev)
    results = {}
    for with_drude in (False, True):
        ce = torch.full((3,) + shape, 0.5, dtype=torch.float32, device=dev)
        d = None
        if with_drude:
            sl = tuple(slice(o, o + n) for o, n in zip(box0, box))
            ce[(slice(None),) + sl] = float(np.float32(0.5) / np.float32(eps_inf))
            d = F.DrudeAde(shape, box0, box, device=dev)
            d.set_coeff(wp, gamma, dt)
        s = F.YeeSolver(shape, ce=ce, npml=npml, sources=src, device=dev, drude=d, tile=args.tile)
        del ce
        for _ in range(args.warmup):
            s.step(1)
        sampler = ClockSampler(0)
        sampler.start()
        ms = _timed_steps(torch, stream, lambda: s.step(1), args.steps)
        clocks = sampler.stop()
        s.check_status()
        results[with_drude] = (statistics.mean(ms), clocks, s.plan_info())
        s.close()
        del s, d
        torch.cuda.empty_cache()
    avg, clocks, info = results[True]
    cells = int(np.prod(shape))
    dcells = int(np.prod(box))
    alg = algorithmic_bytes_per_step(shape, npml) + dcells * 48
    peak, psrc = measured_peak()
    achieved = alg / (avg / 1e3) / 1e9
    line = _base_line("Mcell-updates/s (Yee+CPML+Drude 512^3, 256^3 Drude box, FP32)", cells / (avg / 1e3) / 1e6,
                      UNIT, args, avg, "f32", "Yee + 12-cell CPML 512x512x512 with a centred 256^3 Drude (ADE) box, "
                      "gold-like parameters, Ez dipole; state 6.4 GB >> L2",
                      {"roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                    "frac": achieved / peak, "traffic": None, "peak_source": psrc,
                                    "alg_bytes_per_launch": alg,
                                    "scope": "one time step: 60 B/cell + 32 B per slab cell + 48 B per Drude "
                                             "cell (J read+written, CJA, CJB read)"},
                       "without_drude_ms_per_step": results[False][0],
                       "clocks": clocks, "gpu_launches": args.steps * info["launches_per_step"]})
    line["config"]["tile"] = info
    print(json.dumps(line), flush=True)


def run_tfsf512(args):
    """512^3 vacuum, 12-cell CPML, a plane wave (TFSF, normal incidence along x,
    wavelength 40 cells, polarisation 0.3 rad) on the box 64..447 in every axis; the
    same grid without the plane wave is timed beside it."""
    import torch
    import fdtd_accelerate_gb300 as F
    dev = torch.device("cuda", 0)
    shape, npml, lo, hi = (512, 512, 512), 12, 64, 447
    stream = torch.cuda.current_stream(dev)
    results = {}
    for with_tfsf in (False, True):
        src = None
        if with_tfsf:
            src = F.Tfsf(shape, (lo,) * 3, (hi,) * 3, wavelength=40.0, propagation_direction=("normal", "x"),
                         polarization_angle=0.3, steps=args.warmup + args.steps + 4, device=dev)
        s = F.YeeSolver(shape, npml=npml, device=dev, tfsf=src, tile=args.tile)
        for _ in range(args.warmup):
            s.step(1)
        sampler = ClockSampler(0)
        sampler.start()
        ms = _timed_steps(torch, stream, lambda: s.step(1), args.steps)
        clocks = sampler.stop()
        s.check_status()
        results[with_tfsf] = (statistics.mean(ms), clocks, s.plan_info())
        s.close()
        del s, src
        torch.cuda.empty_cache()
    avg, clocks, info = results[True]
    cells = int(np.prod(shape))
    side = hi - lo + 2
    face_cells = 6 * side * side
    alg = algorithmic_bytes_per_step(shape, npml) + face_cells * 2 * 2 * 8
    peak, psrc = measured_peak()
    achieved = alg / (avg / 1e3) / 1e9
    line = _base_line("Mcell-updates/s (Yee+CPML+TFSF plane wave 512^3, FP32)", cells / (avg / 1e3) / 1e6,
                      UNIT, args, avg, "f32", "Yee + 12-cell CPML 512x512x512, vacuum, TFSF plane wave on the box "
                      "64..447 (x incidence, wavelength 40 cells); state 6.4 GB >> L2",
                      {"roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                    "frac": achieved / peak, "traffic": None, "peak_source": psrc,
                                    "alg_bytes_per_launch": alg,
                                    "scope": "one time step (fused kernel, band kernels, 1-D grid kernel): "
                                             "60 B/cell + 32 B per slab cell + 16 B per TFSF face cell and half"},
                       "without_tfsf_ms_per_step": results[False][0],
                       "clocks": clocks, "gpu_launches": args.steps * info["launches_per_step"]})
    line["config"]["tile"] = info
    print(json.dumps(line), flush=True)


def run_batched64(args):
    """64 ragged grids in one launch per step (autotuned, graph-captured) against
    the same 64 grids solved one after another with the single-grid path."""
    import torch
    import fdtd_accelerate_gb300 as F
    from fdtd_accelerate_gb300 import configs
    dev = torch.device("cuda", 0)
    works = configs.batched64()
    batch = F.BatchSolver.from_workloads(works, device=dev)
    tune = batch.autotune()
    stream = torch.cuda.current_stream(dev)
    n = args.steps
    for _ in range(args.warmup):
        batch.step(1)
    g = batch.capture(n)
    g.replay()  # first replay outside the timed region
    batch._advance(n)
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    g.replay()
    b.record(stream)
    b.synchronize()
    clocks = sampler.stop()
    batch._advance(n)
    batch.check_status()
    ms_batch = a.elapsed_time(b) / n
    # sequential: each grid alone, one single-grid fused step per launch group
    for sv in batch.solvers:
        sv.step(2)
    torch.cuda.synchronize()
    a.record(stream)
    for sv in batch.solvers:
        sv.step(n)
    b.record(stream)
    b.synchronize()
    ms_seq = a.elapsed_time(b) / n
    cells = batch.cells
    info = batch.plan_info()
    # one step = the batched fused launch plus the two batched z-band launches
    # when any grid has a z face with CPML; bytes summed over the grids
    band = any(sv.cpml.active and sv.cpml.npml[2] > 0 for sv in batch.solvers)
    per_step = 3 if band else 1
    alg = sum(algorithmic_bytes_per_step(sv.shape, sv.cpml.npml[0]) for sv in batch.solvers)
    peak, peak_src = measured_peak()
    achieved = alg / (ms_batch / 1e3) / 1e9
    line = _base_line("Mcell-updates/s (64 ragged Yee+CPML grids, one launch per step, FP32)",
                      cells / (ms_batch / 1e3) / 1e6, UNIT, args, ms_batch, "f32",
                      "64 grids, axes from {32..192 step 16}, 8-cell CPML, 10 spheres eps_r U[1,8] each, Ez "
                      "centre source; %d steps captured in one CUDA graph; %d cells in all" % (n, cells),
                      {"sequential": {"value": cells / (ms_seq / 1e3) / 1e6, "unit": UNIT, "ms_per_step": ms_seq,
                                      "how": "the same 64 grids stepped one after another (single-grid plans)"},
                       "speedup_vs_sequential": ms_seq / ms_batch,
                       "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                    "frac": achieved / peak, "traffic": None, "alg_bytes_per_launch": alg,
                                    "peak_source": peak_src, "avg_launch_ms": ms_batch,
                                    "scope": "one batched step (%d launch%s in the graph, timed together)"
                                             % (per_step, "es" if per_step > 1 else "")},
                       "clocks": clocks, "gpu_launches": n * per_step})
    line["config"]["tile"] = info
    line["config"]["autotune"] = tune
    print(json.dumps(line), flush=True)


def adjoint_launches(nsteps, segment, monitors, cpml):
    """Kernel launches of one forward + backward run of YeeAdjoint: a forward
    step is the fused kernel and the two z-band kernels (CPML on the z faces)
    plus the probe gather; the backward recomputes every segment but the
    last (three launches a step) and runs one reverse step per step (probe
    injection, the two psi-transpose launches, the E and H cell kernels)."""
    fused = 3 if cpml else 1
    last = nsteps - (math.ceil(nsteps / segment) - 1) * segment
    forward = nsteps * (fused + (1 if monitors else 0))
    reverse = nsteps * ((1 if monitors else 0) + (2 if cpml else 0) + 2)
    return forward + (nsteps - last) * fused + reverse


def run_adjoint256(args):
    """Gradient of a probe loss w.r.t. the permittivity of a 128x128x64 design
    region: forward and backward cost, and central differences at 32 cells."""
    import torch
    import fdtd_accelerate_gb300 as F
    from fdtd_accelerate_gb300 import configs
    dev = torch.device("cuda", 0)
    w = configs.adjoint256(steps=args.steps)
    # the gradient the workload asks for: every design-cell eps (dL/dCE is
    # accumulated over the design region only)
    eng = F.YeeAdjoint(w.shape, w.steps, npml=w.npml, sources=w.sources, monitors=w.monitors,
                       segment=w.segment, device=dev, grad_region=w.design)
    eps = w.eps.to(dev)
    stream = torch.cuda.current_stream(dev)

    def ce_of(e):
        return (w.dt / e).float().unsqueeze(0).expand(3, -1, -1, -1).contiguous()

    def loss_of(mon):
        return (mon.double() ** 2).sum()

    times = []
    for rep in range(3):  # rep 0 warms up
        e = eps.clone().requires_grad_(True)
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t2 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        mon, _ = F.fdtd_run(ce_of(e), eng)
        t1.record(stream)
        L = loss_of(mon)
        L.backward()
        t2.record(stream)
        t2.synchronize()
        if rep:
            times.append((t0.elapsed_time(t1), t1.elapsed_time(t2)))
        grad = e.grad.detach()
        L0 = float(L.detach())
    eng.check_status()
    fwd = statistics.mean(t[0] for t in times)
    bwd = statistics.mean(t[1] for t in times)
    # central differences at random design cells: the loss of the same discrete
    # problem evaluated by the FP64 step on the GPU (FP32 forward runs cannot
    # resolve it: the perturbation moves the loss by 1e-7..1e-5 relative)
    from fdtd_accelerate_gb300.fp64 import YeeRun64
    r64 = YeeRun64(w.shape, npml=w.npml, sources=w.sources, monitors=w.monitors, device=dev)
    rng = np.random.default_rng(7)
    cells, errs, g_fd = [], [], []
    h = 1e-3
    ds = w.design
    t_fd = time.perf_counter()
    with torch.no_grad():
        for _ in range(args.fd_cells):
            c = tuple(int(rng.integers(sl.start, sl.stop)) for sl in ds)
            vals = []
            for sgn in (1, -1):
                e2 = eps.clone()
                e2[c] += sgn * h
                r64.set_ce(ce_of(e2))
                vals.append(float((r64.run(w.steps) ** 2).sum()))
            fd = (vals[0] - vals[1]) / (2 * h)
            gc = float(grad[c])
            cells.append(c)
            g_fd.append((gc, fd))
            errs.append(abs(gc - fd) / max(abs(fd), 1e-300))
    gmax = max(abs(f) for _, f in g_fd) if g_fd else 0.0
    norm_err = max(abs(a - b) for a, b in g_fd) / gmax if gmax else None
    nc = int(np.prod(w.shape))
    line = _base_line("adjoint cost: backward time / forward time (gradient run 256x256x128, 3000 steps)",
                      bwd / fwd, "x", args, (fwd + bwd) / w.steps, "f32",
                      w.name + "; loss = sum_t sum_p Ez^2; checkpoints every %d steps" % w.segment,
                      {"higher_is_better": False,
                       "forward": {"ms": fwd, "Mcells_per_s": nc * w.steps / (fwd / 1e3) / 1e6},
                       "backward": {"ms": bwd, "Mcells_per_s": nc * w.steps / (bwd / 1e3) / 1e6,
                                    "what": "segment recompute from checkpoints + reverse-time adjoint steps, "
                                            "dL/dCE accumulated over the 128x128x64 design region"},
                       "gradient_over_forward": (fwd + bwd) / fwd,
                       "fd_check": {"cells": len(cells), "h": h, "loss": L0,
                                    "median_rel_err": float(np.median(errs)) if errs else None,
                                    "max_rel_err": float(max(errs)) if errs else None,
                                    "max_err_over_max_fd": norm_err,
                                    "seconds": time.perf_counter() - t_fd,
                                    "how": "dL/deps from the FP32 adjoint against central differences "
                                           "(h = 1e-3 in eps) of the loss computed by the FP64 step on the GPU "
                                           "(fdtd_step_unfused_f64) for the same FP32-rounded CE"},
                       "gpu_launches": adjoint_launches(w.steps, w.segment, bool(w.monitors), w.npml > 0)})
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 200; plain128 1000, symp512 50, batched64 500, adjoint256 3000, "
                         "drude512 100, tfsf512 100)")
    ap.add_argument("--workload", default="cpml1024",
                    choices=["cpml1024", "plain128", "symp512", "batched64", "adjoint256", "drude512", "tfsf512"])
    ap.add_argument("--fd-cells", type=int, default=32)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--symp-shape", type=lambda s: tuple(int(v) for v in s.split(",")), default=(512, 512, 512),
                    help="grid of --workload symp512 (a smaller one for profiling)")
    ap.add_argument("--symp-stages", action="store_true",
                    help="--workload symp512 on the per-stage kernels instead of the stage-pair path")
    ap.add_argument("--shape", type=lambda s: tuple(int(v) for v in s.split(",")), default=SHAPE,
                    help="grid (default 1024,1024,512); other sizes scale the same workload")
    ap.add_argument("--tile", type=lambda s: tuple(int(v) for v in s.split(",")), default=None)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--accuracy-steps", type=int, default=None,
                    help="steps of the FP32-vs-FP64 accuracy run reported in the line (default: the workload's "
                         "own count, 2000 for cpml1024, 1000 for symp512; 0 skips it)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.accuracy_steps is None:
        args.accuracy_steps = {"cpml1024": 2000, "symp512": 1000}.get(args.workload, 0)
    if args.steps is None:
        args.steps = {"cpml1024": 200, "plain128": 1000, "symp512": 50, "batched64": 500,
                      "adjoint256": 3000, "drude512": 100, "tfsf512": 100}[args.workload]
    if args.workload != "cpml1024":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "workload": args.workload,
                              "unavailable": "the reference arm covers the headline workload only"}), flush=True)
            return
        {"plain128": run_plain128, "symp512": run_symp512, "batched64": run_batched64,
         "adjoint256": run_adjoint256, "drude512": run_drude512, "tfsf512": run_tfsf512}[args.workload](args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.init_process_group("nccl")
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world)
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
