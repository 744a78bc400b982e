"""Benchmark: Yee+CPML time step, 1024 x 1024 x 512 cells, 12-cell CPML on
all faces, 200 seeded dielectric spheres, 6 Gaussian dipoles (FP32).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one fused kernel launch advancing the whole grid by one time
step (E + E-CPML + sources + H + H-CPML).  The state (33 GB) is far larger
than L2, so no flush is needed between steps.  Prints one JSON line.

--impl reference times the reference's CPU path on the host cores: the
reference's own C cannot be built on the benchmark host (SSE intrinsics,
Python-2 extension API), so the C oracle -- a line-by-line restatement of
the reference's CPU arithmetic, OpenMP over all host threads -- stands in
(kind "port"), on a bounded sample of the same workload.

N > 1: the path has no exchange step on one GPU per box (replicas only);
each rank runs an independent replica and `value` sums over ranks.
"""
import argparse
import json
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
# DRAM bytes per cell-step of the fused kernel from an ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum over one launch / cells);
# see profiles/k_yee_fused_cpml1024.md (512x512x256 capture of the same workload,
# scaled by cells: an upper bound at full size, where the CPML fraction is smaller).
NCU_DRAM_BYTES_PER_CELL = 81.4


def algorithmic_bytes_per_step(shape, npml):
    """Compulsory FP32 traffic of one step: every field read+written once
    (6 x 8 B), every E coefficient read once (3 x 4 B), every psi value read
    and written once (4 psi arrays per slab cell, 8 B each)."""
    nx, ny, nz = shape
    cells = nx * ny * nz
    slab_cells = 2 * npml * (ny * nz + nx * nz + nx * ny) if npml else 0
    return cells * 60 + slab_cells * 32


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


def cpu_oracle_sample(seconds=12.0, sample_shape=(256, 1024, 512)):
    """Time the oracle (reference CPU arithmetic, OpenMP) on a bounded sample."""
    import oracle
    from fdtd_accelerate_gb300 import configs
    work = configs.scaled(configs.cpml1024(steps=4), sample_shape, steps=4)
    ce = [c.numpy() for c in configs.ce_from_spheres(sample_shape, work.spheres)]
    tables = [oracle.cpml_tables(NPML) for _ in range(3)]
    tab = {k: [t[k] for t in tables] for k in tables[0]}
    f = {k: np.zeros(sample_shape, np.float32) for k in ("ex", "ey", "ez", "hx", "hy", "hz")}
    f.update(cex=ce[0], cey=ce[1], cez=ce[2])
    srcs = [(c, ijk, a.astype(np.float32)) for c, ijk, a in work.source_list(1000)]
    sim = oracle.OracleSim(f, (NPML,) * 3, 0x3F, tab, srcs)
    sim.tstep = 150
    sim.step(1)  # warm-up (page faults, thread pool)
    steps = 0
    t0 = time.perf_counter()
    while True:
        sim.step(1)
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds or steps >= 2000:
            break
    cells = int(np.prod(sample_shape))
    return {"value": cells * steps / el / 1e6, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": "oracle (C restatement of the reference CPU path, OpenMP %d threads) on a %dx%dx%d "
                      "scaled copy of the workload, %d steps, %.1f s" % (os.cpu_count(), *sample_shape, steps, el)}


def run_reference(args, rank, world):
    if rank != 0:
        return
    base = cpu_oracle_sample(seconds=max(3.0, min(20.0, 2.0 * args.steps)))
    line = {"metric": METRIC, "value": base["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded spheres/dipoles)", "impl": "reference",
            "config": {"workload": "Yee+CPML %dx%dx%d, 12-cell CPML, 200 spheres, 6 dipoles (bounded CPU sample)"
                                   % SHAPE},
            "cpu_baseline": base,
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
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
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
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        solver.load_host(host_f, host_ce)
        solver.step(args.steps)
        solver.store_host(host_f)
        e1.record(stream)
        torch.cuda.synchronize()
        solver.check_status()
        e_ms = e0.elapsed_time(e1)
        h2d = 9 * cells * 4
        d2h = 6 * cells * 4
        e2e = {"value": cells * args.steps * world / (e_ms / 1e3) / 1e6, "unit": UNIT,
               "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
               "note": "one public-API run of %d steps: H2D of fields+coefficients from pinned host "
                       "memory, %d fused steps, D2H of the fields" % (args.steps, args.steps)}
        del host_f, host_ce

    if rank != 0:
        return
    alg = algorithmic_bytes_per_step(shape, NPML)
    avg_launch_s = statistics.mean(per_launch_ms) / 1e3
    peak, peak_src = measured_peak()
    achieved = alg / avg_launch_s / 1e9
    traffic = None if NCU_DRAM_BYTES_PER_CELL is None else NCU_DRAM_BYTES_PER_CELL * cells
    if shape != SHAPE:
        line_note = "scaled workload %dx%dx%d (not the headline size)" % tuple(shape)
    else:
        line_note = None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded spheres and dipoles, normalised units)",
        "config": {"workload": "Yee+CPML %dx%dx%d, 12-cell CPML (m=4, R=1e-8, kappa_max=5, alpha_max=0.05), "
                               "200 spheres eps_r U[1,12], 6 Gaussian dipoles" % tuple(shape),
                   "cells": cells, "l2": "state 33 GB >> L2 (no flush needed)",
                   "kernel": "k_yee_fused (TMA 3-D boxes, ping-pong state)",
                   "tile": solver.plan_info(),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "alg_bytes_per_launch": alg, "peak_source": peak_src,
                     "avg_launch_ms": avg_launch_s * 1e3},
        "clocks": clocks,
        "e2e": e2e,
        "gpu_launches": args.steps,
    }
    if line_note:
        line["config"]["note"] = line_note
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_oracle_sample(seconds=args.cpu_seconds)
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--shape", type=lambda s: tuple(int(v) for v in s.split(",")), default=SHAPE,
                    help="grid (default 1024,1024,512); other sizes scale the same workload")
    ap.add_argument("--tile", type=lambda s: tuple(int(v) for v in s.split(",")), default=None)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
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
