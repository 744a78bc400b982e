"""In-tree build of libfdtd_gb300.so (sm_103a) with nvcc.

Each csrc/*.cu translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a -lineinfo --fmad=false`` (no
multiply-add contraction anywhere: every kernel reproduces the separately
rounded products and sums of the reference's FP32 arithmetic); the objects are
linked into fdtd_accelerate_gb300/libfdtd_gb300.so next to this file.
Object files live in fdtd_accelerate_gb300/_build/.  A unit is rebuilt
when it or any header is newer than its object.  build(check=True) makes the
bounds-checked debug build (-DFDTD_CHECK) as libfdtd_gb300_check.so, objects
in _build_check/.
"""
import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libfdtd_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC,-O2",
              "-I" + os.path.join(ROOT, "include"), "--expt-relaxed-constexpr"]


def nvcc():
    path = shutil.which("nvcc")
    if path:
        return path
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfdtd_gb300.so")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_flags=(), check=False):
    build_dir = BUILD + "_check" if check else BUILD
    lib = LIB[:-3] + "_check.so" if check else LIB
    if check:
        extra_flags = tuple(extra_flags) + ("-DFDTD_CHECK",)
    os.makedirs(build_dir, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdrs = _headers()
    jobs = []
    objs = []
    for src in srcs:
        obj = os.path.join(build_dir, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append([nvcc(), *ARCH, *NVCC_FLAGS, *extra_flags, "-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), p.stderr))
        if verbose and p.stderr.strip():
            print(p.stderr)
        return p

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(lib, objs):
        tmp = lib + ".tmp"
        run([nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-ldl", "-o", tmp])
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, check="--check" in sys.argv))
