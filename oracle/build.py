"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/fdtd_oracle.c twice (REAL=float and REAL=double) into
oracle/_build/.  Plain gcc + OpenMP, no ISA-specific flags, and
-ffp-contract=off so that x86_64 and aarch64 hosts round identically.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "fdtd_oracle.c")

VARIANTS = {
    "f32": ["-DREAL=float", "-DSFX=_f32"],
    "f64": ["-DREAL=double", "-DSFX=_f64"],
}


def lib_path(kind):
    return os.path.join(OUT, "liboracle_%s.so" % kind)


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    procs = []
    for kind, defs in VARIANTS.items():
        out = lib_path(kind)
        if (not force and os.path.exists(out)
                and os.path.getmtime(out) >= os.path.getmtime(SRC)):
            continue
        cmd = ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp",
               "-ffp-contract=off", "-fno-fast-math", *defs, SRC, "-o", out + ".tmp"]
        if verbose:
            print(" ".join(cmd))
        procs.append((out, subprocess.Popen(cmd, stderr=subprocess.PIPE)))
    for out, p in procs:
        _, err = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + err.decode())
        os.replace(out + ".tmp", out)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
