"""Recipe: compile pieces of the reference's own CPU code into oracle/_ref/.

Test infrastructure only.  Runs where the reference checkout is present
(FDTD_REFERENCE_ROOT, else the checkout location this recipe names in REF)
and the host is x86_64 (the reference's C uses SSE intrinsics).  Nothing is copied into the repository:
sources are read in place and every artefact lands in oracle/_ref/
(git-ignored).

Artefacts
  kemp_core_<coeff>_pad<p>.so   KEMP/v0.7_pml/fdtd3d/cpu/src/core.c after the
                                macro substitution that
                                KEMP/v0.7_pml/fdtd3d/cpu/core.py:52-87 performs
                                (single precision, OpenMP), compiled with the
                                flags of util/common_cpu.py:73.
  ref_cpml_non_kappa*.so        kuFDTD/v0.2.0/dim3/cpu/core/cpml_non_kappa.c
                                (Python extension, Py3 init shim).
  ref_symp_dielectric*.so       4th_order-Symplectic/Python-C/dielectric.c
                                (Python extension, Py3 init shim).
  ref_drude_ade*.so             kuFDTD/v0.2.0/dim3/cpu/core/drude_ade.c
                                (Python extension, Py3 init shim).
  ref_cpml_core*.so             kuFDTD/before_CUDA/v0.3.0/boundary/core/cpml_core.c
                                (the kappa CPML, Python extension, Py3 init shim).
"""
import os
import platform
import subprocess
import sys
import sysconfig
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# the reference checkout: FDTD_REFERENCE_ROOT, else where this build recipe reads it
REF = os.environ.get("FDTD_REFERENCE_ROOT", "/root/reference")

KEMP_SRC = "KEMP/v0.7_pml/fdtd3d/cpu/src/core.c"
KUFDTD_CPML = "kuFDTD/v0.2.0/dim3/cpu/core/cpml_non_kappa.c"
KUFDTD_INC = "kuFDTD/v0.2.0/dim3/cpu/core"
SYMP_SRC = "4th_order-Symplectic/Python-C/dielectric.c"
KUFDTD_DRUDE = "kuFDTD/v0.2.0/dim3/cpu/core/drude_ade.c"
KUFDTD_KAPPA = "kuFDTD/before_CUDA/v0.3.0/boundary/core/cpml_core.c"
KUFDTD_KAPPA_INC = "kuFDTD/before_CUDA/v0.3.0/boundary/core"


def available():
    return os.path.isdir(REF) and platform.machine() in ("x86_64", "AMD64")


def _kemp_source(coeff_use, pad):
    """Macro substitution in the order of KEMP cpu/core.py:161-189."""
    align = 4
    mask0 = [1] * align
    mask_h = list(mask0)
    mask_h[0] = 0
    mask_exy = list(mask0)
    for q in range(1, pad + 2):
        mask_exy[-q] = 0
    mask = list(mask0)
    for q in range(1, pad + 1):
        mask[-q] = 0
    fmt = lambda m: ", ".join(str(v) for v in m)
    macros = ["OMP_HEADER", "OMP_FOR_E", "OMP_FOR_H",
              "ARGS_CE", "INIT_CE", "PRIVATE_CE", "CEX", "CEY", "CEZ",
              "ARGS_CH", "INIT_CH", "PRIVATE_CH", "CHX", "CHY", "CHZ",
              "DTYPE", "MM_HEADER", "PSD", "TYPE128", "INCRE",
              "MASK_H", "MASK_EXY", "MASK"]
    values = ["#include <omp.h>",
              "#pragma omp parallel for private(idx, i, j, k, hx0, hy0, hz0, h1, h2, e PRIVATE_CE)",
              "#pragma omp parallel for private(idx, i, j, k, ex0, ey0, ez0, e1, e2, h PRIVATE_CH)",
              "", "ce=SET1(0.5)", "", "", "", "",
              "", "ch=SET1(0.5)", "", "", "", "",
              "float", "xmmintrin.h", "ps", "__m128", "4",
              fmt(mask_h), fmt(mask_exy), fmt(mask)]
    if "e" in coeff_use:
        values[3:9] = [", DTYPE *cex, DTYPE *cey, DTYPE *cez", "ce", ", ce",
                       "ce = LOAD(cex+idx);", "ce = LOAD(cey+idx);", "ce = LOAD(cez+idx);"]
    if "h" in coeff_use:
        values[9:15] = [", DTYPE *chx, DTYPE *chy, DTYPE *chz", "ch", ", ch",
                        "ch = LOAD(chx+idx);", "ch = LOAD(chy+idx);", "ch = LOAD(chz+idx);"]
    src = open(os.path.join(REF, KEMP_SRC)).read()
    for old, new in zip(macros, values):
        src = src.replace(old, new)
    return src


def kemp_lib_path(coeff_use, pad):
    return os.path.join(OUT, "kemp_core_%s_pad%d.so" % (coeff_use or "none", pad))


def _ext_suffix():
    return sysconfig.get_config_var("EXT_SUFFIX")


def build(verbose=False):
    if not available():
        return False
    import numpy as np
    os.makedirs(OUT, exist_ok=True)
    jobs = []
    tmp = tempfile.mkdtemp(prefix="fdtd_ref_")  # substituted sources stay outside the repo
    for coeff_use in ("", "eh"):
        for pad in range(4):
            cfile = os.path.join(tmp, "kemp_core_%s_pad%d.c" % (coeff_use or "none", pad))
            with open(cfile, "w") as fh:
                fh.write(_kemp_source(coeff_use, pad))
            jobs.append(["gcc", "-O3", "-std=c99", "-fpic", "-shared", "-fopenmp", "-msse",
                         cfile, "-o", kemp_lib_path(coeff_use, pad)])
    pyinc = sysconfig.get_paths()["include"]
    npinc = np.get_include()
    shim = os.path.join(HERE, "ref_pymod_shim.c")
    for name, src, old_init, extra in (
            ("ref_cpml_non_kappa", KUFDTD_CPML, "initcpml_non_kappa", ["-I" + os.path.join(REF, KUFDTD_INC)]),
            ("ref_symp_dielectric", SYMP_SRC, "initdielectric", []),
            ("ref_drude_ade", KUFDTD_DRUDE, "initdrude_ade", ["-I" + os.path.join(REF, KUFDTD_INC)]),
            ("ref_cpml_core", KUFDTD_KAPPA, "initcpml_core", ["-I" + os.path.join(REF, KUFDTD_KAPPA_INC)])):
        jobs.append(["gcc", "-O2", "-fPIC", "-shared", "-w", "-I" + pyinc, "-I" + npinc, *extra,
                     '-DREF_SRC="%s"' % os.path.join(REF, src),
                     '-DSHIM_NAME="%s"' % name, "-DSHIM_INIT=PyInit_" + name,
                     "-DSHIM_OLD_INIT=" + old_init,
                     shim, "-o", os.path.join(OUT, name + _ext_suffix())])
    procs = []
    for cmd in jobs:
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd, stderr=subprocess.PIPE)))
    for cmd, p in procs:
        _, err = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("reference build failed: %s\n%s" % (" ".join(cmd), err.decode()))
    return True


if __name__ == "__main__":
    ok = build(verbose=True)
    print("built" if ok else "reference not available here")
    sys.exit(0)
