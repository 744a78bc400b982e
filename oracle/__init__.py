"""CPU oracle for the Yee time step: TEST INFRASTRUCTURE, not product code.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package.  It restates the reference's CPU
arithmetic (see fdtd_oracle.c for the file:line citations) in C, FP32 and
FP64, and runs the canonical step order of the reference:

    update_e -> cpml_e -> source -> update_h -> cpml_h

(2nd_order-Yee/CUDA/fdtd3d_201_250x250x320cell_15npml_100000tstep.cu:718-742,
kuFDTD/v0.2.0/dim3/cpu/test/021-dielectric-cpml.py:72-80).
"""
from .oracle import *  # noqa: F401,F403
