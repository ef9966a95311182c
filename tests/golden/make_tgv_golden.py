"""Generate the TGV golden fixtures from the reference's own test data.

Source (read here, in the build container; not available on the GPU machine):
  tests/TGV-Taylor-Green-vortex/reference_time_evol.dat         (FP64 build)
  tests/TGV-Taylor-Green-vortex/reference_time_evol_single.dat  (FP32 build)
of the reference repository: 65^3 free-slip (ncl=1) Taylor-Green vortex on
[0, pi]^3, Re=1600, RK3, dt=0.005, 500 steps, one row every 10 steps with
columns (t, E_k, eps, eps2, enstrophy) (src/Case-TGV.f90:375-377).

Written: tgv_freeslip65_rk3_fp64.txt and tgv_freeslip65_rk3_fp32.txt (the same
numbers, re-printed with full precision).
"""
import os
import sys

import numpy as np

SRC = sys.argv[1] if len(sys.argv) > 1 else "/root/reference/tests/TGV-Taylor-Green-vortex"
HERE = os.path.dirname(os.path.abspath(__file__))

for name, out in (("reference_time_evol.dat", "tgv_freeslip65_rk3_fp64.txt"),
                  ("reference_time_evol_single.dat", "tgv_freeslip65_rk3_fp32.txt")):
    a = np.loadtxt(os.path.join(SRC, name))
    assert a.shape == (50, 5)
    np.savetxt(os.path.join(HERE, out), a, fmt="%.17e",
               header="t E_k eps eps2 enstrophy  (from %s)" % name)
    print(out, a.shape)
