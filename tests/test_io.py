"""File formats around the time step: the time_evol.dat writer (Fortran
(20e20.12), src/Case-TGV.f90:375-377), the .i3d namelist reader
(src/parameters.f90) and restart files (src/tools.f90:205-514)."""
import os

import numpy as np
import pytest

from incompact3d_gb300 import io as x3dio

HERE = os.path.dirname(os.path.abspath(__file__))


def test_fortran_e_matches_reference_rows():
    # the reference's own file is re-printed byte for byte from its numbers
    gold = np.loadtxt(os.path.join(HERE, "golden", "tgv_freeslip65_rk3_fp64.txt"))
    row = x3dio.format_time_evol_row(gold[0])
    assert row == ("  0.450000000000E-01  0.124976562661E+00  0.468784149986E-03"
                   "  0.468784149990E-03  0.375027319989E+00")
    assert len(row) == 100


@pytest.mark.parametrize("v,w,d,out", [
    (0.0, 20, 12, "  0.000000000000E+00"),
    (-1.5, 20, 12, " -0.150000000000E+01"),
    (9.9999999999996, 20, 12, "  0.100000000000E+02"),
    (1.23456789e-105, 14, 6, "  0.123457-104"),
    (0.5, 14, 6, "  0.500000E+00"),
])
def test_fortran_e_cases(v, w, d, out):
    assert x3dio.fortran_e(v, w, d) == out


I3D = """
&BasicParam
itype = 3
nx=32 ; ny=33
nz=16                 ! z nodes
istret = 2            ! refinement
beta = 0.259065151
xlx = 8.  , yly = 2., zlz = 3.
nclx1 = 0
nclxn = 0
ncly1 = 2
nclyn = 2
nclz1 = 0
nclzn = 0
re  = 4200.
dt = 0.005
ifirst = 1
ilast = 100
ilesmod=1
cpg = F
/End
&NumOptions
ifirstder = 4
isecondder = 5
itimescheme = 5
nu0nu = 4.0
cnu = 0.44
/End
&LESModel
jles = 3
maxdsmagcst = 0.25
/End
&Statistics
wrotation = 0.12
spinup_time = 5000
/End
"""


def test_read_namelist_and_case():
    g = x3dio.read_namelist(I3D.replace(" ; ", "\n"))
    assert g["basicparam"]["cpg"] is False and g["basicparam"]["xlx"] == 8.0
    case = x3dio.case_from_i3d(I3D.replace(" ; ", "\n"))
    c = case["context"]
    assert (c["nx"], c["ny"], c["nz"]) == (32, 33, 16)
    assert c["bc"] == ((0, 0), (2, 2), (0, 0)) and c["istret"] == 2 and c["isecondder"] == 5
    assert case["solver"] == {"dt": 0.005, "xnu": 1 / 4200.0, "itimescheme": 5}
    assert case["itype"] == x3dio.ITYPE_CHANNEL
    assert case["les"] == (3, 0.15, 0.25)
    assert case["channel"] == (0.12, 5000)


@pytest.mark.gpu
def test_restart_round_trip(gpu_lib, tmp_path):
    L = 2 * np.pi
    c = gpu_lib.Context(32, 32, 32, L, L, L)
    a = gpu_lib.Solver(c, 0.005, 1 / 1600.0, itimescheme=3, precision=gpu_lib.PREC_FP64)
    a.init_tgv()
    a.step(5)
    x3dio.write_restart(str(tmp_path), a, 5 * 0.005, a.itime)
    a.step(5)
    ref = a.get_velocity()
    b = gpu_lib.Solver(c, 0.005, 1 / 1600.0, itimescheme=3, precision=gpu_lib.PREC_FP64)
    t, it = x3dio.read_restart(str(tmp_path), b)
    assert it == 5 and abs(t - 0.025) < 1e-12
    b.step(5)
    for u, v in zip(b.get_velocity(), ref):
        assert np.array_equal(u, v)
