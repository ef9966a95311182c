"""ctypes binding of libx3dgpu.so (the C ABI declared in include/x3d_gpu.h).

The library is built in-tree (incompact3d_gb300/_build/libx3dgpu.so).  There
is no CPU fallback: if the library is missing, loading raises.
"""
import ctypes
import os
import re
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libx3dgpu.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "x3d_gpu.h")

X3D_OK = 0
ERRORS = {
    -1: "X3D_ERR_ARG", -2: "X3D_ERR_SHAPE", -3: "X3D_ERR_BC", -4: "X3D_ERR_DTYPE",
    -5: "X3D_ERR_CUDA", -6: "X3D_ERR_COEF", -7: "X3D_ERR_UNSUPPORTED", -8: "X3D_ERR_NOMEM",
    -9: "X3D_ERR_STATE", -10: "X3D_ERR_SCRATCH",
}

OP_DER1, OP_DER2, OP_FIL, OP_DVP, OP_IVP, OP_DPV, OP_IPV = range(7)
PREC_FP64, PREC_MIXED = 0, 1

COEF_NAMES = ["FF", "FS", "FW", "FFP", "FSP", "FWP", "SF", "SS", "SW", "SFP", "SSP", "SWP",
              "FIFF", "FIFS", "FIFW", "FIFFP", "FIFSP", "FIFWP", "CF6", "CS6", "CW6",
              "CIF6", "CIS6", "CIW6", "CIFP6", "CISP6", "CIWP6", "CFIP6", "CSIP6", "CWIP6",
              "CIFIP6", "CISIP6", "CIWIP6", "CFI6", "CSI6", "CWI6", "CIFI6", "CISI6", "CIWI6",
              "CFP6", "CSP6", "CWP6"]
COEF = {n: i for i, n in enumerate(COEF_NAMES)}


class X3DError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = "%s failed: %s (%d)" % (what, ERRORS.get(status, "?"), status)
        if status == -5 and _lib is not None:
            msg += ": " + _lib.x3d_last_cuda_error().decode()
        super().__init__(msg)


class Grid(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("xlx", ctypes.c_double), ("yly", ctypes.c_double), ("zlz", ctypes.c_double),
                ("nclx1", ctypes.c_int), ("nclxn", ctypes.c_int), ("ncly1", ctypes.c_int),
                ("nclyn", ctypes.c_int), ("nclz1", ctypes.c_int), ("nclzn", ctypes.c_int),
                ("istret", ctypes.c_int), ("beta", ctypes.c_double)]


class NumOpts(ctypes.Structure):
    _fields_ = [("ifirstder", ctypes.c_int), ("isecondder", ctypes.c_int), ("ipinter", ctypes.c_int),
                ("filter_alpha", ctypes.c_double), ("nu0nu", ctypes.c_double), ("cnu", ctypes.c_double)]


class SolverOpts(ctypes.Structure):
    _fields_ = [("itimescheme", ctypes.c_int), ("dt", ctypes.c_double), ("xnu", ctypes.c_double),
                ("precision", ctypes.c_int)]


_lock = threading.Lock()
_lib = None


def declared_symbols():
    """Names of every x3d_* function declared in include/x3d_gpu.h."""
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(x3d_[a-z0-9_]+)\s*\(", txt)))


def load():
    """Load the library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libx3dgpu.so not built: run __graft_entry__.build() "
                               "(or python incompact3d_gb300/build.py)")
        lib = ctypes.CDLL(LIB_PATH)
        P, I, D, LL = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_longlong
        lib.x3d_strerror.restype = ctypes.c_char_p
        lib.x3d_strerror.argtypes = [I]
        lib.x3d_last_cuda_error.restype = ctypes.c_char_p
        lib.x3d_last_cuda_error.argtypes = []
        lib.x3d_ctx_create.argtypes = [ctypes.POINTER(Grid), ctypes.POINTER(NumOpts), ctypes.POINTER(P)]
        lib.x3d_ctx_destroy.argtypes = [P]
        lib.x3d_get_coeffs.argtypes = [P, I, I, P, I]
        lib.x3d_apply.argtypes = [P, I, I, I, I, I, P, P, P, P]
        lib.x3d_plan_info.argtypes = [P, I, I, I, I, P, P, P]
        lib.x3d_conv_diff_f32.argtypes = [P, I, I, P, P, P, P, ctypes.c_float, P, P]
        colloc = [P, P, P, P, P, P, P, P, I, I, I, I, D, P]
        for n in ("derx", "derz", "derxx", "deryy", "derzz", "filx", "fily", "filz"):
            getattr(lib, "x3d_" + n).argtypes = colloc
        lib.x3d_dery.argtypes = [P, P, P, P, P, P, P, P, P, I, I, I, I, D, P]
        for n in ("derx", "dery", "derz", "derxx", "deryy", "derzz", "filx", "fily", "filz"):
            getattr(lib, "x3d_%s_f32" % n).argtypes = [P, P, P, I, I, I, I, P]
        vp = [P, P, P, P, P, P, P, P, I, I, I, I, I, P]
        for n in ("derxvp", "interxvp", "interyvp", "derzvp", "interzvp"):
            getattr(lib, "x3d_" + n).argtypes = vp
        lib.x3d_deryvp.argtypes = [P, P, P, P, P, P, P, P, P, I, I, I, I, I, P]
        pv = [P, P, P, P, P, P, P, P, P, P, P, I, I, I, I, I, P]
        for n in ("derxpv", "interxpv", "interypv", "derzpv", "interzpv"):
            getattr(lib, "x3d_" + n).argtypes = pv
        lib.x3d_derypv.argtypes = [P, P, P, P, P, P, P, P, P, P, P, P, I, I, I, I, I, P]
        lib.x3d_poisson.argtypes = [P, P, P]
        lib.x3d_poisson_ex.argtypes = [P, P, I, P]
        lib.x3d_poisson_noalloc.argtypes = [P, P, P]
        for n in ("x_to_y", "y_to_z", "z_to_y", "y_to_x"):
            getattr(lib, "x3d_transpose_" + n).argtypes = [P, P, P, LL, P]
        lib.x3d_divergence.argtypes = [P, P, P, P, P, P]
        lib.x3d_gradp.argtypes = [P, P, P, P, P, P]
        lib.x3d_divergence_f32.argtypes = [P, P, P, P, P, P]
        lib.x3d_gradp_f32.argtypes = [P, P, P, P, P, P]
        lib.x3d_cor_vel.argtypes = [P, P, P, P, P, P, P, P]
        lib.x3d_solver_create.argtypes = [P, ctypes.POINTER(SolverOpts), ctypes.POINTER(P)]
        lib.x3d_solver_destroy.argtypes = [P]
        lib.x3d_solver_set_velocity.argtypes = [P, P, P, P, I]
        lib.x3d_solver_get_velocity.argtypes = [P, P, P, P, I]
        lib.x3d_solver_set_velocity_async.argtypes = [P, P, P, P, P]
        lib.x3d_solver_get_velocity_async.argtypes = [P, P, P, P, P]
        lib.x3d_solver_sync.argtypes = [P]
        lib.x3d_solver_init_tgv.argtypes = [P]
        lib.x3d_solver_step.argtypes = [P, I, P]
        lib.x3d_solver_tgv_stats.argtypes = [P, P, P]
        lib.x3d_solver_divmax.argtypes = [P, P, P]
        lib.x3d_solver_launches_per_step.argtypes = [P]
        lib.x3d_solver_set_channel.argtypes = [P, D, D, I]
        lib.x3d_solver_bulk_velocity.argtypes = [P, P, I]
        lib.x3d_get_stretching.argtypes = [P, I, P, I]
        lib.x3d_solver_set_les.argtypes = [P, I, D, D]
        lib.x3d_solver_get_field.argtypes = [P, I, P, I]
        lib.x3d_mlp_create.argtypes = [I, I, I, ctypes.POINTER(P)]
        lib.x3d_mlp_destroy.argtypes = [P]
        lib.x3d_mlp_param_count.argtypes = []
        lib.x3d_mlp_set_params.argtypes = [P, P, P]
        lib.x3d_mlp_get_params.argtypes = [P, P, P]
        lib.x3d_mlp_infer.argtypes = [P, P, P, LL, P]
        lib.x3d_mlp_train_step.argtypes = [P, P, P, LL, ctypes.c_float, P, P]
        lib.x3d_box_filter4.argtypes = [P, P, P, I, I, I, P, P, P, P, P]
        lib.x3d_mlp_set_flux_loss.argtypes = [P, ctypes.c_float, ctypes.c_float]
        lib.x3d_mlp_set_tensor_cores.argtypes = [P, I]
        lib.x3d_mlp_status.argtypes = [P]
        lib.x3d_solver_set_les_mlp.argtypes = [P, P]
        lib.x3d_solver_set_field.argtypes = [P, I, P, I]
        lib.x3d_solver_get_itime.argtypes = [P]
        lib.x3d_solver_set_itime.argtypes = [P, I]
        lib.x3d_solver_les_fields.argtypes = [P, P, P, P, P, P]
        _lib = lib
        return lib


def check(status, what=""):
    if status < 0:
        raise X3DError(status, what)
    return status
