"""ctypes binding of libmflbm.so (the C ABI declared in include/mflbm.h).

The library is the only compute path: importing this module never falls back to a CPU
implementation.  ``load()`` raises if libmflbm.so has not been built; the calls that
need a GPU fail with MFLBM_ENODEV when none is present.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libmflbm.so")

MFLBM_ABI_VERSION = 2
LAYOUT_AUTO, LAYOUT_DENSE, LAYOUT_LIST = 0, 1, 2
MFLBM_OK = 0
MFLBM_EINVAL = -1
MFLBM_ECUDA = -2
MFLBM_ENOMEM = -3
MFLBM_ESTATE = -4
MFLBM_ETIMEOUT = -5
MFLBM_ENODEV = -6
MFLBM_ERANGE = -7
MFLBM_RUNNING = 0
MFLBM_FAILED = 3
MFLBM_FP64 = 0
MFLBM_FP32 = 1
MFLBM_FP16 = 2
MFLBM_FP64FF = 3
MFLBM_FF = 4
MFLBM_NOALLOC_MAX_NZ = 16384

ERROR_NAMES = {
    MFLBM_EINVAL: "MFLBM_EINVAL", MFLBM_ECUDA: "MFLBM_ECUDA", MFLBM_ENOMEM: "MFLBM_ENOMEM",
    MFLBM_ESTATE: "MFLBM_ESTATE", MFLBM_ETIMEOUT: "MFLBM_ETIMEOUT", MFLBM_ENODEV: "MFLBM_ENODEV",
    MFLBM_ERANGE: "MFLBM_ERANGE",
}


class Params(C.Structure):
    """mflbm_params (include/mflbm.h)."""
    _fields_ = [
        ("abi_version", C.c_int32), ("multiphase", C.c_int32),
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("iper", C.c_int32), ("jper", C.c_int32), ("kper", C.c_int32),
        ("wall_x_min", C.c_int32), ("wall_x_max", C.c_int32),
        ("wall_y_min", C.c_int32), ("wall_y_max", C.c_int32),
        ("wall_z_min", C.c_int32), ("wall_z_max", C.c_int32),
        ("inlet_bc", C.c_int32), ("outlet_bc", C.c_int32), ("mrt", C.c_int32),
        ("porous_plate_cmd", C.c_int32), ("z_porous_plate", C.c_int32),
        ("precision", C.c_int32), ("strict_fp", C.c_int32), ("device", C.c_int32),
        ("layout", C.c_int32),
        ("la_nu1", C.c_double), ("la_nu2", C.c_double), ("gamma", C.c_double), ("beta", C.c_double),
        ("sa_inject", C.c_double), ("force_z", C.c_double), ("uin_avg", C.c_double),
        ("rho_in", C.c_double), ("rho_out", C.c_double), ("relaxation", C.c_double),
    ]


class SolidBnd(C.Structure):
    """mflbm_solid_bnd: Fortran type indirect_solid_boundary_nodes (96 bytes)."""
    _fields_ = [("ix", C.c_int32), ("iy", C.c_int32), ("iz", C.c_int32), ("i_fluid_num", C.c_int32),
                ("neighbor_list", C.c_int32 * 18), ("la_weight", C.c_double)]


class FluidBnd(C.Structure):
    """mflbm_fluid_bnd: Fortran type indirect_fluid_boundary_nodes (48 bytes)."""
    _fields_ = [("ix", C.c_int32), ("iy", C.c_int32), ("iz", C.c_int32), ("_pad", C.c_int32),
                ("nwx", C.c_double), ("nwy", C.c_double), ("nwz", C.c_double), ("theta", C.c_double)]


assert C.sizeof(SolidBnd) == 96 and C.sizeof(FluidBnd) == 48

# numpy dtypes with the same byte layout (for building lists without Python loops)
SOLID_DTYPE = [("ix", "<i4"), ("iy", "<i4"), ("iz", "<i4"), ("i_fluid_num", "<i4"),
               ("neighbor_list", "<i4", (18,)), ("la_weight", "<f8")]
FLUID_DTYPE = [("ix", "<i4"), ("iy", "<i4"), ("iz", "<i4"), ("_pad", "<i4"),
               ("nwx", "<f8"), ("nwy", "<f8"), ("nwz", "<f8"), ("theta", "<f8")]

P = C.c_void_p
DP = C.POINTER(C.c_double)
PP = C.POINTER(C.c_void_p)

# exported symbol -> (restype, argtypes)
SIGNATURES = {
    "mflbm_version": (C.c_int32, []),
    "mflbm_preprocess_geometry": (C.c_int32, [C.POINTER(Params), P, C.c_double, P, C.c_int32, P, P, C.c_int32, P]),
    "mflbm_preprocess_last_error": (C.c_char_p, []),
    "mflbm_nn_gemm_bf16": (C.c_int32, [P, C.c_int32, P, C.c_int32, P, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                       C.c_int32, P, P]),
    "mflbm_nn_gemm_bf16_splitk": (C.c_int32, [P, C.c_int32, P, C.c_int32, P, C.c_int32, C.c_int32, C.c_int32,
                                              C.c_int32, C.c_int32, C.c_int32, P, P, P]),
    "mflbm_nn_im2col": (C.c_int32, [P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, P, P]),
    "mflbm_nn_col2im": (C.c_int32, [P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, P, P]),
    "mflbm_nn_transpose_bf16": (C.c_int32, [P, C.c_int32, C.c_int64, C.c_int64, C.c_int64, P, C.c_int64, C.c_int64,
                                            C.c_int64, P]),
    "mflbm_nn_bias_act": (C.c_int32, [P, P, P, P, P, C.c_int64, C.c_int32, C.c_int32, C.c_int32, P]),
    "mflbm_nn_relu_back": (C.c_int32, [P, P, C.c_int64, P]),
    "mflbm_nn_bias_grad": (C.c_int32, [P, P, C.c_int64, C.c_int32, P]),
    "mflbm_nn_avgpool2": (C.c_int32, [P, P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, P]),
    "mflbm_nn_avgpool2_back": (C.c_int32, [P, P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, P]),
    "mflbm_nn_up2_concat": (C.c_int32, [P, C.c_int32, P, C.c_int32, P, C.c_int32, C.c_int32, C.c_int32, P]),
    "mflbm_nn_up2_concat_back": (C.c_int32, [P, P, C.c_int32, P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, P]),
    "mflbm_nn_add": (C.c_int32, [P, P, C.c_int64, P]),
    "mflbm_nn_to_bf16": (C.c_int32, [P, P, C.c_int64, P]),
    "mflbm_nn_mse": (C.c_int32, [P, C.c_int32, P, P, P, P, C.c_int64, C.c_int32, C.c_float, P]),
    "mflbm_nn_adam": (C.c_int32, [P, P, P, P, P, C.c_int64, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int32,
                                  P]),
    "mflbm_ensemble_create": (C.c_int32, [C.POINTER(Params), C.c_int32, P, P, C.POINTER(C.c_void_p)]),
    "mflbm_ensemble_destroy": (None, [P]),
    "mflbm_ensemble_last_error": (C.c_char_p, [P]),
    "mflbm_ensemble_init": (C.c_int32, [P]),
    "mflbm_ensemble_set_active": (C.c_int32, [P, P]),
    "mflbm_ensemble_run": (C.c_int32, [P, C.c_int32, C.c_int32]),
    "mflbm_ensemble_flux": (C.c_int32, [P, P, P, P]),
    "mflbm_ensemble_configure": (C.c_int32, [P, C.c_int32, C.c_int32]),
    "mflbm_ensemble_tune": (C.c_int32, [P, C.c_int32, P, C.c_int32]),
    "mflbm_ensemble_info": (C.c_int32, [P, P, P, P, P]),
    "mflbm_ensemble_set_wait": (C.c_int32, [P, C.c_int64, C.c_int32]),
    "mflbm_nn_set_wait": (C.c_int32, [C.c_int64, C.c_int32]),
    "mflbm_layout": (C.c_int32, [P]),
    "mflbm_init_velocity": (C.c_int32, [P, P, P, P, P, C.c_int32]),
    "mflbm_steady_monitor": (C.c_int32, [P, C.c_int32, P]),
    "mflbm_create": (C.c_int32, [C.POINTER(Params), C.POINTER(C.c_void_p)]),
    "mflbm_destroy": (None, [P]),
    "mflbm_last_error": (C.c_char_p, [P]),
    "mflbm_set_geometry": (C.c_int32, [P, P, P, C.c_int32, P, C.c_int32, P]),
    "mflbm_upload_state": (C.c_int32, [P, P, P, P, P, P, P]),
    "mflbm_download_state": (C.c_int32, [P, P, P, P, P, P, P]),
    "mflbm_init_equilibrium": (C.c_int32, [P, P]),
    "mflbm_step": (C.c_int32, [P, C.c_int32]),
    "mflbm_change_inlet_fluid_phase": (C.c_int32, [P, C.c_int32, C.c_double]),
    "mflbm_run": (C.c_int32, [P, C.c_int32, C.c_int32]),
    "mflbm_color_gradient": (C.c_int32, [P]),
    "mflbm_get_gradient": (C.c_int32, [P, P, P, P, P, P]),
    "mflbm_macro": (C.c_int32, [P, P, P, P, P, P]),
    "mflbm_monitor": (C.c_int32, [P, P, P, P]),
    "mflbm_saturation": (C.c_int32, [P, P, P]),
    "mflbm_synchronize": (C.c_int32, [P]),
    "mflbm_set_profiling": (C.c_int32, [P, C.c_int32]),
    "mflbm_get_profile": (C.c_int32, [P, P, P, P, P]),
    "mflbm_saturation_noalloc": (C.c_int32, [P, P, C.c_int32, C.c_int32, C.c_int32, P, P]),
}

_lib = None


class MflbmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


def load(path=None):
    """Load libmflbm.so once and attach the prototypes; raise if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"libmflbm.so is not built ({p}); run mf-lbm_gb300/build.py")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.mflbm_version() != MFLBM_ABI_VERSION:
        raise RuntimeError("libmflbm.so ABI version mismatch")
    if path is None:
        _lib = lib
    return lib


def check(lib, ctx, rc):
    if rc != MFLBM_OK:
        msg = lib.mflbm_last_error(ctx)
        raise MflbmError(rc, msg.decode() if msg else "")
    return rc
