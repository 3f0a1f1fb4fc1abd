"""ctypes declarations of the C ABI in include/saras_gb300.h.

The product library is ``saras_gb300/_build/libsaras_gb300.so`` (built by
``saras_gb300.build``).  Loading it never touches a GPU; every compute entry
point returns SARAS_NO_DEVICE when no CUDA device is present, and the Python
layer raises on any non-zero status.  There is no CPU fallback.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libsaras_gb300.so")

OK, NOT_CONVERGED, DIVERGENCE_LIMIT, BAD_CONFIG, CUDA_ERROR, BAD_ARG, NO_DEVICE, NOT_FINITE, TOO_LARGE = range(9)
STATUS_NAMES = {
    0: "SARAS_OK", 1: "SARAS_NOT_CONVERGED", 2: "SARAS_DIVERGENCE_LIMIT", 3: "SARAS_BAD_CONFIG",
    4: "SARAS_CUDA_ERROR", 5: "SARAS_BAD_ARG", 6: "SARAS_NO_DEVICE", 7: "SARAS_NOT_FINITE", 8: "SARAS_TOO_LARGE",
}

(FIELD_VX, FIELD_VY, FIELD_VZ, FIELD_P, FIELD_T, FIELD_PP, FIELD_MGRHS, FIELD_NSE_X, FIELD_NSE_Y,
 FIELD_NSE_Z, FIELD_TRHS, FIELD_GRAD_X, FIELD_GRAD_Y, FIELD_GRAD_Z) = range(14)
NUM_FIELDS = 14
FIELD_NAMES = ["Vx", "Vy", "Vz", "P", "T", "Pp", "mgRHS", "nseRHS.Vx", "nseRHS.Vy", "nseRHS.Vz",
               "tmpRHS", "pressureGradient.Vx", "pressureGradient.Vy", "pressureGradient.Vz"]

MG_REFERENCE, MG_PLAIN_TARGET, MG_MIXED = 0, 1, 2
GUESS_PREVIOUS, GUESS_LEARNED, GUESS_EXTRAPOLATE, GUESS_QUADRATIC, GUESS_PARITY, GUESS_NETWORK = 0, 1, 2, 3, 4, 5
SMOOTHER_JACOBI, SMOOTHER_CHEBYSHEV = 0, 1

_I, _D = ctypes.c_int, ctypes.c_double


class saras_params(ctypes.Structure):
    """Mirror of ``struct saras_params`` (field order must match the header)."""
    _fields_ = [
        ("probType", _I), ("icType", _I), ("rbcType", _I), ("forceType", _I),
        ("xPer", _I), ("yPer", _I), ("zPer", _I),
        ("Re", _D), ("Ra", _D), ("Pr", _D), ("Ro", _D), ("Ta", _D),
        ("Lx", _D), ("Ly", _D), ("Lz", _D),
        ("nonHgBC", _I), ("patchRadius", _D),
        ("xGrid", _I), ("yGrid", _I), ("zGrid", _I),
        ("betaX", _D), ("betaY", _D), ("betaZ", _D),
        ("xInd", _I), ("yInd", _I), ("zInd", _I),
        ("nThreads", _I), ("npX", _I), ("npY", _I),
        ("dScheme", _I), ("iScheme", _I),
        ("cnTolerance", _D),
        ("restartFlag", _I), ("useCFL", _I),
        ("courantNumber", _D), ("tStp", _D), ("tMax", _D),
        ("ioCnt", _I), ("solnFormat", _I),
        ("fwInt", _D), ("rsInt", _D),
        ("readProbes", _I),
        ("prInt", _D),
        ("vcDepth", _I), ("vcCount", _I),
        ("mgTolerance", _D),
        ("gsSmooth", _I), ("preSmooth", _I), ("postSmooth", _I), ("resType", _I), ("printResidual", _I),
        ("testPoisson", _I), ("mgMode", _I),
        ("mgTarget", _D),
        ("mgMaxCycles", _I), ("mixedCycles", _I), ("guessMode", _I),
        ("jacobiWeight", _D),
        ("seed", _I),
        ("fastKernels", _I),
        ("smoother", _I),
        ("coarseSmooth", _I),
        ("coarseCycles", _I),
    ]

    def to_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class saras_step_stats(ctypes.Structure):
    _fields_ = [
        ("cn_iters", _I * 4), ("vcycles", _I), ("refine_steps", _I), ("coarse_iters", _I),
        ("mg_residual", _D), ("fine_residual", _D), ("guess_residual", _D),
        ("guess_source", _I), ("status", _I),
    ]


def default_params():
    """Same defaults as the C ``saras_default_params`` (used when the library is absent)."""
    p = saras_params()
    p.probType, p.icType, p.rbcType, p.forceType = 2, 1, 1, 0
    p.xPer = p.yPer = p.zPer = 1
    p.Re, p.Ra, p.Pr, p.Ro, p.Ta = 1000.0, 1.0e4, 0.71, 12.0, 0.0
    p.Lx = p.Ly = p.Lz = 1.0
    p.nonHgBC, p.patchRadius = 0, 0.25
    p.xGrid = p.yGrid = p.zGrid = 0
    p.betaX = p.betaY = p.betaZ = 1.0
    p.xInd = p.yInd = p.zInd = 5
    p.nThreads, p.npX, p.npY = 1, 1, 1
    p.dScheme, p.iScheme = 1, 1
    p.cnTolerance = 1.0e-8
    p.restartFlag, p.useCFL = 0, 0
    p.courantNumber, p.tStp, p.tMax = 0.1, 1.0e-3, 0.1
    p.ioCnt, p.solnFormat = 1, 1
    p.fwInt, p.rsInt = 0.1, 0.1
    p.readProbes, p.prInt = 0, 0.1
    p.vcDepth, p.vcCount = 3, 200
    p.mgTolerance = 1.0e-8
    p.gsSmooth, p.preSmooth, p.postSmooth, p.resType, p.printResidual = 0, 3, 3, 1, 0
    p.testPoisson, p.mgMode = 0, MG_REFERENCE
    p.mgTarget, p.mgMaxCycles, p.mixedCycles, p.guessMode = 1.0e-8, 200, 1, GUESS_PREVIOUS
    p.jacobiWeight, p.seed = 1.0, 42
    p.fastKernels = 0
    p.smoother = SMOOTHER_JACOBI
    p.coarseSmooth = 0
    p.coarseCycles = 0
    return p


_lib = None


def load():
    """Load the product library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            "saras_gb300: native library %s is missing; run saras_gb300.build.build() "
            "(there is no CPU fallback)" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    vp, ip, dp, cp = ctypes.c_void_p, ctypes.POINTER(_I), ctypes.POINTER(_D), ctypes.c_char_p
    P = ctypes.POINTER(saras_params)
    sigs = {
        "saras_default_params": (_I, [P]),
        "saras_parse_yaml": (_I, [cp, P, ctypes.c_char_p, _I]),
        "saras_create": (_I, [P, ctypes.POINTER(vp)]),
        "saras_destroy": (_I, [vp]),
        "saras_last_error": (cp, [vp]),
        "saras_field_dims": (_I, [vp, _I, ip]),
        "saras_grid_coords": (_I, [vp, _I, _I, dp, _I, ip]),
        "saras_upload": (_I, [vp, _I, dp]),
        "saras_download": (_I, [vp, _I, dp]),
        "saras_upload_fields": (_I, [vp, _I, ip, ctypes.POINTER(dp)]),
        "saras_download_fields": (_I, [vp, _I, ip, ctypes.POINTER(dp)]),
        "saras_synchronize": (_I, [vp]),
        "saras_launch_count": (ctypes.c_longlong, [vp]),
        "saras_plane_tma_active": (_I, [vp]),
        "saras_apply_bc": (_I, [vp, _I]),
        "saras_sync_field": (_I, [vp, _I]),
        "saras_vfield_compute_diff": (_I, [vp]),
        "saras_vfield_compute_nlin": (_I, [vp]),
        "saras_sfield_gradient": (_I, [vp, _I]),
        "saras_vfield_divergence": (_I, [vp]),
        "saras_tfield_compute_diff": (_I, [vp]),
        "saras_tfield_compute_nlin": (_I, [vp]),
        "saras_axpby": (_I, [vp, _I, _D, _I, _D]),
        "saras_cn_solve": (_I, [vp, _I, ip, dp]),
        "saras_cn_solve_noalloc": (_I, [P, _I, vp, vp, vp, ip, dp]),
        "saras_mg_solve": (_I, [vp, ip, dp]),
        "saras_mg_set_mode": (_I, [vp, _I, _D, _I]),
        "saras_time_advance": (_I, [vp, ctypes.POINTER(saras_step_stats)]),
        "saras_diagnostics": (_I, [vp, dp, dp, dp]),
        "saras_compute_tstp": (_I, [vp, dp]),
        "saras_set_dt": (_I, [vp, _D]),
        "saras_parse_probes": (_I, [cp, ip, _I, ip, ctypes.c_char_p, _I]),
        "saras_probe": (_I, [vp, _I, ip, _I, ip, dp]),
        "saras_write_restart": (_I, [vp, cp, _D]),
        "saras_read_restart": (_I, [vp, cp, dp]),
        "saras_mg_test_prolong": (_I, [vp, dp]),
        "saras_mg_test_transfer": (_I, [vp, dp]),
        "saras_mg_test_periodic": (_I, [vp, dp]),
        "saras_hydro_test_periodic": (_I, [vp, dp]),
        "saras_mg_level_dims": (_I, [vp, _I, ip]),
        "saras_mg_set_level": (_I, [vp, _I, _I, dp]),
        "saras_mg_get_level": (_I, [vp, _I, _I, dp]),
        "saras_mg_smooth": (_I, [vp, _I, _I]),
        "saras_mg_restrict": (_I, [vp, _I]),
        "saras_mg_prolong_add": (_I, [vp, _I]),
        "saras_mg_compute_error": (_I, [vp, _I, dp]),
        "saras_unet_collect": (_I, [vp]),
        "saras_unet_train": (_I, [vp, _I, _D, dp]),
        "saras_unet_infer": (_I, [vp, _I]),
        "saras_set_guess_mode": (_I, [vp, _I]),
        "saras_unet_shape": (_I, [vp, ctypes.POINTER(ctypes.c_longlong), ip]),
        "saras_unet_grad_check": (_I, [vp, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, dp, ctypes.c_void_p]),
        "saras_conv3d_check": (_I, [_I, _I, _I, _I, _I, _I, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _I,
                                    ctypes.POINTER(ctypes.c_float)]),
        "saras_profile_enable": (_I, [vp, _I, _I]),
        "saras_profile_read": (_I, [vp, _I, ctypes.POINTER(ctypes.c_longlong), dp, dp]),
        "saras_profile_name": (cp, [_I]),
        "saras_profile_count": (_I, []),
        "saras_profile_sample": (_I, [vp, _I]),
        "saras_event_record": (_I, [vp, _I]),
        "saras_event_elapsed": (_I, [vp, _I, _I, dp]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


# Every function the header declares (checked by the CPU test suite).
HEADER_SYMBOLS = None


def header_symbols():
    """Parse include/saras_gb300.h and return the declared entry-point names."""
    import re
    hdr = os.path.join(os.path.dirname(_HERE), "include", "saras_gb300.h")
    text = open(hdr).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(saras_[a-z0-9_]+)\s*\(", text)))
