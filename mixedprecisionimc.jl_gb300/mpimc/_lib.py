"""ctypes binding of the C ABI in include/imc.h (libimc.so).

The structures below mirror the C declarations field for field.  The library
is loaded from the in-tree build folder; if it is missing the import of the
engine fails loudly -- there is no CPU fallback for any stage.
"""
import ctypes as C
import os

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "_build", "libimc.so")

IMC_ABI_VERSION = 1

# status codes
IMC_OK = 0
IMC_ERR_INVALID_ARG = 1
IMC_ERR_CUDA = 2
IMC_ERR_OOM = 3
IMC_ERR_CAPACITY = 4
IMC_ERR_NUMERIC = 5
IMC_ERR_SEGMENT_CAP = 6
IMC_ERR_NO_ENERGY = 7
IMC_ERR_STATE = 8
IMC_ERR_NO_DEVICE = 9
IMC_ERR_TIMEOUT = 10

ERROR_NAMES = {
    0: "IMC_OK", 1: "IMC_ERR_INVALID_ARG", 2: "IMC_ERR_CUDA", 3: "IMC_ERR_OOM", 4: "IMC_ERR_CAPACITY",
    5: "IMC_ERR_NUMERIC", 6: "IMC_ERR_SEGMENT_CAP", 7: "IMC_ERR_NO_ENERGY", 8: "IMC_ERR_STATE",
    9: "IMC_ERR_NO_DEVICE", 10: "IMC_ERR_TIMEOUT",
}

# error-flag bits
IMC_FLAG_NAN = 1 << 0
IMC_FLAG_NEG_TALLY = 1 << 1
IMC_FLAG_SEGMENT_CAP = 1 << 2
IMC_FLAG_CAPACITY = 1 << 3
IMC_FLAG_NO_ENERGY = 1 << 4
IMC_FLAG_FIXPOINT_RANGE = 1 << 5
IMC_FLAG_SURROGATE_DOMAIN = 1 << 6

IMC_GEOM_1D, IMC_GEOM_2D = 1, 2
IMC_FP64, IMC_FP32, IMC_FP16 = 0, 1, 2
IMC_BC_VACUUM, IMC_BC_REFLECT = 0, 1
IMC_TS_CONSTANT, IMC_TS_RAMP = 0, 1
IMC_LEFT, IMC_RIGHT, IMC_TOP, IMC_BOTTOM = 0, 1, 2, 3

FIELDS = {
    "temp": 0, "radenergydens": 1, "matenergydens": 2, "fleck": 3, "beta": 4,
    "sigma_a": 5, "sigma_s": 6, "bee": 7, "energydep": 8, "emittedenergy": 9,
}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class ImcDeck(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32), ("geometry", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32),
        ("precision", C.c_int32), ("scale_select_precision", C.c_int32),
        ("dx", _dp), ("dy", _dp), ("temp", _dp), ("sigma_a_val", _dp), ("sigma_a_pow", _dp),
        ("sigma_s_val", _dp), ("sigma_s_pow", _dp), ("bee", _dp), ("radsource", _dp), ("t_surface", _dp),
        ("bc", C.c_int32 * 4),
        ("phys_c", C.c_double), ("phys_a", C.c_double), ("alpha", C.c_double),
        ("n_scales", C.c_int32), ("energyscales", _dp),
        ("distancescale", C.c_double),
        ("n_input", C.c_int64), ("n_max", C.c_int64),
        ("cellmin", C.c_double),
        ("linearized", C.c_int32), ("marshak_opacity", C.c_int32),
        ("temp_floor", C.c_double),
        ("seed", C.c_uint64),
        ("timestepping", C.c_int32), ("sort_census", C.c_int32),
        ("dt", C.c_double), ("dt0", C.c_double), ("k", C.c_double), ("dtmax", C.c_double),
        ("t_end", C.c_double),
        ("capacity", C.c_int64), ("segment_cap", C.c_int64),
    ]


class ImcStepStats(C.Structure):
    _fields_ = [
        ("t", C.c_double), ("dt", C.c_double), ("total_energy", C.c_double), ("energy_dep", C.c_double),
        ("rad_energy", C.c_double), ("rad_energy_old", C.c_double), ("lost_energy", C.c_double),
        ("energy_error", C.c_double),
        ("n_census_in", C.c_int64), ("n_sourced", C.c_int64), ("n_census_out", C.c_int64),
        ("segments", C.c_int64), ("surrogate_calls", C.c_int64),
        ("error_flags", C.c_uint32), ("step_index", C.c_uint32),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class ImcParticles(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("t", _dp), ("x", _dp), ("y", _dp), ("mu", _dp), ("ux", _dp), ("uy", _dp), ("E", _dp), ("E0", _dp),
        ("cell", _ip), ("scale", _ip),
    ]


class ImcSurrogateTrainConfig(C.Structure):
    """struct ImcSurrogateTrainConfig of include/imc.h."""
    _fields_ = [("seed", C.c_uint64), ("n_samples", C.c_int64), ("batch", C.c_int32), ("iterations", C.c_int32),
                ("lr", C.c_float), ("lr_min", C.c_float)]


class ImcDeviceParticles(C.Structure):
    """Caller-owned device arrays for imc_clean_noalloc (device pointers)."""
    _fields_ = [("t", C.c_void_p), ("x", C.c_void_p), ("y", C.c_void_p), ("ux", C.c_void_p), ("uy", C.c_void_p),
                ("E", C.c_void_p), ("E0", C.c_void_p), ("cs", C.c_void_p), ("alive", C.c_void_p)]


class ImcError(RuntimeError):
    def __init__(self, code, msg):
        self.code = code
        super().__init__("%s: %s" % (ERROR_NAMES.get(code, str(code)), msg))


# name -> (restype, argtypes)
_H = C.c_void_p
SIGNATURES = {
    "imc_create": (C.c_int, [C.POINTER(ImcDeck), C.POINTER(_H)]),
    "imc_destroy": (C.c_int, [_H]),
    "imc_last_error": (C.c_int, [_H, C.c_char_p, C.c_size_t]),
    "imc_abi_version": (C.c_int, []),
    "imc_device_info": (C.c_int, [C.c_char_p, C.c_size_t, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "imc_update": (C.c_int, [_H]),
    "imc_sourcing": (C.c_int, [_H]),
    "imc_transport": (C.c_int, [_H]),
    "imc_clean": (C.c_int, [_H]),
    "imc_tally": (C.c_int, [_H]),
    "imc_energycheck": (C.c_int, [_H, C.POINTER(C.c_double)]),
    "imc_timestep": (C.c_int, [_H, C.POINTER(C.c_int)]),
    "imc_step": (C.c_int, [_H, C.POINTER(ImcStepStats), C.POINTER(C.c_int)]),
    "imc_run": (C.c_int, [_H, C.c_int64, C.POINTER(ImcStepStats), C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
    "imc_get_time": (C.c_int, [_H, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "imc_set_time": (C.c_int, [_H, C.c_double, C.c_double]),
    "imc_num_particles": (C.c_int, [_H, C.POINTER(C.c_int64)]),
    "imc_get_field": (C.c_int, [_H, C.c_int, _dp, C.c_int64]),
    "imc_set_field": (C.c_int, [_H, C.c_int, _dp, C.c_int64]),
    "imc_get_particles": (C.c_int, [_H, C.POINTER(ImcParticles)]),
    "imc_set_particles": (C.c_int, [_H, C.POINTER(ImcParticles)]),
    "imc_get_stats": (C.c_int, [_H, C.POINTER(ImcStepStats)]),
    "imc_set_timing": (C.c_int, [_H, C.c_int]),
    "imc_transport_timing": (C.c_int, [_H, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "imc_kernels_per_step": (C.c_int, [_H, C.POINTER(C.c_int)]),
    "imc_clean_noalloc": (C.c_int, [C.c_int, C.c_int, C.POINTER(ImcDeviceParticles), C.POINTER(ImcDeviceParticles),
                                    C.c_int64, C.POINTER(C.c_int64), C.c_void_p]),
    "imc_surrogate_param_count": (C.c_int, [C.POINTER(C.c_int)]),
    "imc_surrogate_train": (C.c_int, [C.POINTER(ImcSurrogateTrainConfig), C.c_void_p, C.c_void_p]),
    "imc_surrogate_walk": (C.c_int, [C.c_uint64, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    "imc_surrogate_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                     C.POINTER(C.c_double)]),
    "imc_surrogate_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "imc_surrogate_sample": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                       C.c_void_p]),
    "imc_set_surrogate": (C.c_int, [_H, C.c_void_p, C.c_int64]),
    "imc_save_state": (C.c_int, [_H, C.c_void_p, C.POINTER(C.c_size_t)]),
    "imc_load_state": (C.c_int, [_H, C.c_void_p, C.c_size_t]),
    "imc_get_totals": (C.c_int, [_H, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "imc_run_batch": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.c_int64, C.c_int32, C.POINTER(C.c_int64),
                                C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
    "imc_get_surrogate_active": (C.c_int, [_H, C.POINTER(C.c_int)]),
    "imc_run_batch_fused": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.c_int64, C.POINTER(C.c_int64),
                                      C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
}

_LIB = None


def load(path=None):
    """Load libimc.so (once) and declare every entry point's signature."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError("libimc.so is not built (%s); run __graft_entry__.build() first" % p)
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.imc_abi_version() != IMC_ABI_VERSION:
        raise ImportError("libimc.so ABI version mismatch")
    if path is None:
        _LIB = lib
    return lib


def check(rc, handle=None, lib=None):
    if rc == IMC_OK:
        return
    lib = lib or load()
    buf = C.create_string_buffer(512)
    lib.imc_last_error(handle, buf, 512)
    raise ImcError(rc, buf.value.decode(errors="replace"))
