"""ctypes binding of libsfwi_gb300.so (the C ABI in include/sfwi_gb300.h).

The library is loaded from sfwi_gb300/lib/ only; there is no other
implementation to fall back to, so a missing build raises ImportError-like
errors at first use.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libsfwi_gb300.so")

_fp, _dp, _ip = C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_int)
_h = C.c_void_p


class ShotDesc(C.Structure):
    _fields_ = [("nx", C.c_int), ("isx", C.c_int), ("isz", C.c_int), ("igz", C.c_int), ("ngx_left", C.c_int),
                ("delta_left", C.c_int), ("record_left_in_v", C.c_int), ("ntr", C.c_int), ("gc", _ip),
                ("rec_z", _fp), ("rec_x", _fp)]


class ModelDesc(C.Structure):
    _fields_ = [("allnx", C.c_int), ("allnz", C.c_int), ("nt", C.c_int), ("vp", _fp), ("vs", _fp), ("rho", _fp),
                ("dvp", _fp), ("dvs", _fp)]


# name: (restype, argtypes)
SIGNATURES = {
    "sfwi_create": (C.c_int, [C.POINTER(_h), C.c_int, _fp, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int,
                              C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    "sfwi_destroy": (C.c_int, [_h]),
    "sfwi_gpu_buffer_vpvs": (C.c_int, [_h, _fp, _fp, _fp]),
    "sfwi_gpu_buffer_m": (C.c_int, [_h, _fp, _fp]),
    "sfwi_buffer_vpvs_htod": (C.c_int, [_h, C.c_int]),
    "sfwi_record_copy_to_gpu": (C.c_int, [_h, _fp, _fp, _ip]),
    "sfwi_set_shot_geometry": (C.c_int, [_h, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    "sfwi_set_misfit": (C.c_int, [_h, C.c_int]),
    "sfwi_image_singleshot": (C.c_int, [_h, _dp]),
    "sfwi_imagebuffer_resettozero": (C.c_int, [_h, _fp, _fp, _fp, _fp, _fp, _fp, _fp]),
    "sfwi_read_gradients_f64": (C.c_int, [_h, _dp, _dp, _dp]),
    "sfwi_set_density_gradient": (C.c_int, [_h, C.c_int]),
    "sfwi_set_snapshots": (C.c_int, [_h, C.c_int, C.c_int]),
    "sfwi_set_cpu_mem": (C.c_int, [_h, C.c_int, C.c_int]),
    "sfwi_strip_bytes": (C.c_int, [_h, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "sfwi_set_pinned_cache": (C.c_int, [C.c_size_t]),
    "sfwi_read_density_gradient_f64": (C.c_int, [_h, _dp]),
    "sfwi_read_records": (C.c_int, [_h, C.c_int, _fp, _fp, _fp, _fp, _fp, _fp]),
    "sfwi_enqueue_shot": (C.c_int, [_h, C.POINTER(ShotDesc)]),
    "sfwi_run": (C.c_int, [_h, _dp, _dp]),
    "sfwi_run_forward": (C.c_int, [_h]),
    "sfwi_born_adjoint": (C.c_int, [_h, _dp, _dp]),
    "sfwi_hessian_vector": (C.c_int, [_h, _fp, _fp, _dp, _dp]),
    "sfwi_run_models": (C.c_int, [_h, C.c_int, C.POINTER(ModelDesc), _ip, _dp, _dp, _dp, _dp, _dp]),
    "sfwi_calculate_alpha_parabola_mb": (C.c_int, [_h, _fp, _fp, C.c_float, C.c_float, _dp, _dp, _dp]),
    "sfwi_calculate_alpha": (C.c_int, [_h, _fp, _fp, _fp, _fp, _dp, _dp]),
    "sfwi_line_search_parabola": (C.c_int, [_h, _fp, _fp, C.c_float, C.c_float, _dp, _dp]),
    "sfwi_line_search_exact": (C.c_int, [_h, _fp, _fp, _fp, _fp, _dp, _dp, _dp]),
    "sfwi_ot": (C.c_int, [_fp, _fp, _fp, _fp, _fp, _fp, C.c_int, C.c_int, C.c_float, _dp]),
    "sfwi_ot_power": (C.c_int, [_fp, _fp, _fp, _fp, _fp, _fp, C.c_int, C.c_int, C.c_float, _dp]),
    "sfwi_ot_alltrace": (C.c_int, [_fp, _fp, _fp, _fp, _fp, _fp, C.c_int, C.c_int, C.c_float, _dp]),
    "sfwi_ot_noalloc": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_int, C.c_int, C.c_float, _dp, C.c_void_p]),
    "sfwi_normalize": (C.c_int, [_fp, C.c_int, C.c_int]),
    "sfwi_last_error": (C.c_char_p, []),
    "sfwi_kernel_launches": (C.c_longlong, [_h]),
    "sfwi_last_timing": (C.c_int, [_h, _fp, _fp, _fp, _fp]),
    "sfwi_time_kernels": (C.c_int, [_h, C.c_int, _fp]),
    "sfwi_set_tile_shape": (C.c_int, [_h, C.c_int]),
    "sfwi_set_launch_overlap": (C.c_int, [_h, C.c_int]),
    "sfwi_set_tile_order": (C.c_int, [_h, C.c_uint]),
    "sfwi_clear_queue": (C.c_int, [_h]),
    "sfwi_set_source": (C.c_int, [_h, C.c_int]),
    "sfwi_wait_selftest": (C.c_int, [_h, C.c_uint]),
    "sfwi_debug_grid_shape": (C.c_int, [_h, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                        C.POINTER(C.c_int)]),
    "sfwi_debug_read_grid": (C.c_int, [_h, C.c_int, _fp]),
    "sfwi_debug_tile_grid": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, _ip, C.c_int, C.POINTER(C.c_int), _ip,
                                       _ip, _ip]),
    "sfwi_get_tile_shape": (C.c_int, [_h, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "sfwi_autotune": (C.c_int, [_h, C.c_int, C.POINTER(C.c_int), _fp]),
    "sfwi_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(C.c_void_p)]),
    "sfwi_host_free": (C.c_int, [C.c_void_p]),
    "sfwi_version": (C.c_char_p, []),
}

_lib = None


def load():
    """Load the library (raises OSError with the build hint if it is absent)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError("libsfwi_gb300.so is not built (%s); run python -m sfwi_gb300.build" % LIB_PATH)
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


class SfwiError(RuntimeError):
    pass


def check(rc):
    if rc != 0:
        msg = load().sfwi_last_error().decode(errors="replace")
        raise SfwiError("sfwi error %d: %s" % (rc, msg))
    return rc
