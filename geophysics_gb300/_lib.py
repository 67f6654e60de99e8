"""ctypes binding of libgeofd.so (the C ABI declared in include/geofd.h).

The library is the product: there is no Python or CPU fallback.  Loading
fails loudly when the extension has not been built.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libgeofd.so")

GEO_OK = 0
GEO_MEM_HOST, GEO_MEM_DEVICE = 0, 1
GEO_VARIANT_CPU, GEO_VARIANT_GPU, GEO_VARIANT_MPI = 0, 1, 2
GEO_MODE_EXACT, GEO_MODE_FAST = 0, 1
GEO_RTM_BOUNDARY, GEO_RTM_SNAPSHOT, GEO_RTM_LEARNED, GEO_RTM_CHECKPOINT = 0, 1, 2, 3

STATUS = {0: "GEO_OK", 1: "GEO_ERR_ARG", 2: "GEO_ERR_CUDA", 3: "GEO_ERR_IO", 4: "GEO_ERR_MODEL",
          5: "GEO_ERR_CFL", 6: "GEO_ERR_WINDOW", 7: "GEO_ERR_NOMEM", 8: "GEO_ERR_NAN"}


class GeoError(RuntimeError):
    def __init__(self, status, where, detail):
        super().__init__("%s: %s (%s)" % (where, STATUS.get(status, status), detail))
        self.status = status


class FD2DDesc(C.Structure):
    _fields_ = [("nx", C.c_int), ("nz", C.c_int), ("npd", C.c_int), ("nt", C.c_int),
                ("dx", C.c_float), ("dz", C.c_float), ("dt", C.c_float),
                ("favg", C.c_float), ("pfac", C.c_float), ("wtype", C.c_int),
                ("fs", C.c_float), ("ds", C.c_float), ("zs", C.c_float), ("is_", C.c_int),
                ("variant", C.c_int), ("sv", C.c_int), ("rec_iz", C.c_int), ("rec_scale", C.c_float),
                ("mute_tt", C.c_int)]


class FD3DDesc(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nx", "ny", "nz", "npd", "nt")] + \
               [(n, C.c_float) for n in ("dx", "dy", "dz", "dt", "favg", "pfac")] + \
               [(n, C.c_int) for n in ("wtype", "sv", "mode", "fsx", "fsy", "fsz", "dsx", "dsy", "dsz",
                                       "rec_iz", "rx0", "drx", "nrx", "ry0", "dry", "nry", "mute_tt")]


class RTM3DDesc(C.Structure):
    _fields_ = [("fd", FD3DDesc), ("ns", C.c_int), ("mute_tt", C.c_int), ("method", C.c_int),
                ("snap_every", C.c_int), ("ae", C.c_void_p), ("na", C.c_int), ("da", C.c_int), ("dcdp", C.c_int),
                ("theta", C.c_void_p), ("phi", C.c_void_p), ("ckpt_every", C.c_int), ("rec_grid", C.c_int)]


class RTM2DGpuDesc(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nx", "nz", "npml", "nt")] + \
               [(n, C.c_float) for n in ("dx", "dz", "dt", "favg", "pfac")] + \
               [(n, C.c_int) for n in ("wtype", "ns", "fs", "ds", "zs", "mute_tt", "nangle", "dangle", "dcdp")]


class RTM2DDesc(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nx", "nz", "npd", "nt")] + \
               [(n, C.c_float) for n in ("dx", "dz", "dt_ms", "favg", "pfac")] + \
               [("zs", C.c_int), ("ns", C.c_int), ("shot_x", C.POINTER(C.c_int)),
                ("shot_nxs", C.POINTER(C.c_int)), ("laplace", C.c_int), ("tile_z", C.c_int), ("tile_x", C.c_int),
                ("mode", C.c_int)]


_lib = None
_vp = C.c_void_p
_i, _f = C.c_int, C.c_float


def lib():
    """Load libgeofd.so, declaring every exported entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH):
        raise RuntimeError("libgeofd.so is not built (run geophysics_gb300.build.build() or "
                           "__graft_entry__.build()); there is no CPU fallback")
    L = C.CDLL(LIBPATH)
    sig = {
        "geo_version": (C.c_char_p, []),
        "geo_strerror": (C.c_char_p, [_i]),
        "geo_last_error": (C.c_char_p, []),
        "geo_launch_count": (C.c_longlong, []),
        "geo_fd2d_shot": (_i, [C.POINTER(FD2DDesc), _vp, _vp, _vp, _vp, _vp, _i, _i, _vp]),
        "geo_fd2d_shot_noalloc": (_i, [C.POINTER(FD2DDesc), _vp, _vp, _vp, _vp, _vp]),
        "geo_fd2d_noalloc_limit": (C.c_size_t, []),
        "geo_fd3d_plan_create": (_i, [C.POINTER(_vp), C.POINTER(FD3DDesc)]),
        "geo_fd3d_plan_destroy": (_i, [_vp]),
        "geo_fd3d_set_model": (_i, [_vp, _vp, _vp, _vp, _i, _vp]),
        "geo_fd3d_set_tilt": (_i, [_vp, _vp, _vp, _i, _vp]),
        "geo_fd3d_run_shot": (_i, [_vp, _i, _vp, _i, _vp]),
        "geo_fd3d_time_steps": (_i, [_vp, _i, C.POINTER(_f), _vp]),
        "geo_fd3d_get_fields": (_i, [_vp, _vp, _vp, _i, _vp]),
        "geo_fd3d_shot": (_i, [C.POINTER(FD3DDesc), _i, _vp, _vp, _vp, _vp, _i, _vp]),
        "geo_rtm2d_batch": (_i, [C.POINTER(RTM2DDesc), _vp, _vp, _vp, _vp, _vp, _i, _vp]),
        "geo_rtm2d_batch_adcig": (_i, [C.POINTER(RTM2DDesc), _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp]),
        "geo_rtm3d": (_i, [C.POINTER(RTM3DDesc), _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp]),
        "geo_rtm3d_adcig": (_i, [C.POINTER(RTM3DDesc), _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp]),
        "geo_su_read": (_i, [C.c_char_p, _i, _i, _i, _vp, _vp]),
        "geo_su_write": (_i, [C.c_char_p, _i, _i, _f, _i, _vp, _vp]),
        "geo_su_replace_data": (_i, [C.c_char_p, C.c_char_p, C.c_char_p, _i, _i]),
        "geo_rtm2d_gpu": (_i, [C.POINTER(RTM2DGpuDesc)] + [_vp] * 9 + [_i, _vp]),
        "geo_rtm2d_tti": (_i, [C.POINTER(RTM2DGpuDesc)] + [_vp] * 9 + [_i, _vp]),
        "geo_smooth_lines": (_i, [_vp, _i, C.c_longlong, C.c_longlong, C.c_longlong, _i, _i, _vp]),
        "geo_smooth2d": (_i, [_i, _i, _i, _i, _vp, _i, _vp]),
        "geo_adcig_smooth_stack": (_i, [_i, _i, _i, _i, _vp, _vp, _i, _vp]),
        "geo_mute_direct": (_i, [_i, _i, _f, _f, _f, _f, _i, _i, _i, _i, _f, _f, _i, _vp, _i, _vp]),
        "geo_smooth_model3d": (_i, [_i, _i, _i, _i, _i, _vp, _i, _vp]),
        "geo_smooth_model2d": (_i, [_i, _i, _i, _i, _vp, _i, _vp]),
        "geo_tti2d_shot": (_i, [C.POINTER(FD2DDesc), _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _vp]),
        "geo_ae_create": (_i, [C.POINTER(_vp), C.c_ulonglong]),
        "geo_ae_destroy": (_i, [_vp]),
        "geo_ae_num_params": (C.c_size_t, []),
        "geo_ae_get_params": (_i, [_vp, _vp]),
        "geo_ae_set_params": (_i, [_vp, _vp]),
        "geo_ae_reserve": (_i, [_vp, C.c_longlong]),
        "geo_ae_num_blocks": (C.c_longlong, [_vp]),
        "geo_ae_add_blocks": (_i, [_vp, _vp, C.c_longlong, _i]),
        "geo_ae_add_shot": (_i, [_vp, _vp, _i, _i, _i, _f, _vp]),
        "geo_ae_train": (_i, [_vp, _i, _i, _f, _vp, _vp]),
        "geo_ae_eval": (_i, [_vp, _vp, _i, _vp, C.POINTER(C.c_double), _vp, _i, _vp]),
        "geo_ae_roundtrip": (_i, [_vp, _i, _i, _i, _vp, _vp, _i, C.POINTER(_i), _vp]),
        "geo_ae_set_escape": (_i, [_vp, _f, _f]),
        "geo_ae_stats": (_i, [_vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
        "geo_tc_gemm_bf16": (_i, [_i, _i, _i, _vp, _vp, _vp, _i, _vp, _i, _vp]),
        "geo_laplace2d": (_i, [_i, _i, _vp, _vp, _i, _vp]),
        "geo_laplace3d": (_i, [_i, _i, _i, _vp, _vp, _i, _vp]),
        "geo_par_load": (_i, [C.c_char_p, C.POINTER(_vp)]),
        "geo_par_get_int": (_i, [_vp, C.c_char_p, C.POINTER(_i)]),
        "geo_par_get_float": (_i, [_vp, C.c_char_p, C.POINTER(_f)]),
        "geo_par_get_string": (_i, [_vp, C.c_char_p, C.c_char_p, _i]),
        "geo_par_free": (None, [_vp]),
        "geo_selftest_bounded_wait": (_i, [_i, C.POINTER(_i), _vp]),
        "geo_selftest_conversions": (_i, [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong),
                                          C.POINTER(C.c_longlong), _vp]),
        "geo_fd2d": (_i, [_vp, _i, _vp, _vp]),
        "geo_fd3d": (_i, [_vp, _i, _vp, _vp]),
        "geo_rtm2d": (_i, [_vp, _i, _vp, _vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    for name in ("GPU_vti2dfd", "CPU_vti2dfd"):
        fn = getattr(L, name)
        fn.restype = None
        fn.argtypes = [_i] * 6 + [C.c_char_p] * 3 + [_i] * 5 + [C.c_char_p] * 2 + [_i] * 3
    L.GPU_vti3dfd.restype = None
    L.GPU_vti3dfd.argtypes = [_i] * 8 + [C.c_char_p] * 3 + [_i] * 8 + [C.c_char_p] * 2 + [_i] * 3
    _lib = L
    return L


def check(status, where):
    if status != GEO_OK:
        raise GeoError(status, where, lib().geo_last_error().decode(errors="replace"))
