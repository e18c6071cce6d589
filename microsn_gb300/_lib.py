"""ctypes binding of the C ABI declared in include/microlc_gb300.h.

The library is built in-tree (microsn_gb300/libmicrolc_gb300.so); loading fails
loudly when it is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmicrolc_gb300.so")

MLC_OK, MLC_ERR_ARG, MLC_ERR_OOM, MLC_ERR_CUDA, MLC_ERR_TIMEOUT, MLC_ERR_UNSUPPORTED, MLC_ERR_LIMIT = range(7)
MLC_F64, MLC_F32 = 0, 1
MLC_CONV_FUSED, MLC_CONV_PLAIN = 0, 1
SHAPES = {"uniform": 0, "gaussian": 1, "gaussian_hole": 2, "thermal_hole": 3, "wavy": 4, "exponential": 5,
          "limb_darkened": 6}


class MlcProfile(C.Structure):
    _fields_ = [("shape", C.c_int), ("ref_compat", C.c_int), ("rhalf", C.c_double), ("pix", C.c_double),
                ("incl", C.c_double), ("orient", C.c_double), ("Rin", C.c_double), ("a", C.c_double),
                ("u", C.c_double)]


class MlcTracks(C.Structure):
    _fields_ = [("ntracks", C.c_int), ("nepochs", C.c_int64), ("x0", C.c_void_p), ("y0", C.c_void_p),
                ("phi", C.c_void_p), ("v", C.c_void_p), ("off", C.c_void_p), ("t", C.c_void_p)]


MLC_IO_HOST, MLC_ASYNC, MLC_GRAPH = 1, 2, 4


class MlcPairStats(C.Structure):
    _fields_ = [("delta", C.c_double), ("threshold", C.c_double), ("refined", C.c_longlong),
                ("candidates", C.c_longlong), ("passes", C.c_int), ("below", C.c_longlong),
                ("above", C.c_longlong)]


class MlcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"mlc error {code}: {msg}")
        self.code = code


vp = C.c_void_p
i32, i64, f64 = C.c_int, C.c_int64, C.c_double
P_i32 = C.POINTER(C.c_int)
P_f64 = C.POINTER(C.c_double)
P_u32 = C.POINTER(C.c_uint32)
P_u64 = C.POINTER(C.c_uint64)

# name -> (restype, argtypes); every entry returns int status unless noted
SIGNATURES = {
    "mlc_version": (i32, []),
    "mlc_ctx_create": (i32, [i32, vp, C.POINTER(vp)]),
    "mlc_ctx_destroy": (i32, [vp]),
    "mlc_ctx_set_stream": (i32, [vp, vp]),
    "mlc_ctx_synchronize": (i32, [vp]),
    "mlc_ctx_last_error": (C.c_char_p, [vp]),
    "mlc_ctx_workspace_bytes": (C.c_size_t, [vp]),
    "mlc_ctx_launch_count": (C.c_ulonglong, [vp]),
    "mlc_ctx_set_timing": (i32, [vp, i32]),
    "mlc_ctx_set_autotune": (i32, [vp, i32]),
    "mlc_ctx_autotune_report": (i32, [vp, C.c_char_p, i32]),
    "mlc_ctx_kernel_times": (i32, [vp, C.c_char_p, i32, vp, vp, i32, i32]),
    "mlc_map_refresh": (i32, [vp, vp]),
    "mlc_map_set_fft": (i32, [vp, i32]),
    "mlc_profile_dims": (i32, [C.POINTER(MlcProfile), P_i32]),
    "mlc_profile_raster": (i32, [C.POINTER(MlcProfile), vp, C.c_long, P_i32]),
    "mlc_map_create": (i32, [vp, vp, i32, i32, i32, i32, i32, C.POINTER(vp)]),
    "mlc_map_destroy": (i32, [vp]),
    "mlc_map_data": (i32, [vp, C.POINTER(vp)]),
    "mlc_map_prepare": (i32, [vp, vp]),
    "mlc_convolve": (i32, [vp, vp, C.POINTER(MlcProfile), i32, vp]),
    "mlc_convolve_direct": (i32, [vp, vp, C.POINTER(MlcProfile), i32, vp]),
    "mlc_expanding_source": (i32, [vp, vp, vp, i32, C.POINTER(MlcProfile), f64, i32, vp, vp, i32, vp, vp]),
    "mlc_sample_nearest": (i32, [vp, vp, i32, i32, i32, i32, i32, vp, vp, vp, vp]),
    "mlc_sample_tracks": (i32, [vp, vp, i32, i32, i32, i32, i32, vp, vp, vp, vp, vp, vp, i32, vp]),
    "mlc_chi2_offset": (i32, [vp, i32, i32, i32, vp, vp, vp, vp, vp]),
    "mlc_interleave_maps": (i32, [vp, vp, i32, i32, i32, i32, i32, vp]),
    "mlc_convolve_sample_tracks": (i32, [vp, vp, vp, i32, C.POINTER(MlcProfile), C.POINTER(MlcTracks), i32, i32, vp,
                                         i32]),
    "mlc_ctx_join": (i32, [vp]),
    "mlc_convolve_many": (i32, [vp, vp, i32, C.POINTER(MlcProfile), i32, vp, C.c_longlong, i32]),
    "mlc_sample_expanding": (i32, [vp, vp, i32, i32, i32, i32, i32, i32, vp, vp, vp, vp, vp, i32, vp]),
    "mlc_track_chi2_offset": (i32, [vp, vp, i32, i32, i32, i32, i32, i32, vp, vp, vp, vp, i32, vp, vp, vp, vp, vp]),
    "mlc_fit_raster": (i32, [f64, f64, i32, vp, vp, vp, vp]),
    "mlc_radius_stack": (i32, [vp, vp, i32, vp, f64, i32, vp]),
    "mlc_track_fit": (i32, [vp, vp, i32, i32, i32, i32, vp, i32, vp, vp, vp, vp, vp, vp, vp, vp]),
    "mlc_flux_ratio_chi2": (i32, [vp, vp, vp, vp, vp, i32, i32, i32, vp, vp]),
    "mlc_find_indices": (i32, [vp, vp, i32, i32, vp]),
    "mlc_map_binned_mpd": (i32, [vp, vp, i32, f64, f64, vp, vp]),
    "mlc_mpd_divide": (i32, [vp, i32, vp, vp, i32, vp, vp, i32, vp, vp]),
    "mlc_ctx_set_chunk_bytes": (i32, [vp, C.c_size_t]),
    "mlc_sample_tracks_interleaved": (i32, [vp, vp, i32, i32, i32, i32, i32, i32, vp, vp, vp, vp, vp, vp, i32, vp]),
    "mlc_pair_setup": (i32, [vp, i32, i32, vp, vp, i32, vp, vp, vp, vp]),
    "mlc_pair_chi2_ratio": (i32, [vp, i32, vp, vp, vp, vp, vp, vp, i32, i32, vp, vp, vp, vp, vp, vp]),
    "mlc_bin_chi2": (i32, [vp, i32, vp, vp, vp, vp, vp]),
    "mlc_pair_bin_fused": (i32, [vp, i32, vp, vp, vp, vp, vp, vp, i32, i32, vp, vp, vp, vp, i32, vp, vp, vp,
                                 vp]),
    "mlc_sort_f64_u32": (i32, [vp, C.c_long, vp, vp]),
    "mlc_histogram_f64": (i32, [vp, C.c_long, vp, i32, f64, f64, i32, vp]),
    "mlc_pair_chi2_magdiff": (i32, [vp, i32, i32, i32, i32, vp, vp, vp, vp, i32, i32, f64, f64, vp, i32, vp, vp, vp,
                                    vp, vp]),
    "mlc_pair_chi2_magdiff_list": (i32, [vp, i32, i32, i32, vp, vp, vp, vp, i32, C.c_long, vp, vp, vp]),
    "mlc_pair_side_curves": (i32, [vp, i32, i32, vp, vp, vp, i32, vp]),
    "mlc_pair_side_expanding": (i32, [vp, vp, i32, i32, i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, i32, vp]),
    "mlc_pair_side_destroy": (i32, [vp]),
    "mlc_ctx_tune_set": (i32, [vp, C.c_char_p, i32]),
    "mlc_ctx_set_profile_cache": (i32, [vp, C.c_longlong]),
    "mlc_pair_chi2_sides": (i32, [vp, vp, vp, i32, f64, f64, vp, i32, vp, vp, vp, vp, vp]),
    "mlc_histogram_f64_noalloc": (i32, [vp, C.c_long, vp, i32, f64, f64, i32, vp]),
    "mlc_selftest_wait_timeout": (i32, [vp, C.c_uint, vp]),
    "mlc_setup_chi2": (i32, [f64, f64, f64, f64, i32, vp, vp, vp, i32, vp, i32, P_i32, vp, vp, vp, vp, vp, vp,
                             P_f64]),
    "mlc_locations_grid": (i32, [i32, i32, i32, vp, vp]),
    "mlc_locations_random": (i32, [i32, i32, i32, i32, vp, vp]),
    "mlc_bin_edges": (i32, [i32, f64, f64, i32, vp]),
    "mlc_trapezium": (f64, [i32, vp, vp, vp]),
    "mlc_read_gerlumph": (i32, [C.c_char_p, P_i32, P_f64, vp, vp, C.c_long]),
    "mlc_host_alloc": (i32, [C.c_size_t, C.POINTER(C.c_void_p)]),
    "mlc_host_free": (i32, [vp]),
    "mlc_rayshoot": (i32, [vp, vp, i32, f64, f64, f64, f64, f64, C.c_long, C.c_long, f64, i32, vp]),
}

_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run microsn_gb300.build.build() (no CPU fallback exists)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib
