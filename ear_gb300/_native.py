"""ctypes view of the C ABI declared in include/ear_gb300.h.

The structures below mirror the header field for field.  ``lib()`` loads
``ear_gb300/lib/libear_gb300.so`` (built in-tree by ``ear_gb300.build``)
and raises if it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libear_gb300.so"

EAR_OK = 0
EAR_ERR_INVALID_ARG = 1
EAR_ERR_OUT_OF_MEMORY = 2
EAR_ERR_CUDA = 3
EAR_ERR_DEVICE_BUDGET = 4
EAR_ERR_STATE = 5
EAR_ERR_UNSUPPORTED = 6

EAR_FLAG_EXACT = 0x1
EAR_FLAG_RAW = 0x2
EAR_FLAG_NO_DIRECT = 0x4

EAR_BVH_DEFAULT = 0
EAR_BVH_LBVH = 1
EAR_BVH_PLOC = 2

EAR_REFERENCE_MAX_BOUNCES = 999
EAR_REFERENCE_CUTOFF = 1e-8
SAMPLE_RATE = 44100

F3 = C.c_float * 3


class EarMaterial(C.Structure):
    _fields_ = [("reflection", F3), ("refraction", F3), ("specularity", F3),
                ("has_refraction", C.c_int32), ("has_specularity", C.c_int32)]


class EarSceneDesc(C.Structure):
    _fields_ = [("num_triangles", C.c_int64), ("vertices", C.POINTER(C.c_float)),
                ("material_ids", C.POINTER(C.c_int32)), ("num_materials", C.c_int32),
                ("materials", C.POINTER(EarMaterial)), ("device", C.c_int32)]


class EarBvhOpts(C.Structure):
    _fields_ = [("box_pad", C.c_float), ("max_leaf_size", C.c_int32), ("builder", C.c_int32),
                ("ploc_radius", C.c_int32), ("width", C.c_int32), ("visibility_order", C.c_int32),
                ("visibility_map", C.c_int32), ("reserved", C.c_int32)]


class EarRecorder(C.Structure):
    _fields_ = [("channels", C.c_int32), ("location", F3), ("right_ear", F3),
                ("head_size", C.c_float), ("head_absorption", F3)]


class EarSource(C.Structure):
    _fields_ = [("location", F3), ("gain", C.c_float), ("num_emitter_triangles", C.c_int64),
                ("emitter_vertices", C.POINTER(C.c_float))]


class EarRenderParams(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("context", C.c_uint32), ("bands_mask", C.c_uint32),
                ("num_rays", C.c_uint64), ("max_bounces", C.c_int32), ("num_bins", C.c_int32),
                ("cutoff", C.c_double), ("air_absorption", F3), ("dry_level", C.c_float),
                ("flags", C.c_uint32), ("traverse_budget", C.c_int32), ("stream", C.c_void_p),
                ("first_ray", C.c_uint64)]


class EarRenderStats(C.Structure):
    _fields_ = [("rays", C.c_uint64), ("segments", C.c_uint64), ("shadow_queries", C.c_uint64),
                ("contributions", C.c_uint64), ("sampler_overflows", C.c_uint64),
                ("node_visits", C.c_uint64), ("triangle_tests", C.c_uint64),
                ("splat_bins", C.c_uint64), ("kernel_ms", C.c_double),
                ("map_entries", C.c_uint64), ("map_build_ms", C.c_double),
                ("map_bytes", C.c_uint64), ("map_res", C.c_int32), ("reserved1", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class EarHistograms(C.Structure):
    _fields_ = [("data", C.c_void_p), ("first_sample", C.c_void_p), ("last_sample", C.c_void_p),
                ("on_device", C.c_int32), ("reserved0", C.c_int32),
                ("raw_first_sample", C.c_void_p), ("raw_last_sample", C.c_void_p)]


class EarBatchJob(C.Structure):
    _fields_ = [("scene", C.c_int32), ("num_recorders", C.c_int32),
                ("recorders", C.POINTER(EarRecorder)), ("source", F3), ("gain", C.c_float),
                ("num_rays", C.c_uint64), ("context", C.c_uint32), ("reserved", C.c_int32)]


class EarBatchConfig(C.Structure):
    _fields_ = [("block", C.c_int32), ("blocks_per_sm", C.c_int32), ("max_leaf_size", C.c_int32),
                ("no_graph", C.c_int32), ("bvh_width", C.c_int32), ("reserved", C.c_int32 * 3)]

    def as_dict(self):
        return {"block": self.block, "blocks_per_sm": self.blocks_per_sm,
                "max_leaf_size": self.max_leaf_size, "no_graph": self.no_graph,
                "bvh_width": self.bvh_width}


class EarTuneOpts(C.Structure):
    _fields_ = [("trial_fraction", C.c_double), ("min_trial_rays", C.c_uint64),
                ("tune_leaf_size", C.c_int32), ("repeats", C.c_int32), ("cache_path", C.c_char_p),
                ("tune_width", C.c_int32), ("reserved", C.c_int32 * 3)]


class EarTuneResult(C.Structure):
    _fields_ = [("best", EarBatchConfig), ("best_ms", C.c_float), ("default_ms", C.c_float),
                ("candidates", C.c_int32), ("from_cache", C.c_int32)]


EAR_AURAL_DEVICE_MEMORY = 1
EAR_SPLIT_CHUNKED = 2
EAR_CONV_FFT = 0
EAR_CONV_DIRECT = 1


class EarConvContext(C.Structure):
    _fields_ = [("ir", C.c_void_p), ("ir_capacity", C.c_int64), ("ir_first", C.c_int64),
                ("ir_length", C.c_int64), ("ir_next", C.c_void_p), ("ir_next_capacity", C.c_int64),
                ("ir_next_first", C.c_int64), ("ir_next_length", C.c_int64), ("dry", C.c_void_p),
                ("dry_length", C.c_int64), ("offset", C.c_int64)]


class EarConvStats(C.Structure):
    _fields_ = [("kernel_ms", C.c_float), ("launches", C.c_int32), ("fft_points", C.c_int64),
                ("multiply_adds", C.c_double)]


# Every exported symbol of include/ear_gb300.h with its ctypes signature.
SIGNATURES = {
    "ear_last_error": (C.c_char_p, []),
    "ear_version": (C.c_char_p, []),
    "ear_abi_version": (C.c_int32, []),
    "ear_scene_create": (C.c_int, [C.POINTER(EarSceneDesc), C.POINTER(C.c_void_p)]),
    "ear_scene_build_bvh": (C.c_int, [C.c_void_p, C.POINTER(EarBvhOpts)]),
    "ear_scene_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                 C.POINTER(C.c_int32), C.POINTER(C.c_float), C.POINTER(C.c_int64)]),
    "ear_scene_destroy": (None, [C.c_void_p]),
    "ear_scene_sah_cost": (C.c_int, [C.c_void_p, C.c_int32, C.c_float, C.c_float,
                                     C.POINTER(C.c_double)]),
    "ear_scene_set_bvh_width": (C.c_int, [C.c_void_p, C.c_int32]),
    "ear_scene_bvh_width": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "ear_num_tracks": (C.c_int32, [C.POINTER(EarRecorder), C.c_int32]),
    "ear_render": (C.c_int, [C.c_void_p, C.POINTER(EarSource), C.POINTER(EarRecorder), C.c_int32,
                             C.POINTER(EarRenderParams), C.POINTER(EarHistograms),
                             C.POINTER(EarRenderStats)]),
    "ear_trace_debug": (C.c_int, [C.c_void_p, C.POINTER(EarSource), C.POINTER(EarRecorder),
                                  C.c_int32, C.POINTER(EarRenderParams), C.c_int32, C.c_int32,
                                  C.c_void_p, C.c_void_p, C.c_void_p]),
    "ear_scene_set_materials": (C.c_int, [C.c_void_p, C.POINTER(EarMaterial), C.c_int32]),
    "ear_render_adjoint": (C.c_int, [C.c_void_p, C.POINTER(EarSource), C.POINTER(EarRecorder),
                                     C.c_int32, C.POINTER(EarRenderParams), C.c_void_p, C.c_int32,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.POINTER(EarRenderStats)]),
    "ear_render_noalloc": (C.c_int, [C.c_void_p, C.POINTER(EarSource), C.POINTER(EarRecorder),
                                     C.c_int32, C.POINTER(EarRenderParams), C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.POINTER(EarRenderStats)]),
    "ear_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(EarBatchJob),
                                   C.c_int32, C.POINTER(EarRenderParams), C.POINTER(C.c_void_p)]),
    "ear_batch_set_config": (C.c_int, [C.c_void_p, C.POINTER(EarBatchConfig)]),
    "ear_batch_get_config": (C.c_int, [C.c_void_p, C.POINTER(EarBatchConfig)]),
    "ear_batch_set_sources": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ear_batch_run": (C.c_int, [C.c_void_p, C.POINTER(EarRenderStats)]),
    "ear_batch_histograms": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(EarHistograms)]),
    "ear_batch_device_view": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_int32),
                                        C.POINTER(C.c_int64), C.c_void_p, C.c_int32]),
    "ear_batch_destroy": (None, [C.c_void_p]),
    "ear_render_batch": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(EarBatchJob),
                                   C.c_int32, C.POINTER(EarRenderParams),
                                   C.POINTER(EarHistograms), C.POINTER(EarRenderStats)]),
    "ear_batch_tune": (C.c_int, [C.c_void_p, C.POINTER(EarTuneOpts), C.POINTER(EarTuneResult)]),
    "ear_track_power": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_float]),
    "ear_track_maximum": (C.c_float, [C.c_void_p, C.c_int32, C.c_int32]),
    "ear_track_multiply": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_float]),
    "ear_track_length": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_float]),
    "ear_track_t60": (C.c_float, [C.c_void_p, C.c_int32, C.c_int32]),
    "ear_statistical_t60": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(EarMaterial),
                                      C.c_float, C.c_void_p]),
    "ear_band_split": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_float), C.c_void_p,
                                 C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_int32]),
    "ear_convolve": (C.c_int, [C.POINTER(EarConvContext), C.c_int32, C.c_int32, C.c_void_p,
                               C.c_int64, C.c_uint32, C.c_void_p, C.c_int32,
                               C.POINTER(EarConvStats)]),
    "ear_convolve_tracks": (C.c_int, [C.POINTER(EarConvContext), C.c_void_p, C.c_int32, C.c_int32,
                                      C.c_void_p, C.c_void_p, C.c_int32, C.c_uint32, C.c_void_p,
                                      C.c_int32, C.POINTER(EarConvStats)]),
    "ear_conv_processed_capacity": (C.c_int64, [C.POINTER(EarConvContext), C.c_int32]),
    "ear_conv_processed_length": (C.c_int64, [C.POINTER(EarConvContext), C.c_int32]),
}

_LIB = None


class EarError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"ear status {status}: {msg}")
        self.status = status


def lib() -> C.CDLL:
    """Load the sm_103a library (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m ear_gb300.build` "
                "(the CUDA path has no fallback)")
        mode = getattr(os, "RTLD_GLOBAL", 0)
        L = C.CDLL(str(LIB_PATH), mode=mode)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def check(status: int) -> None:
    if status != EAR_OK:
        msg = lib().ear_last_error()
        raise EarError(status, msg.decode() if msg else "")
