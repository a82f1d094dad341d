"""ctypes mirror of ``include/sharpray.h``: struct layouts, status codes and function prototypes.

Loading fails loudly (ImportError with the build command) when the native library has not been
built: there is no pure-Python fallback for any part of the render path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libsharpray_gb300.so"

SR_OK = 0
SR_ERR_INVALID_ARG = 1
SR_ERR_STATE = 2
SR_ERR_CUDA = 3
SR_ERR_OUT_OF_MEMORY = 4
SR_ERR_DEVICE = 5
SR_ERR_IO = 6

SR_SHAPE_MESH = 0
SR_SHAPE_SPHERE = 1
SR_SHAPE_AABOX = 2

SR_AOV_NORMAL, SR_AOV_DEPTH, SR_AOV_VARIANCE, SR_AOV_SAMPLES, SR_AOV_UV = 0, 1, 2, 3, 4
SR_ALIGN_TOP_LEFT, SR_ALIGN_CENTER = 0, 1
SR_ADJOINT_ALBEDO, SR_ADJOINT_ROUGHNESS, SR_ADJOINT_FOG_DENSITY = 0, 1, 2
SR_ADJOINT_REPLAY_WAVEFRONT, SR_ADJOINT_REPLAY_PIXEL = 0, 1
SR_TEXTURE_SRGB = 0
SR_TEXTURE_LINEAR = 1
SR_TEXTURE_HDR = 2

SR_BVH_BUILD_HOST = 0
SR_BVH_BUILD_DEVICE = 1

SR_RENDER_AUTO = 0
SR_RENDER_MEGAKERNEL = 1
SR_RENDER_WAVEFRONT = 2
SR_RENDER_WAVEFRONT_GRAPH = 3

SR_TONEMAP_REINHARD = 0
SR_TONEMAP_LINEAR_SMOOTH = 1

COUNTER_NAMES = [
    "sample", "sample_bounce", "scene_trace", "scene_occlude", "tlas_node", "tlas_shape", "blas_node",
    "blas_shape", "hit_inflate", "tex_sample", "cdf_probe", "light_sample", "env_lookup",
]
SR_COUNTER_COUNT = len(COUNTER_NAMES)

_f3 = C.c_float * 3
_f4 = C.c_float * 4
_f2 = C.c_float * 2


class SrTriangle(C.Structure):
    _fields_ = [("pos_a", _f3), ("ab", _f3), ("ac", _f3), ("norm_a", _f3), ("norm_b", _f3), ("norm_c", _f3),
                ("tan_a", _f4), ("tan_b", _f4), ("tan_c", _f4), ("uv_a", _f2), ("uv_b", _f2), ("uv_c", _f2)]


# numpy view of an SrTriangle array: 36 float32 per triangle.
TRIANGLE_FLOATS = 36
assert C.sizeof(SrTriangle) == TRIANGLE_FLOATS * 4


class SrTransform(C.Structure):
    _fields_ = [("pos", _f3), ("rot", _f4), ("scale", _f3)]


class SrMaterial(C.Structure):
    _fields_ = [("albedo", _f3), ("roughness", C.c_float), ("metallic", C.c_float), ("transparency", C.c_float),
                ("ior", C.c_float), ("radiance", _f3), ("color_texture", C.c_int32),
                ("roughness_texture", C.c_int32), ("metallic_texture", C.c_int32), ("normal_texture", C.c_int32)]


class SrShape(C.Structure):
    _fields_ = [("kind", C.c_int32), ("mesh", C.c_int32), ("params", C.c_float * 6)]


class SrFog(C.Structure):
    _fields_ = [("density", C.c_float), ("color", _f3), ("anisotropy", C.c_float), ("height_falloff", C.c_float),
                ("top_height", C.c_float)]


class SrSkyProcedural(C.Structure):
    _fields_ = [("top", _f3), ("middle", _f3), ("bottom", _f3), ("sun_dir", _f3), ("sun_radiance", _f3),
                ("sun_angle", C.c_float)]


class SrView(C.Structure):
    _fields_ = [("transform", SrTransform), ("fov", C.c_float), ("near_plane", C.c_float)]


class SrRenderParams(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("block_size", C.c_uint32),
                ("min_samples", C.c_uint32), ("max_samples", C.c_uint32), ("variance_threshold", C.c_float),
                ("bounces", C.c_uint32), ("indirect_clamp", C.c_float)]


class SrAovs(C.Structure):
    _fields_ = [("radiance", C.c_void_p), ("radiance_fog", C.c_void_p), ("normals", C.c_void_p),
                ("uv", C.c_void_p), ("depth", C.c_void_p), ("samples", C.c_void_p), ("variance", C.c_void_p)]


class SrComposeParams(C.Structure):
    _fields_ = [("tonemapper", C.c_int32), ("exposure", C.c_float), ("denoise_radius", C.c_float),
                ("denoise_strength", C.c_float), ("denoise_strength_max", C.c_float),
                ("denoise_luminance_boost", C.c_float), ("denoise_luminance_limit", C.c_float),
                ("denoise_normal_limit", C.c_float), ("denoise_depth_limit", C.c_float),
                ("denoise_fog_radius", C.c_float), ("denoise_fog_strength", C.c_float)]


class SrTuning(C.Structure):
    _fields_ = [("trace_blocks_per_sm", C.c_int32), ("fog_shade_blocks_per_sm", C.c_int32),
                ("surface_shade_blocks_per_sm", C.c_int32), ("tail_divisor", C.c_uint32), ("ms", C.c_float),
                ("default_ms", C.c_float), ("max_bounce_iterations", C.c_uint32), ("max_traversal_steps", C.c_uint32),
                ("trace_block_threads", C.c_uint32), ("max_slots", C.c_uint32)]


class SrAovImageParams(C.Structure):
    _fields_ = [("variance_threshold", C.c_float), ("min_samples", C.c_uint32), ("max_samples", C.c_uint32)]


class SrOverlayLine(C.Structure):
    _fields_ = [("a", _f3), ("b", _f3), ("color", _f3), ("depth_test", C.c_int32), ("depth_bias", C.c_float)]


class SrOverlayText(C.Structure):
    _fields_ = [("text", C.c_char_p), ("in_world", C.c_int32), ("world_pos", _f3), ("screen_pos", C.c_int32 * 2),
                ("color", _f3), ("align", C.c_int32)]


class SrFont(C.Structure):
    _fields_ = [("glyphs", C.c_void_p), ("first_char", C.c_int32), ("last_char", C.c_int32)]


_P = C.c_void_p
_I = C.c_int
_U = C.c_uint32
_F = C.c_float

# name -> (restype, argtypes); every function declared in include/sharpray.h.
PROTOTYPES = {
    "sr_version": (C.c_char_p, []),
    "sr_last_error_message": (C.c_char_p, []),
    "sr_ctx_create": (_I, [_I, C.POINTER(_P)]),
    "sr_ctx_destroy": (_I, [_P]),
    "sr_triangles_from_corners": (_I, [_P, _P, _P, _U, C.c_int32, _P]),
    "sr_texture_create": (_I, [_P, _P, _U, _U, C.c_int32, _F, _F, C.POINTER(C.c_int32)]),
    "sr_mesh_create": (_I, [_P, _P, _U, C.POINTER(C.c_int32)]),
    "sr_ctx_set_bvh_build": (_I, [_P, C.c_int32]),
    "sr_bvh_build": (_I, [_P, _P, _U, _F, _F, C.c_int32, C.c_int32, _P, _P, _P, C.POINTER(_U)]),
    "sr_mesh_bvh_size": (_I, [_P, C.c_int32, C.POINTER(_U), C.POINTER(_U)]),
    "sr_image_load": (_I, [C.c_char_p, C.POINTER(_U), C.POINTER(_U), C.POINTER(_U), _P, C.c_uint64]),
    "sr_texture_load": (_I, [_P, C.c_char_p, C.c_int32, _F, C.c_int32, _F, _F, C.POINTER(C.c_int32)]),
    "sr_obj_load": (_I, [_P, C.c_char_p, _P, _P, C.c_int32, C.POINTER(_U)]),
    "sr_texture_export": (_I, [_P, C.c_int32, C.POINTER(_U), C.POINTER(_U), _P]),
    "sr_mesh_export": (_I, [_P, C.c_int32, C.POINTER(_U), _P]),
    "sr_scene_object_count": (_I, [_P, C.POINTER(_U)]),
    "sr_scene_object_info": (_I, [_P, _U, _P, _P, _P, C.c_char_p, _U]),
    "sr_mesh_bvh_export": (_I, [_P, C.c_int32, _P, _P, _P]),
    "sr_scene_create": (_I, [_P, C.POINTER(_P)]),
    "sr_scene_destroy": (_I, [_P]),
    "sr_scene_set_sky_texture": (_I, [_P, C.c_int32, _F, _F]),
    "sr_scene_set_sky_procedural": (_I, [_P, C.POINTER(SrSkyProcedural)]),
    "sr_scene_set_fog": (_I, [_P, C.POINTER(SrFog)]),
    "sr_scene_add_object": (_I, [_P, C.POINTER(SrTransform), C.POINTER(SrMaterial), C.POINTER(SrShape),
                                 C.POINTER(C.c_int32)]),
    "sr_scene_build": (_I, [_P]),
    "sr_scene_bvh_size": (_I, [_P, C.POINTER(_U), C.POINTER(_U)]),
    "sr_scene_bvh_export": (_I, [_P, _P, _P, _P]),
    "sr_scene_trace": (_I, [_P, _P, _U, _P, _P, _P, _P]),
    "sr_render": (_I, [_P, C.POINTER(SrView), C.POINTER(SrRenderParams), C.POINTER(SrAovs)]),
    "sr_render_device": (_I, [_P, C.POINTER(SrView), C.POINTER(SrRenderParams), C.POINTER(SrAovs), _P]),
    "sr_render_compose": (_I, [_P, C.POINTER(SrView), C.POINTER(SrRenderParams), C.POINTER(SrComposeParams),
                               C.POINTER(SrAovs), _P]),
    "sr_scene_set_render_mode": (_I, [_P, C.c_int32]),
    "sr_scene_render_info": (_I, [_P, C.POINTER(_U), C.POINTER(_U)]),
    "sr_scene_set_counting": (_I, [_P, C.c_int32]),
    "sr_scene_counters": (_I, [_P, _P]),
    "sr_scene_set_kernel_timing": (_I, [_P, C.c_int32]),
    "sr_scene_trace_time": (_I, [_P, C.POINTER(C.c_float), C.POINTER(_U)]),
    "sr_compose": (_I, [_P, C.POINTER(SrAovs), _U, _U, C.POINTER(SrComposeParams), _P]),
    "sr_compose_device": (_I, [_P, C.POINTER(SrAovs), _U, _U, C.POINTER(SrComposeParams), _P, _P]),
    "sr_compose_device_static": (_I, [_P, C.POINTER(SrAovs), _U, _U, C.POINTER(SrComposeParams), _P, _P]),
    "sr_compose_float_device": (_I, [_P, C.POINTER(SrAovs), _U, _U, C.POINTER(SrComposeParams), _P, _P, _P]),
    "sr_preview": (_I, [_P, C.POINTER(SrAovs), _U, _U, C.POINTER(SrComposeParams), _P]),
    "sr_render_batch": (_I, [_P, _P, _P, _P, _U, _P]),
    "sr_render_progress": (_I, [_P, C.POINTER(_U), C.POINTER(_U)]),
    "sr_scene_set_tuning": (_I, [_P, _P]),
    "sr_scene_set_seed": (_I, [_P, _U]),
    "sr_scene_set_adjoint_replay": (_I, [_P, C.c_int32]),
    "sr_render_checkpointed": (_I, [_P, _P, _P, _P, _P, C.POINTER(C.c_uint64)]),
    "sr_adjoint_checkpointed": (_I, [_P, _P, C.c_int32, _P, C.c_int32, _P, _P, _P]),
    "sr_scene_release_checkpoint": (_I, [_P]),
    "sr_scene_get_seed": (_I, [_P, C.POINTER(_U)]),
    "sr_scene_get_tuning": (_I, [_P, C.POINTER(SrTuning)]),
    "sr_scene_autotune": (_I, [_P, C.POINTER(SrView), C.POINTER(SrRenderParams), _U, C.POINTER(SrTuning)]),
    "sr_aov_image": (_I, [_P, C.POINTER(SrAovs), _U, _U, C.c_int32, C.POINTER(SrAovImageParams), _P]),
    "sr_aov_image_device": (_I, [_P, C.POINTER(SrAovs), _U, _U, C.c_int32, C.POINTER(SrAovImageParams), _P, _P]),
    "sr_overlay_draw": (_I, [_P, _P, _U, _U, C.POINTER(SrView), _P, _P, _U, _P, _U, C.POINTER(SrFont)]),
    "sr_overlay_draw_device": (_I, [_P, _P, _U, _U, C.POINTER(SrView), _P, _P, _U, _P, _U, C.POINTER(SrFont), _P]),
    "sr_image_save": (_I, [C.c_char_p, _U, _U, _P]),
    "sr_adjoint_albedo": (_I, [_P, C.POINTER(SrView), C.POINTER(SrRenderParams), C.POINTER(SrAovs), _P, C.c_int32,
                               _P, _P, _P]),
    "sr_adjoint_texture": (_I, [_P, C.POINTER(SrView), C.POINTER(SrRenderParams), C.POINTER(SrAovs), _P, C.c_int32,
                                C.c_int32, _P, _P, _P]),
    "sr_adjoint_all": (_I, [_P, C.POINTER(SrView), C.POINTER(SrRenderParams), C.POINTER(SrAovs), _P, C.c_int32, _P,
                            C.c_int32, _P, _P, _P, _P]),
    "sr_scene_update_texture": (_I, [_P, C.c_int32, _P]),
    "sr_scene_update_fog_density": (_I, [_P, C.c_float]),
    "sr_scene_update_texture_device": (_I, [_P, C.c_int32, _P, _P]),
}


class SharpRayError(RuntimeError):
    """A non-zero status from the native library, with its message."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


class StateError(SharpRayError):
    """Build-state misuse (the reference raises InvalidOperationException)."""


_lib = None


def load(path: Path | str | None = None):
    """Load the native library once; raises ImportError if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"native library {p} is missing: build it with `python -m sharpray_gb300.build` "
                          "(there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code: int) -> None:
    if code != SR_OK:
        msg = _lib.sr_last_error_message().decode(errors="replace") if _lib else ""
        cls = StateError if code == SR_ERR_STATE else SharpRayError
        raise cls(code, msg)


def ptr(a: np.ndarray | None):
    """Raw data pointer of a C-contiguous numpy array (None -> NULL)."""
    if a is None:
        return None
    assert a.flags.c_contiguous, "arrays passed to the C ABI must be C-contiguous"
    return a.ctypes.data
