"""Python host API over the C ABI, mirroring the C# reference's render-path classes.

Names, argument meanings and error behaviour follow the reference:

=========================  ==========================================================
reference (C#)             here
=========================  ==========================================================
``Texture`` texture.cs     :class:`Texture` (``from_srgb`` / ``from_linear`` / ``from_hdr``)
``Mesh`` mesh.cs           :class:`Mesh` (``from_corners`` = ObjLoader triangle path)
``Sphere``/``AABox``       :class:`Sphere`, :class:`AABox`
``Material`` scene.cs      :class:`Material`
``Transform``/``Quat``     :class:`Transform`, :class:`Quat`
``Object`` scene.cs        :class:`Object`
``SkyTexture``/``SkyProcedural``  :class:`SkyTexture`, :class:`SkyProcedural`
``Fog`` scene.cs           :class:`Fog`
``Scene`` scene.cs         :class:`Scene` (``set_sky``/``set_fog``/``add_object``/``build``)
``View`` math.cs           :class:`View`
``Renderer`` renderer.cs   :class:`Renderer` (renders on construction; ``tick`` + AOV arrays)
``Compositor`` compose.cs  :class:`Compositor` (``compose`` / ``preview``)
=========================  ==========================================================

Build-state misuse raises :class:`StateError` (the reference's InvalidOperationException).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from enum import IntEnum
from typing import Optional, Sequence, Union

import numpy as np

from . import _abi
from ._abi import (SharpRayError, SrAovs, SrComposeParams, SrFog, SrMaterial, SrRenderParams, SrShape,
                   SrSkyProcedural, SrTransform, SrView, StateError, check, ptr)

__all__ = [
    "Context", "Texture", "TextureFilter", "Mesh", "Sphere", "AABox", "Material", "Quat", "Transform", "Object",
    "SkyTexture", "SkyProcedural", "Fog", "Scene", "View", "Renderer", "Compositor", "Tonemapper",
    "SharpRayError", "StateError", "load_image", "mesh_triangles", "AovKind", "aov_image", "save_image", "Font",
    "Overlay", "render_batch",
]


def _f32(v) -> np.float32:
    return np.float32(v)


_SRGB_TABLE = None


def _srgb_table() -> np.ndarray:
    global _SRGB_TABLE
    if _SRGB_TABLE is None:
        import ctypes.util
        libm = C.CDLL(ctypes.util.find_library("m") or "libm.so.6")
        libm.powf.restype, libm.powf.argtypes = C.c_float, [C.c_float, C.c_float]
        g = float(np.float32(2.233333333))
        _SRGB_TABLE = np.array([libm.powf(float(np.float32(i) / np.float32(255.0)), g) for i in range(256)],
                               np.float32)
    return _SRGB_TABLE


class Context:
    """One CUDA device + stream; owns textures, meshes and scenes (no reference counterpart)."""

    def __init__(self, device: int = 0):
        self._lib = _abi.load()
        h = C.c_void_p()
        check(self._lib.sr_ctx_create(device, C.byref(h)))
        self.handle = h
        self.device = device

    def set_bvh_build(self, where: int) -> None:
        """Where meshes and scenes build their BVHs: _abi.SR_BVH_BUILD_HOST (default) or
        SR_BVH_BUILD_DEVICE (bit-identical result; no reference counterpart)."""
        check(self._lib.sr_ctx_set_bvh_build(self.handle, int(where)))

    def build_bvh(self, bounds: np.ndarray, cost_traverse: float, cost_intersect: float, bins: int,
                  where: int = _abi.SR_BVH_BUILD_HOST):
        """The reference's Bvh over arbitrary shape bounds (N, 6) = min xyz, max xyz (bvh.cs:58-75).
        Returns (node bounds (M,6), node links (M,2) = child/shapeCount, item permutation (N,))."""
        b = np.ascontiguousarray(bounds, dtype=np.float32).reshape(-1, 6)
        n = b.shape[0]
        nb = np.zeros((max(2 * n, 1), 6), np.float32)
        nl = np.zeros((max(2 * n, 1), 2), np.int32)
        it = np.zeros(n, np.int32)
        cnt = C.c_uint32()
        check(self._lib.sr_bvh_build(self.handle, ptr(b), n, float(cost_traverse), float(cost_intersect), int(bins),
                                     int(where), ptr(nb), ptr(nl), ptr(it), C.byref(cnt)))
        m = cnt.value
        return nb[:m], nl[:m], it

    def close(self) -> None:
        if self.handle:
            self._lib.sr_ctx_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class TextureFilter(IntEnum):
    Bilinear = 0
    Point = 1


class Texture:
    """Float RGB texels, repeat-wrapped with tiling (texture.cs:6-69)."""

    def __init__(self, ctx: Context, texels: np.ndarray, filter: TextureFilter = TextureFilter.Bilinear,
                 tiling: Sequence[float] = (1.0, 1.0)):
        t = np.ascontiguousarray(texels, dtype=np.float32)
        if t.ndim != 3 or t.shape[2] != 3:
            raise ValueError("texels must be (height, width, 3)")
        self.ctx, self.texels = ctx, t
        self.height, self.width = t.shape[:2]
        self.filter, self.tiling = TextureFilter(filter), (float(tiling[0]), float(tiling[1]))
        out = C.c_int32()
        check(ctx._lib.sr_texture_create(ctx.handle, ptr(t), self.width, self.height, int(self.filter),
                                         self.tiling[0], self.tiling[1], C.byref(out)))
        self.id = out.value

    @classmethod
    def load(cls, ctx: Context, path, encoding: int = _abi.SR_TEXTURE_SRGB,
             max_luminance: float = float(np.finfo(np.float32).max), filter: TextureFilter = TextureFilter.Bilinear,
             tiling: Sequence[float] = (1.0, 1.0)) -> "Texture":
        """Texture.FromSrgb/FromLinear(Image.Load(path)) for .tga or FromHdr(ImageHdr.Load(path)) for
        .hdr (texture.cs:138-163), parsed by the library."""
        out = C.c_int32()
        check(ctx._lib.sr_texture_load(ctx.handle, str(path).encode(), int(encoding), float(max_luminance), int(filter),
                                       float(tiling[0]), float(tiling[1]), C.byref(out)))
        return cls.from_id(ctx, out.value, filter, tiling)

    @classmethod
    def from_id(cls, ctx: Context, tid: int, filter: TextureFilter = TextureFilter.Bilinear,
                tiling: Sequence[float] = (1.0, 1.0)) -> "Texture":
        """A texture the library created (e.g. from an MTL map), with its texels read back."""
        w, h = C.c_uint32(), C.c_uint32()
        check(ctx._lib.sr_texture_export(ctx.handle, int(tid), C.byref(w), C.byref(h), None))
        t = np.zeros((h.value, w.value, 3), np.float32)
        check(ctx._lib.sr_texture_export(ctx.handle, int(tid), C.byref(w), C.byref(h), ptr(t)))
        obj = cls.__new__(cls)
        obj.ctx, obj.texels, obj.height, obj.width = ctx, t, h.value, w.value
        obj.filter, obj.tiling, obj.id = TextureFilter(filter), (float(tiling[0]), float(tiling[1])), int(tid)
        return obj

    # Color.FromPixel(Pixel) math.cs:184-191: sRGB decode pow(x/255, 2.2333).
    @staticmethod
    def srgb_to_linear(pixels: np.ndarray) -> np.ndarray:
        """MathF.Pow(c / 255f, 2.233333333f) per channel: the C runtime's powf, as the library's
        file loader (sr_texture_load) uses it."""
        return _srgb_table()[np.asarray(pixels)[..., :3]]

    @classmethod
    def from_srgb(cls, ctx: Context, pixels: np.ndarray, **kw) -> "Texture":
        """Texture.FromSrgb texture.cs:138-144 (RGB8/RGBA8 pixels, alpha dropped)."""
        return cls(ctx, cls.srgb_to_linear(pixels), **kw)

    @classmethod
    def from_linear(cls, ctx: Context, pixels: np.ndarray, **kw) -> "Texture":
        """Texture.FromLinear texture.cs:146-152."""
        p = np.asarray(pixels)[..., :3].astype(np.float32) / np.float32(255.0)
        return cls(ctx, p, **kw)

    @staticmethod
    def rgbe_to_linear(rgbe: np.ndarray, max_luminance: float = float(np.finfo(np.float32).max)) -> np.ndarray:
        """Color.FromPixel(PixelHdr) math.cs:196-202 + ClampLuminance math.cs:118-122."""
        rgbe = np.asarray(rgbe, dtype=np.uint8)
        e = rgbe[..., 3].astype(np.int32)
        scale = (np.ldexp(np.float32(1.0), e - 128).astype(np.float32) / np.float32(256.0)).astype(np.float32)
        c = rgbe[..., :3].astype(np.float32) * scale[..., None]
        c[e == 0] = 0.0
        lum = (np.float32(0.2126) * c[..., 0] + np.float32(0.7152) * c[..., 1]) + np.float32(0.0722) * c[..., 2]
        m = np.float32(max_luminance)
        over = lum > m
        if np.any(over):
            c[over] = c[over] * (m / lum[over])[:, None]
        return c.astype(np.float32)

    @classmethod
    def from_hdr(cls, ctx: Context, rgbe: np.ndarray, max_luminance: float = float(np.finfo(np.float32).max),
                 **kw) -> "Texture":
        """Texture.FromHdr texture.cs:154-163 from RGBE pixels (H, W, 4) uint8."""
        return cls(ctx, cls.rgbe_to_linear(rgbe, max_luminance), **kw)


class Mesh:
    """Triangle mesh with its own binned-SAH BVH built on the host (mesh.cs:18-45)."""

    def __init__(self, ctx: Context, triangles: np.ndarray):
        tris = np.ascontiguousarray(triangles, dtype=np.float32).reshape(-1, _abi.TRIANGLE_FLOATS)
        self.ctx, self.triangles = ctx, tris
        out = C.c_int32()
        check(ctx._lib.sr_mesh_create(ctx.handle, ptr(tris), tris.shape[0], C.byref(out)))
        self.id = out.value

    @staticmethod
    def triangles_from_corners(ctx: Context, positions: np.ndarray, uvs: Optional[np.ndarray] = None,
                               normals: Optional[np.ndarray] = None, smooth_normals: bool = True) -> np.ndarray:
        """Triangle ctors + Mesh.ComputeSmoothNormals, the ObjLoader path (obj.cs:170-190, 403-443)."""
        p = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 9)
        u = None if uvs is None else np.ascontiguousarray(uvs, dtype=np.float32).reshape(-1, 6)
        n = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 9)
        out = np.zeros((p.shape[0], _abi.TRIANGLE_FLOATS), np.float32)
        check(ctx._lib.sr_triangles_from_corners(ptr(p), ptr(u), ptr(n), p.shape[0], int(smooth_normals), ptr(out)))
        return out

    @classmethod
    def from_corners(cls, ctx: Context, positions, uvs=None, normals=None, smooth_normals: bool = True) -> "Mesh":
        return cls(ctx, cls.triangles_from_corners(ctx, positions, uvs, normals, smooth_normals))

    def bvh(self):
        """(node bounds (M,6), node links (M,2) = child/shapeCount, item permutation (N,))."""
        lib, h = self.ctx._lib, self.ctx.handle
        nn, ni = C.c_uint32(), C.c_uint32()
        check(lib.sr_mesh_bvh_size(h, self.id, C.byref(nn), C.byref(ni)))
        b = np.zeros((nn.value, 6), np.float32)
        l = np.zeros((nn.value, 2), np.int32)
        it = np.zeros(ni.value, np.int32)
        check(lib.sr_mesh_bvh_export(h, self.id, ptr(b), ptr(l), ptr(it)))
        return b, l, it


@dataclass
class Sphere:
    """Analytic sphere shape (math.cs:1179-1234)."""
    center: Sequence[float]
    radius: float


@dataclass
class AABox:
    """Analytic axis-aligned box shape (math.cs:936-1059)."""
    min: Sequence[float]
    max: Sequence[float]


Shape = Union[Mesh, Sphere, AABox]


@dataclass
class Material:
    """scene.cs:161-187.  Textures multiply the scalar values."""
    albedo: Sequence[float]
    roughness: float
    metallic: float = 0.0
    transparency: float = 0.0
    ior: float = 1.5
    radiance: Sequence[float] = (0.0, 0.0, 0.0)
    color_texture: Optional[Texture] = None
    roughness_texture: Optional[Texture] = None
    metallic_texture: Optional[Texture] = None
    normal_texture: Optional[Texture] = None

    def to_c(self) -> SrMaterial:
        tid = lambda t: -1 if t is None else t.id
        m = SrMaterial()
        m.albedo[:] = [float(x) for x in self.albedo]
        m.roughness, m.metallic, m.transparency, m.ior = (float(self.roughness), float(self.metallic),
                                                          float(self.transparency), float(self.ior))
        m.radiance[:] = [float(x) for x in self.radiance]
        m.color_texture, m.roughness_texture = tid(self.color_texture), tid(self.roughness_texture)
        m.metallic_texture, m.normal_texture = tid(self.metallic_texture), tid(self.normal_texture)
        return m


@dataclass
class Quat:
    """Rotation quaternion (x, y, z, w) in float32 (math.cs:551-667)."""
    x: float = 0.0
    y: float = 0.0
    z: float = 0.0
    w: float = 1.0

    @staticmethod
    def identity() -> "Quat":
        return Quat(0.0, 0.0, 0.0, 1.0)

    @staticmethod
    def angle_axis(angle: float, axis: Sequence[float]) -> "Quat":
        """Quat.AngleAxis math.cs:620-625 (float32 arithmetic)."""
        half = _f32(angle) * _f32(0.5)
        s = _f32(math.sin(half))
        a = [_f32(v) * s for v in axis]
        return Quat(float(a[0]), float(a[1]), float(a[2]), float(_f32(math.cos(half))))

    def __mul__(self, b: "Quat") -> "Quat":
        a = self
        ax, ay, az, aw = map(_f32, (a.x, a.y, a.z, a.w))
        bx, by, bz, bw = map(_f32, (b.x, b.y, b.z, b.w))
        return Quat(float(aw * bx + ax * bw + ay * bz - az * by), float(aw * by + ay * bw + az * bx - ax * bz),
                    float(aw * bz + az * bw + ax * by - ay * bx), float(aw * bw - ax * bx - ay * by - az * bz))

    def as_tuple(self):
        return (self.x, self.y, self.z, self.w)


@dataclass
class Transform:
    """Position, rotation, scale (math.cs:773-879)."""
    pos: Sequence[float] = (0.0, 0.0, 0.0)
    rot: Quat = field(default_factory=Quat.identity)
    scale: Sequence[float] = (1.0, 1.0, 1.0)

    @staticmethod
    def identity() -> "Transform":
        return Transform()

    def to_c(self) -> SrTransform:
        t = SrTransform()
        t.pos[:] = [float(v) for v in self.pos]
        t.rot[:] = [float(v) for v in self.rot.as_tuple()]
        t.scale[:] = [float(v) for v in self.scale]
        return t


@dataclass
class Object:
    """A shape placed in the scene with a material (scene.cs:204-225)."""
    name: str
    trans: Transform
    material: Material
    shape: Shape

    def shape_c(self) -> SrShape:
        s = SrShape()
        if isinstance(self.shape, Mesh):
            s.kind, s.mesh = _abi.SR_SHAPE_MESH, self.shape.id
        elif isinstance(self.shape, Sphere):
            s.kind, s.mesh = _abi.SR_SHAPE_SPHERE, -1
            s.params[:4] = [*map(float, self.shape.center), float(self.shape.radius)]
        elif isinstance(self.shape, AABox):
            s.kind, s.mesh = _abi.SR_SHAPE_AABOX, -1
            s.params[:] = [*map(float, self.shape.min), *map(float, self.shape.max)]
        else:
            raise TypeError(f"unsupported shape {type(self.shape).__name__}")
        return s


@dataclass
class SkyTexture:
    """Equirectangular HDR sky with CDF importance sampling (scene.cs:379-435)."""
    texture: Texture
    multiplier: float = 1.0
    rot_yaw: float = 0.0


@dataclass
class SkyProcedural:
    """Three-band gradient sky with a cone sun (scene.cs:281-377)."""
    radiance_top: Sequence[float]
    radiance_middle: Sequence[float]
    radiance_bottom: Sequence[float]
    sun_dir: Sequence[float]
    sun_radiance: Sequence[float]
    sun_angle: float

    def to_c(self) -> SrSkyProcedural:
        s = SrSkyProcedural()
        s.top[:], s.middle[:], s.bottom[:] = (list(map(float, self.radiance_top)),
                                              list(map(float, self.radiance_middle)),
                                              list(map(float, self.radiance_bottom)))
        s.sun_dir[:], s.sun_radiance[:] = list(map(float, self.sun_dir)), list(map(float, self.sun_radiance))
        s.sun_angle = float(self.sun_angle)
        return s


@dataclass
class Fog:
    """Exponential height fog (scene.cs:438-505) for ``height_falloff`` > 0; with ``height_falloff``
    0, a homogeneous medium below ``top_height`` (an extension; the top must be finite)."""
    density: float
    color: Sequence[float]
    anisotropy: float
    height_falloff: float
    top_height: float = math.inf

    def to_c(self) -> SrFog:
        f = SrFog()
        f.density, f.anisotropy, f.height_falloff = float(self.density), float(self.anisotropy), float(self.height_falloff)
        f.top_height = float(self.top_height)
        f.color[:] = [float(c) for c in self.color]
        return f


class Scene:
    """Objects + sky + optional fog; ``build`` makes the scene BVH and uploads (scene.cs:507-571)."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self._lib = ctx._lib
        h = C.c_void_p()
        check(self._lib.sr_scene_create(ctx.handle, C.byref(h)))
        self.handle = h
        self.objects: list[Object] = []
        self.sky = None
        self.fog: Optional[Fog] = None
        self.built = False

    def set_sky(self, sky) -> None:
        if isinstance(sky, SkyTexture):
            check(self._lib.sr_scene_set_sky_texture(self.handle, sky.texture.id, float(sky.multiplier),
                                                     float(sky.rot_yaw)))
        elif isinstance(sky, SkyProcedural):
            c = sky.to_c()
            check(self._lib.sr_scene_set_sky_procedural(self.handle, C.byref(c)))
        else:
            raise TypeError("sky must be SkyTexture or SkyProcedural")
        self.sky = sky

    def set_fog(self, fog: Fog) -> None:
        c = fog.to_c()
        check(self._lib.sr_scene_set_fog(self.handle, C.byref(c)))
        self.fog = fog

    def add_object(self, obj: Object) -> int:
        t, m, s = obj.trans.to_c(), obj.material.to_c(), obj.shape_c()
        idx = C.c_int32()
        check(self._lib.sr_scene_add_object(self.handle, C.byref(t), C.byref(m), C.byref(s), C.byref(idx)))
        self.objects.append(obj)
        return idx.value

    def build(self) -> None:
        check(self._lib.sr_scene_build(self.handle))
        self.built = True

    def set_tuning(self, trace_blocks_per_sm: int = 0, fog_shade_blocks_per_sm: int = 0,
                   surface_shade_blocks_per_sm: int = 0, tail_divisor: int = 0, max_bounce_iterations: int = 0,
                   max_traversal_steps: int = 0, trace_block_threads: int = 0, max_slots: int = 0) -> None:
        """Launch geometry of the wavefront kernels (0 = default); results do not depend on it.
        The two caps (0 = the built-in runaway guards) end a render that exceeds them with
        SR_ERR_DEVICE (loop cap) instead of running on.  max_slots: paths in flight (0 = one per
        pixel; fewer: slots take the next pixel as theirs finish)."""
        t = _abi.SrTuning(trace_blocks_per_sm, fog_shade_blocks_per_sm, surface_shade_blocks_per_sm, tail_divisor,
                          0.0, 0.0, max_bounce_iterations, max_traversal_steps, trace_block_threads, max_slots)
        check(self._lib.sr_scene_set_tuning(self.handle, C.byref(t)))

    def get_tuning(self) -> dict:
        """sr_scene_get_tuning: the scene's current launch geometry and loop caps."""
        t = _abi.SrTuning()
        check(self._lib.sr_scene_get_tuning(self.handle, C.byref(t)))
        return {f: getattr(t, f) for f, _ in _abi.SrTuning._fields_ if f not in ("ms", "default_ms")}

    def autotune(self, view: "View", params: SrRenderParams, trial_spp: int = 8) -> dict:
        """sr_scene_autotune: times candidate launch geometries on `params` at trial_spp samples per
        pixel and keeps the fastest; returns it with the trial times (ms) of it and of the defaults."""
        if not self.built:
            self.build()
        t = _abi.SrTuning()
        v = view.to_c()
        check(self._lib.sr_scene_autotune(self.handle, C.byref(v), C.byref(params), int(trial_spp), C.byref(t)))
        return {"trace_block_threads": t.trace_block_threads or 128, "trace_blocks_per_sm": t.trace_blocks_per_sm,
                "fog_shade_blocks_per_sm": t.fog_shade_blocks_per_sm,
                "surface_shade_blocks_per_sm": t.surface_shade_blocks_per_sm, "tail_divisor": t.tail_divisor,
                "max_slots": t.max_slots, "ms": t.ms, "default_ms": t.default_ms, "gain": t.default_ms / t.ms if t.ms > 0 else None,
                # not a tuned dimension: the traversal walks the reference's binary tree (bvh.cs), whose
                # child order the bit-exact hits rest on; two-level (4-wide) node blocks that keep that
                # order measured 22 % slower on the 1080p fog workload
                "bvh_node_width": 2, "bvh_node_width_4_measured": "-22 %"}

    def update_texture(self, texture, texels: np.ndarray) -> None:
        """sr_scene_update_texture: new rgb texels (the texture's height x width x 3) for the built
        scene's device copy of `texture` (a Texture or its id)."""
        tid = texture.id if isinstance(texture, Texture) else int(texture)
        t = np.ascontiguousarray(texels, dtype=np.float32)
        check(self._lib.sr_scene_update_texture(self.handle, tid, ptr(t)))

    def progress(self) -> tuple:
        """sr_render_progress: (finished pixels, pixels) of the last render launch, without waiting
        (Renderer.Tick's (Step, Total), renderer.cs:98-105, at pixel granularity)."""
        d, t = C.c_uint32(), C.c_uint32()
        check(self._lib.sr_render_progress(self.handle, C.byref(d), C.byref(t)))
        return d.value, t.value

    def set_seed(self, seed: int) -> None:
        """sr_scene_set_seed: random-number stream of renders and adjoints (0 = the reference's).
        The stream is a 32-bit value: seeds outside [0, 2^32) are rejected."""
        seed = int(seed)
        if not 0 <= seed <= 0xFFFFFFFF:
            raise ValueError(f"seed must be in [0, 2^32), got {seed}")
        check(self._lib.sr_scene_set_seed(self.handle, seed))

    def get_seed(self) -> int:
        """sr_scene_get_seed: the stream the scene's renders use now (also after a direct
        sr_scene_set_seed call through the C ABI)."""
        v = C.c_uint32()
        check(self._lib.sr_scene_get_seed(self.handle, C.byref(v)))
        return v.value

    @property
    def seed(self) -> int:
        return self.get_seed()

    def set_adjoint_replay(self, form: int) -> None:
        """sr_scene_set_adjoint_replay: SR_ADJOINT_REPLAY_WAVEFRONT (default) or SR_ADJOINT_REPLAY_PIXEL."""
        check(self._lib.sr_scene_set_adjoint_replay(self.handle, int(form)))

    def render_checkpointed(self, view: "View", params: SrRenderParams, device_out: SrAovs,
                            stream: Optional[int] = None) -> int:
        """sr_render_checkpointed: sr_render_device keeping every sample's path vertices for
        adjoint_checkpointed; returns the bytes they take."""
        v = view.to_c()
        n = C.c_uint64()
        check(self._lib.sr_render_checkpointed(self.handle, C.byref(v), C.byref(params), C.byref(device_out),
                                               C.c_void_p(stream) if stream else None, C.byref(n)))
        return n.value

    def adjoint_checkpointed(self, d_image: int, albedo_texture=None, albedo_grad: Optional[int] = None,
                             roughness_texture=None, roughness_grad: Optional[int] = None,
                             fog_density_grad: Optional[int] = None, stream: Optional[int] = None) -> None:
        """sr_adjoint_checkpointed: the gradients of the last checkpointed render's image for
        dL/dI = d_image (device pointers; a None gradient skips its part)."""
        tid = lambda t: -1 if t is None else (t.id if isinstance(t, Texture) else int(t))
        p = lambda x: C.c_void_p(x) if x else None
        check(self._lib.sr_adjoint_checkpointed(self.handle, C.c_void_p(d_image), tid(albedo_texture), p(albedo_grad),
                                                tid(roughness_texture), p(roughness_grad), p(fog_density_grad),
                                                p(stream)))

    def release_checkpoint(self) -> None:
        check(self._lib.sr_scene_release_checkpoint(self.handle))

    def update_fog_density(self, density: float) -> None:
        """sr_scene_update_fog_density: the built scene's fog density (its fog must exist)."""
        check(self._lib.sr_scene_update_fog_density(self.handle, float(density)))

    def update_texture_device(self, texture, d_texels: int, stream: Optional[int] = None) -> None:
        """sr_scene_update_texture_device: the same from a device pointer (float32 h x w x 3),
        asynchronous on `stream`."""
        tid = texture.id if isinstance(texture, Texture) else int(texture)
        check(self._lib.sr_scene_update_texture_device(self.handle, tid, C.c_void_p(d_texels),
                                                       C.c_void_p(stream) if stream else None))

    def load_obj(self, path, transform: Optional["Transform"] = None, material: Optional["Material"] = None,
                 smooth_normals: bool = True) -> int:
        """ObjLoader.Load(path, scene, config) obj.cs:139-259: adds one object per OBJ group; returns
        the number added."""
        t = C.byref(transform.to_c()) if transform is not None else None
        m = C.byref(material.to_c()) if material is not None else None
        n = C.c_uint32()
        check(self._lib.sr_obj_load(self.handle, str(path).encode(), t, m, int(smooth_normals), C.byref(n)))
        return n.value

    def object_count(self) -> int:
        n = C.c_uint32()
        check(self._lib.sr_scene_object_count(self.handle, C.byref(n)))
        return n.value

    def object_info(self, index: int) -> dict:
        """Name, transform, material and shape of object `index` as the library holds them."""
        t, m, sh = _abi.SrTransform(), _abi.SrMaterial(), _abi.SrShape()
        name = C.create_string_buffer(512)
        check(self._lib.sr_scene_object_info(self.handle, int(index), C.byref(t), C.byref(m), C.byref(sh), name, 512))
        return {"name": name.value.decode(), "transform": t, "material": m, "shape": sh}

    def bvh(self):
        nn, ni = C.c_uint32(), C.c_uint32()
        check(self._lib.sr_scene_bvh_size(self.handle, C.byref(nn), C.byref(ni)))
        b = np.zeros((nn.value, 6), np.float32)
        l = np.zeros((nn.value, 2), np.int32)
        it = np.zeros(ni.value, np.int32)
        check(self._lib.sr_scene_bvh_export(self.handle, ptr(b), ptr(l), ptr(it)))
        return b, l, it

    def trace(self, rays: np.ndarray) -> dict:
        """Closest hit of world rays (N, 6) = origin, unit dir; on the GPU."""
        r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        n = r.shape[0]
        obj = np.empty(n, np.int32)
        tri = np.empty(n, np.int32)
        dist = np.empty(n, np.float32)
        uv = np.empty((n, 2), np.float32)
        check(self._lib.sr_scene_trace(self.handle, ptr(r), n, ptr(obj), ptr(tri), ptr(dist), ptr(uv)))
        return {"object": obj, "triangle": tri, "dist": dist, "uv": uv}

    def set_render_mode(self, mode: int) -> None:
        """0 auto, 1 megakernel, 2 wavefront (host loop), 3 wavefront (device graph loop)."""
        check(self._lib.sr_scene_set_render_mode(self.handle, int(mode)))

    def render_info(self) -> dict:
        """Kernel launches and wavefront bounce iterations of the last render."""
        k, b = C.c_uint32(), C.c_uint32()
        check(self._lib.sr_scene_render_info(self.handle, C.byref(k), C.byref(b)))
        return {"kernel_launches": k.value, "bounce_iterations": b.value}

    def set_counting(self, enabled: bool) -> None:
        check(self._lib.sr_scene_set_counting(self.handle, int(enabled)))

    def set_kernel_timing(self, enabled: bool) -> None:
        """Time every traversal kernel of host-loop renders (render mode 2) with CUDA events."""
        check(self._lib.sr_scene_set_kernel_timing(self.handle, int(enabled)))

    def trace_time(self) -> dict:
        """Summed traversal-kernel time (ms) and launches of the last timed host-loop render."""
        ms, n = C.c_float(), C.c_uint32()
        check(self._lib.sr_scene_trace_time(self.handle, C.byref(ms), C.byref(n)))
        return {"total_ms": ms.value, "launches": n.value}

    def counters(self) -> dict:
        out = np.zeros(_abi.SR_COUNTER_COUNT, np.uint64)
        check(self._lib.sr_scene_counters(self.handle, ptr(out)))
        return dict(zip(_abi.COUNTER_NAMES, (int(v) for v in out)))

    def close(self) -> None:
        if self.handle:
            self._lib.sr_scene_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class View:
    """Pinhole camera (math.cs:1582-1636): fov in radians, horizontal when aspect >= 1."""
    trans: Transform = field(default_factory=Transform.identity)
    fov: float = math.radians(60.0)
    near: float = 0.1

    def to_c(self) -> SrView:
        v = SrView()
        v.transform = self.trans.to_c()
        v.fov, v.near_plane = float(self.fov), float(self.near)
        return v


def render_params(width, height, block_size, min_samples, max_samples, variance_threshold, bounces,
                  indirect_clamp) -> SrRenderParams:
    p = SrRenderParams()
    p.width, p.height, p.block_size = int(width), int(height), int(block_size)
    p.min_samples, p.max_samples = int(min_samples), int(max_samples)
    p.variance_threshold, p.bounces, p.indirect_clamp = float(variance_threshold), int(bounces), float(indirect_clamp)
    return p


class Aovs:
    """The seven AOV planes of a render as numpy arrays (renderer.cs:14-20)."""

    def __init__(self, width: int, height: int):
        n = width * height
        self.width, self.height = width, height
        self.radiance = np.zeros((n, 3), np.float32)
        self.radiance_fog = np.zeros((n, 3), np.float32)
        self.normals = np.zeros((n, 3), np.float32)
        self.uv = np.zeros((n, 2), np.float32)
        self.depth = np.zeros(n, np.float32)
        self.samples = np.zeros(n, np.uint32)
        self.variance = np.zeros(n, np.float32)

    def to_c(self) -> SrAovs:
        a = SrAovs()
        a.radiance, a.radiance_fog, a.normals = ptr(self.radiance), ptr(self.radiance_fog), ptr(self.normals)
        a.uv, a.depth, a.samples, a.variance = ptr(self.uv), ptr(self.depth), ptr(self.samples), ptr(self.variance)
        return a


class Renderer:
    """Renders the whole image on construction (the GPU finishes all tiles in one call).

    ``tick()`` returns ``(Step, Total)`` like renderer.cs:98-105 and is always complete; the AOV arrays
    ``radiance``, ``radiance_fog``, ``normals``, ``uv``, ``depth``, ``samples``, ``variance`` match
    renderer.cs:14-20 (flattened row-major, one entry per pixel).
    """

    def __init__(self, scene: Scene, view: View, width: int, height: int, block_size: int, min_samples: int,
                 max_samples: int, variance_threshold: float, bounces: int, indirect_clamp: float):
        if not scene.built:
            scene.build()  # the reference's ctor calls scene.Build (renderer.cs:77)
        self.scene, self.view = scene, view
        self.width, self.height = int(width), int(height)
        self.params = render_params(width, height, block_size, min_samples, max_samples, variance_threshold,
                                    bounces, indirect_clamp)
        self.aovs = Aovs(self.width, self.height)
        v, a = view.to_c(), self.aovs.to_c()
        check(scene._lib.sr_render(scene.handle, C.byref(v), C.byref(self.params), C.byref(a)))
        bx = (self.width + block_size - 1) // block_size
        by = (self.height + block_size - 1) // block_size
        self._total = bx * by

    def tick(self):
        return (self._total, self._total)

    def __getattr__(self, name):
        if name in ("radiance", "radiance_fog", "normals", "uv", "depth", "samples", "variance"):
            return getattr(self.aovs, name)
        raise AttributeError(name)


class Tonemapper(IntEnum):
    Reinhard = _abi.SR_TONEMAP_REINHARD
    LinearSmooth = _abi.SR_TONEMAP_LINEAR_SMOOTH


@dataclass
class Compositor:
    """Denoise + tonemap (compose.cs:22-48); defaults are program.cs:29-40."""
    tonemapper: Tonemapper = Tonemapper.LinearSmooth
    exposure: float = 1.0
    denoise_radius: float = 0.0075
    denoise_strength: float = 0.1
    denoise_strength_max: float = 1.75
    denoise_luminance_boost: float = 0.25
    denoise_luminance_limit: float = 2.0
    denoise_normal_limit: float = 0.125
    denoise_depth_limit: float = 0.2
    denoise_fog_radius: float = 0.002
    denoise_fog_strength: float = 0.05

    def to_c(self) -> SrComposeParams:
        p = SrComposeParams()
        p.tonemapper, p.exposure = int(self.tonemapper), float(self.exposure)
        p.denoise_radius, p.denoise_strength = float(self.denoise_radius), float(self.denoise_strength)
        p.denoise_strength_max = float(self.denoise_strength_max)
        p.denoise_luminance_boost = float(self.denoise_luminance_boost)
        p.denoise_luminance_limit = float(self.denoise_luminance_limit)
        p.denoise_normal_limit, p.denoise_depth_limit = float(self.denoise_normal_limit), float(self.denoise_depth_limit)
        p.denoise_fog_radius, p.denoise_fog_strength = float(self.denoise_fog_radius), float(self.denoise_fog_strength)
        return p

    def compose(self, rend: Renderer, overlay: Optional["Overlay"] = None) -> np.ndarray:
        """Compositor.Compose compose.cs:74-99 -> (H, W, 3) uint8, then the overlay if given."""
        out = np.zeros((rend.height, rend.width, 3), np.uint8)
        a, p = rend.aovs.to_c(), self.to_c()
        ctx = rend.scene.ctx
        check(ctx._lib.sr_compose(ctx.handle, C.byref(a), rend.width, rend.height, C.byref(p), ptr(out)))
        if overlay is not None:
            overlay.draw(ctx, out, rend.view, rend.depth.reshape(rend.height, rend.width))
        return out

    def preview(self, rend: Renderer, overlay: Optional["Overlay"] = None) -> np.ndarray:
        """Compositor.Preview compose.cs:57-65 (tonemap without denoise), then the overlay if given."""
        out = np.zeros((rend.height, rend.width, 3), np.uint8)
        a, p = rend.aovs.to_c(), self.to_c()
        ctx = rend.scene.ctx
        check(ctx._lib.sr_preview(ctx.handle, C.byref(a), rend.width, rend.height, C.byref(p), ptr(out)))
        if overlay is not None:
            overlay.draw(ctx, out, rend.view, rend.depth.reshape(rend.height, rend.width))
        return out


class AovKind(IntEnum):
    Normal = _abi.SR_AOV_NORMAL
    Depth = _abi.SR_AOV_DEPTH
    Variance = _abi.SR_AOV_VARIANCE
    Samples = _abi.SR_AOV_SAMPLES
    Uv = _abi.SR_AOV_UV


def aov_image(rend: Renderer, kind: AovKind) -> np.ndarray:
    """The normal / depth / variance / samples / uv dumps of program.cs:211-263 as (H, W, 3) uint8,
    with the renderer's own variance threshold and sample range."""
    out = np.zeros((rend.height, rend.width, 3), np.uint8)
    p = _abi.SrAovImageParams(rend.params.variance_threshold, rend.params.min_samples, rend.params.max_samples)
    ctx = rend.scene.ctx
    a = rend.aovs.to_c()
    check(ctx._lib.sr_aov_image(ctx.handle, C.byref(a), rend.width, rend.height, int(kind), C.byref(p), ptr(out)))
    return out


def save_image(path, rgb8: np.ndarray) -> None:
    """Image.Save image.cs:198-212: .tga, .ppm or .bmp by extension."""
    img = np.ascontiguousarray(rgb8, np.uint8)
    if img.ndim != 3 or img.shape[2] != 3:
        raise ValueError("image must be (height, width, 3) uint8")
    check(_abi.load().sr_image_save(str(path).encode(), img.shape[1], img.shape[0], ptr(img)))


@dataclass
class Font:
    """An 8x8 bitmap font: glyphs[c - first_char] is 8 row bytes, most significant bit leftmost
    (the layout of the reference's Font table, font.cs).  No font ships with the library."""
    glyphs: np.ndarray
    first_char: int = 32

    def to_c(self) -> "_abi.SrFont":
        g = np.ascontiguousarray(self.glyphs, np.uint8).reshape(-1, 8)
        self._keep = g
        return _abi.SrFont(g.ctypes.data, int(self.first_char), int(self.first_char) + g.shape[0] - 1)


class Overlay:
    """Debug overlay (overlay.cs): lines and boxes in world space, text in world or screen space,
    drawn by the library into an RGB8 image (sr_overlay_draw)."""

    TopLeft, Center = _abi.SR_ALIGN_TOP_LEFT, _abi.SR_ALIGN_CENTER

    def __init__(self, font: Optional[Font] = None):
        self.font = font
        self.lines: list = []
        self.texts: list = []

    def add_line(self, a, b, color, depth_test: bool = True, depth_bias: float = 0.005) -> None:
        self.lines.append((tuple(map(float, a)), tuple(map(float, b)), tuple(map(float, color)), bool(depth_test),
                           float(depth_bias)))

    def add_line_box(self, box: AABox, color, depth_test: bool = True, depth_bias: float = 0.005,
                     rot: Optional[Quat] = None) -> None:
        """AddLineBox overlay.cs:23-44 with Box.Corners math.cs:1086-1096 (float32)."""
        lo, hi = np.asarray(box.min, np.float32), np.asarray(box.max, np.float32)
        center, half = (lo + hi) * np.float32(0.5), (hi - lo) * np.float32(0.5)
        q = rot if rot is not None else Quat.identity()
        corners = []
        for i in range(8):
            v = np.array([half[0] if i & 1 else -half[0], half[1] if i & 2 else -half[1],
                          half[2] if i & 4 else -half[2]], np.float32)
            corners.append(center + _rotate_f32(q, v))
        for i, j in ((0, 1), (2, 3), (4, 5), (6, 7), (0, 2), (1, 3), (4, 6), (5, 7), (0, 4), (1, 5), (2, 6), (3, 7)):
            self.add_line(corners[i], corners[j], color, depth_test, depth_bias)

    def add_text(self, text: str, pos, color, align: Optional[int] = None) -> None:
        """A 3-component `pos` is a world position (default centred), a 2-component one a screen
        pixel (default top-left), as the two AddText overloads of overlay.cs:46-52."""
        world = len(pos) == 3
        if align is None:
            align = self.Center if world else self.TopLeft
        self.texts.append((text.encode("latin-1", "replace"), world, tuple(pos), tuple(map(float, color)), int(align)))

    def _c_arrays(self):
        lines = (_abi.SrOverlayLine * max(1, len(self.lines)))()
        for k, (a, b, c, dt, bias) in enumerate(self.lines):
            lines[k].a[:], lines[k].b[:], lines[k].color[:] = a, b, c
            lines[k].depth_test, lines[k].depth_bias = int(dt), bias
        texts = (_abi.SrOverlayText * max(1, len(self.texts)))()
        for k, (t, world, pos, c, align) in enumerate(self.texts):
            texts[k].text, texts[k].in_world, texts[k].align = t, int(world), align
            if world:
                texts[k].world_pos[:] = [float(x) for x in pos]
            else:
                texts[k].screen_pos[:] = [int(x) for x in pos]
            texts[k].color[:] = c
        return lines, texts

    def draw(self, ctx: Context, image: np.ndarray, view: View, depth: Optional[np.ndarray] = None) -> np.ndarray:
        """Overlay.Draw overlay.cs:54-96 into `image` ((H, W, 3) uint8, modified in place)."""
        if image.dtype != np.uint8 or image.ndim != 3 or image.shape[2] != 3 or not image.flags.c_contiguous:
            raise ValueError("image must be a C-contiguous (height, width, 3) uint8 array")
        h, w = image.shape[:2]
        d = None if depth is None else np.ascontiguousarray(depth, np.float32).reshape(h * w)
        lines, texts = self._c_arrays()
        font = self.font.to_c() if self.font is not None else _abi.SrFont(None, 0, -1)
        v = view.to_c()
        check(ctx._lib.sr_overlay_draw(ctx.handle, ptr(image), w, h, C.byref(v), ptr(d), lines, len(self.lines),
                                       texts, len(self.texts), C.byref(font) if self.font is not None else None))
        return image


def _rotate_f32(q: Quat, v: np.ndarray) -> np.ndarray:
    """Quat * Vec3 math.cs:609-617 in float32."""
    axis = np.array([q.x, q.y, q.z], np.float32)
    w = np.float32(q.w)
    sqr = np.float32(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2])
    d = np.float32(axis[0] * v[0] + axis[1] * v[1] + axis[2] * v[2])
    a = axis * np.float32(d * np.float32(2))
    b = v * np.float32(w * w - sqr)
    c = np.array([axis[1] * v[2] - axis[2] * v[1], axis[2] * v[0] - axis[0] * v[2], axis[0] * v[1] - axis[1] * v[0]],
                 np.float32) * np.float32(w * np.float32(2))
    return (a + b + c).astype(np.float32)


def render_compose(scene: Scene, view: View, width: int, height: int, block_size: int, min_samples: int,
                   max_samples: int, variance_threshold: float, bounces: int, indirect_clamp: float,
                   compositor: Compositor, aovs: Optional[Aovs] = None, image: Optional[np.ndarray] = None):
    """Render + Compose in one native call (sr_render_compose); returns (image, aovs)."""
    if not scene.built:
        scene.build()
    p = render_params(width, height, block_size, min_samples, max_samples, variance_threshold, bounces,
                      indirect_clamp)
    v, cp = view.to_c(), compositor.to_c()
    if image is None:
        image = np.zeros((height, width, 3), np.uint8)
    a = C.byref(aovs.to_c()) if aovs is not None else None
    check(scene._lib.sr_render_compose(scene.handle, C.byref(v), C.byref(p), C.byref(cp), a, ptr(image)))
    return image, aovs


def render_batch(scenes: Sequence["Scene"], views: Sequence["View"], params: Sequence[SrRenderParams],
                 device_aovs: Sequence[SrAovs], stream: Optional[int] = None) -> None:
    """sr_render_batch: several built scenes, each with its view, render parameters
    (`render_params(...)`) and device AOV planes (an `SrAovs` of device pointers), in one graph
    launch on `stream` (a CUDA stream handle; None = the context's).  Asynchronous."""
    n = len(scenes)
    if not (len(views) == len(params) == len(device_aovs) == n):
        raise ValueError("scenes, views, params and device_aovs must have the same length")
    if n == 0:
        return
    for s in scenes:
        if not s.built:
            s.build()
    arr_s = (C.c_void_p * n)(*[s.handle.value for s in scenes])
    arr_v = (_abi.SrView * n)(*[v.to_c() for v in views])
    arr_p = (SrRenderParams * n)(*params)
    arr_a = (SrAovs * n)(*device_aovs)
    lib = scenes[0]._lib
    check(lib.sr_render_batch(arr_s, arr_v, arr_p, arr_a, n, C.c_void_p(stream) if stream else None))


def adjoint_texture(scene: "Scene", view: "View", params: SrRenderParams, forward: SrAovs, d_image: int,
                    texture, grad: int, parameter: int = _abi.SR_ADJOINT_ALBEDO, replay: Optional[int] = None,
                    stream: Optional[int] = None) -> None:
    """sr_adjoint_texture: adds dL/d(texels of `texture`) into `grad`, given d_image = dL/dI for the
    image I = radiance + radiance_fog of `forward` (device AOV planes of sr_render_device with the
    same scene, view and params), for the texture as the albedo (SR_ADJOINT_ALBEDO) or the roughness
    (SR_ADJOINT_ROUGHNESS: channel 0 of grad) lookup, or for the fog density (SR_ADJOINT_FOG_DENSITY:
    `texture` ignored, grad one float).  d_image / grad / replay are device pointers (float32,
    H x W x 3 and the texture's h x w x 3); asynchronous on `stream`."""
    tid = -1 if texture is None else (texture.id if isinstance(texture, Texture) else int(texture))
    v = view.to_c()
    check(scene._lib.sr_adjoint_texture(scene.handle, C.byref(v), C.byref(params), C.byref(forward),
                                        C.c_void_p(d_image), tid, int(parameter), C.c_void_p(grad),
                                        C.c_void_p(replay) if replay else None,
                                        C.c_void_p(stream) if stream else None))


def adjoint_albedo(scene: "Scene", view: "View", params: SrRenderParams, forward: SrAovs, d_image: int,
                   texture, grad: int, replay: Optional[int] = None, stream: Optional[int] = None) -> None:
    """sr_adjoint_albedo: adjoint_texture for the albedo lookup."""
    tid = texture.id if isinstance(texture, Texture) else int(texture)
    v = view.to_c()
    check(scene._lib.sr_adjoint_albedo(scene.handle, C.byref(v), C.byref(params), C.byref(forward),
                                       C.c_void_p(d_image), tid, C.c_void_p(grad),
                                       C.c_void_p(replay) if replay else None, C.c_void_p(stream) if stream else None))


def load_image(path) -> np.ndarray:
    """Image.Load (.tga: RGB8) or ImageHdr.Load (.hdr: RGBE8) as parsed by the library; (H, W, C)."""
    lib = _abi.load()
    w, h, ch = C.c_uint32(), C.c_uint32(), C.c_uint32()
    check(lib.sr_image_load(str(path).encode(), C.byref(w), C.byref(h), C.byref(ch), None, 0))
    out = np.zeros((h.value, w.value, ch.value), np.uint8)
    check(lib.sr_image_load(str(path).encode(), C.byref(w), C.byref(h), C.byref(ch), ptr(out), out.nbytes))
    return out


def mesh_triangles(ctx: Context, mesh_id: int) -> np.ndarray:
    """The SrTriangles (N, 36) of a library mesh."""
    n = C.c_uint32()
    check(ctx._lib.sr_mesh_export(ctx.handle, int(mesh_id), C.byref(n), None))
    out = np.zeros((n.value, _abi.TRIANGLE_FLOATS), np.float32)
    check(ctx._lib.sr_mesh_export(ctx.handle, int(mesh_id), C.byref(n), ptr(out)))
    return out
