"""ctypes wrapper of the CPU oracle (``oracle/sr_oracle.cpp``).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` to check and time the GPU library.  The product never imports this module.

The oracle is a scalar C++ restatement of the C# reference's render path (see the header of
sr_oracle.cpp for the file:line map).  Parity against the C# binary itself is unpinned: no .NET
runtime exists on either machine, so the restatement is pinned by published known answers
(splitmix64) and analytic checks instead.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "sr_oracle.cpp"
LIB = HERE / "liboracle.so"

# Same POD layouts as the C ABI (imported only for the struct definitions).
from sharpray_gb300._abi import (SR_COUNTER_COUNT, COUNTER_NAMES, TRIANGLE_FLOATS, SrAovImageParams, SrAovs,
                                 SrComposeParams, SrFog, SrFont, SrMaterial, SrRenderParams, SrShape, SrSkyProcedural,
                                 SrTransform, SrView)

CXXFLAGS = ["-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread"]


def build(force: bool = False) -> Path:
    """Compile the oracle with the reference's float rules (no FMA contraction)."""
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    subprocess.run(["g++", *CXXFLAGS, str(SRC), "-o", str(tmp)], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P, I, U, F = C.c_void_p, C.c_int, C.c_uint32, C.c_float
        sig = {
            "oracle_last_error": (C.c_char_p, []),
            "oracle_rng_stream": (None, [U, U, U, P, P]),
            "oracle_splitmix64": (None, [C.c_uint64, U, P]),
            "oracle_triangles_from_corners": (I, [P, P, P, U, C.c_int32, P]),
            "oracle_scene_create": (P, []),
            "oracle_scene_destroy": (None, [P]),
            "oracle_texture_create": (I, [P, P, U, U, C.c_int32, F, F]),
            "oracle_mesh_create": (I, [P, P, U]),
            "oracle_mesh_bvh_size": (None, [P, C.c_int32, C.POINTER(U), C.POINTER(U)]),
            "oracle_mesh_bvh_export": (None, [P, C.c_int32, P, P, P]),
            "oracle_scene_set_sky_texture": (None, [P, C.c_int32, F, F]),
            "oracle_scene_set_sky_procedural": (None, [P, C.POINTER(SrSkyProcedural)]),
            "oracle_scene_set_fog": (None, [P, C.POINTER(SrFog)]),
            "oracle_scene_add_object": (I, [P, C.POINTER(SrTransform), C.POINTER(SrMaterial), C.POINTER(SrShape)]),
            "oracle_scene_build": (I, [P]),
            "oracle_scene_bvh_size": (None, [P, C.POINTER(U), C.POINTER(U)]),
            "oracle_scene_bvh_export": (None, [P, P, P, P]),
            "oracle_scene_trace": (None, [P, P, U, P, P, P, P, C.c_int32]),
            "oracle_render": (I, [P, C.POINTER(SrView), C.POINTER(SrRenderParams), C.c_int32, U, U,
                                  C.POINTER(SrAovs), P]),
            "oracle_compose": (None, [C.POINTER(SrAovs), U, U, C.POINTER(SrComposeParams), P, C.c_int32]),
            "oracle_preview": (None, [C.POINTER(SrAovs), U, U, C.POINTER(SrComposeParams), P]),
            "oracle_denoise": (None, [C.POINTER(SrAovs), U, U, C.POINTER(SrComposeParams), P, C.c_int32]),
            "oracle_aov_image": (None, [C.POINTER(SrAovs), U, U, C.c_int32, C.POINTER(SrAovImageParams), P]),
            "oracle_overlay_draw": (I, [P, U, U, C.POINTER(SrView), P, P, U, P, U, C.POINTER(SrFont)]),
            "oracle_adjoint": (I, [P, C.POINTER(SrView), C.POINTER(SrRenderParams), C.c_int32, P, P, C.c_int32, P,
                                   C.c_int32, P, P, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype, fn.argtypes = res, args
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def rng_stream(seed_a: int, seed_b: int, n: int):
    u = np.zeros(n, np.uint32)
    f = np.zeros(n, np.float32)
    lib().oracle_rng_stream(seed_a, seed_b, n, _p(u), _p(f))
    return u, f


def splitmix64(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint64)
    lib().oracle_splitmix64(seed, n, _p(out))
    return out


def triangles_from_corners(positions, uvs=None, normals=None, smooth_normals=True) -> np.ndarray:
    p = np.ascontiguousarray(positions, np.float32).reshape(-1, 9)
    u = None if uvs is None else np.ascontiguousarray(uvs, np.float32).reshape(-1, 6)
    n = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 9)
    out = np.zeros((p.shape[0], TRIANGLE_FLOATS), np.float32)
    rc = lib().oracle_triangles_from_corners(_p(p), _p(u), _p(n), p.shape[0], int(smooth_normals), _p(out))
    assert rc == 0
    return out


class OracleScene:
    """A scene inside the oracle, built from the same arrays/structs as the GPU library's."""

    def __init__(self):
        self.L = lib()
        self.h = self.L.oracle_scene_create()

    def __del__(self):
        try:
            self.L.oracle_scene_destroy(self.h)
        except Exception:
            pass

    def texture(self, texels: np.ndarray, filter: int = 0, tiling=(1.0, 1.0)) -> int:
        t = np.ascontiguousarray(texels, np.float32)
        return self.L.oracle_texture_create(self.h, _p(t), t.shape[1], t.shape[0], int(filter), float(tiling[0]),
                                            float(tiling[1]))

    def mesh(self, triangles: np.ndarray) -> int:
        t = np.ascontiguousarray(triangles, np.float32).reshape(-1, TRIANGLE_FLOATS)
        return self.L.oracle_mesh_create(self.h, _p(t), t.shape[0])

    def mesh_bvh(self, mesh: int):
        nn, ni = C.c_uint32(), C.c_uint32()
        self.L.oracle_mesh_bvh_size(self.h, mesh, C.byref(nn), C.byref(ni))
        b = np.zeros((nn.value, 6), np.float32)
        l = np.zeros((nn.value, 2), np.int32)
        it = np.zeros(ni.value, np.int32)
        self.L.oracle_mesh_bvh_export(self.h, mesh, _p(b), _p(l), _p(it))
        return b, l, it

    def set_sky_texture(self, tex: int, multiplier: float = 1.0, yaw: float = 0.0):
        self.L.oracle_scene_set_sky_texture(self.h, tex, multiplier, yaw)

    def set_sky_procedural(self, sky: SrSkyProcedural):
        self.L.oracle_scene_set_sky_procedural(self.h, C.byref(sky))

    def set_fog(self, fog: SrFog):
        self.L.oracle_scene_set_fog(self.h, C.byref(fog))

    def add_object(self, tr: SrTransform, mat: SrMaterial, shape: SrShape) -> int:
        return self.L.oracle_scene_add_object(self.h, C.byref(tr), C.byref(mat), C.byref(shape))

    def build(self):
        rc = self.L.oracle_scene_build(self.h)
        if rc:
            raise RuntimeError(self.L.oracle_last_error().decode())

    def bvh(self):
        nn, ni = C.c_uint32(), C.c_uint32()
        self.L.oracle_scene_bvh_size(self.h, C.byref(nn), C.byref(ni))
        b = np.zeros((nn.value, 6), np.float32)
        l = np.zeros((nn.value, 2), np.int32)
        it = np.zeros(ni.value, np.int32)
        self.L.oracle_scene_bvh_export(self.h, _p(b), _p(l), _p(it))
        return b, l, it

    def trace(self, rays: np.ndarray, threads: int = 0) -> dict:
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        n = r.shape[0]
        obj = np.empty(n, np.int32)
        tri = np.empty(n, np.int32)
        dist = np.empty(n, np.float32)
        uv = np.empty((n, 2), np.float32)
        self.L.oracle_scene_trace(self.h, _p(r), n, _p(obj), _p(tri), _p(dist), _p(uv), threads or os.cpu_count())
        return {"object": obj, "triangle": tri, "dist": dist, "uv": uv}

    def adjoint(self, view: SrView, params: SrRenderParams, d_image: np.ndarray, samples: np.ndarray,
                tex_albedo: int = -1, albedo_shape=None, tex_roughness: int = -1, roughness_shape=None,
                threads: int = 0):
        """FP64 path-replay adjoint (oracle_adjoint): for dL/dI = d_image (h x w x 3) and the forward
        render's sample counts, returns (dL/d albedo texels (th, tw, 3) or None, dL/d roughness texels
        (th, tw, 3; channel 0) or None, dL/d fog density, replayed image (h*w, 3)), all in double."""
        d = np.ascontiguousarray(d_image, np.float32).reshape(-1)
        smp = np.ascontiguousarray(samples, np.uint32).reshape(-1)
        ga = np.zeros((*albedo_shape, 3), np.float64) if tex_albedo >= 0 else None
        gr = np.zeros((*roughness_shape, 3), np.float64) if tex_roughness >= 0 else None
        gf = np.zeros(1, np.float64)
        rep = np.zeros((params.width * params.height, 3), np.float32)
        rc = self.L.oracle_adjoint(self.h, C.byref(view), C.byref(params), threads or os.cpu_count(), _p(d), _p(smp),
                                   tex_albedo, _p(ga), tex_roughness, _p(gr), _p(gf), _p(rep))
        if rc:
            raise RuntimeError(self.L.oracle_last_error().decode())
        return ga, gr, float(gf[0]), rep

    def render(self, view: SrView, params: SrRenderParams, threads: int = 0, rows=None, counters: bool = False):
        """AOV planes of rows [y0, y1) (others stay zero) and optionally the work counters."""
        from sharpray_gb300.api import Aovs
        a = Aovs(params.width, params.height)
        y0, y1 = rows if rows else (0, params.height)
        ctr = np.zeros(SR_COUNTER_COUNT, np.uint64) if counters else None
        c = a.to_c()
        rc = self.L.oracle_render(self.h, C.byref(view), C.byref(params), threads or os.cpu_count(), y0, y1,
                                  C.byref(c), _p(ctr))
        if rc:
            raise RuntimeError(self.L.oracle_last_error().decode())
        return a, (dict(zip(COUNTER_NAMES, (int(v) for v in ctr))) if counters else None)


def compose(aovs, params: SrComposeParams, threads: int = 0) -> np.ndarray:
    out = np.zeros((aovs.height, aovs.width, 3), np.uint8)
    c = aovs.to_c()
    lib().oracle_compose(C.byref(c), aovs.width, aovs.height, C.byref(params), _p(out), threads or os.cpu_count())
    return out


def preview(aovs, params: SrComposeParams) -> np.ndarray:
    out = np.zeros((aovs.height, aovs.width, 3), np.uint8)
    c = aovs.to_c()
    lib().oracle_preview(C.byref(c), aovs.width, aovs.height, C.byref(params), _p(out))
    return out


def aov_image(aovs, kind: int, params: SrAovImageParams) -> np.ndarray:
    """program.cs:211-263 AOV dump of one kind as (H, W, 3) RGB8."""
    out = np.zeros((aovs.height, aovs.width, 3), np.uint8)
    lib().oracle_aov_image(C.byref(aovs.to_c()), aovs.width, aovs.height, int(kind), C.byref(params), _p(out))
    return out


def overlay_draw(image: np.ndarray, view: SrView, depth, lines, texts, font: SrFont) -> np.ndarray:
    """Overlay.Draw on a copy of `image` ((H, W, 3) uint8); lines / texts are ctypes arrays."""
    out = np.ascontiguousarray(image, np.uint8).copy()
    h, w = out.shape[:2]
    d = None if depth is None else np.ascontiguousarray(depth, np.float32)
    rc = lib().oracle_overlay_draw(_p(out), w, h, C.byref(view), _p(d), lines, len(lines) if lines else 0, texts,
                                   len(texts) if texts else 0, C.byref(font))
    if rc:
        raise ValueError("overlay line end point outside the int range")
    return out


def denoise(aovs, params: SrComposeParams, threads: int = 0) -> np.ndarray:
    out = np.zeros((aovs.height * aovs.width, 3), np.float32)
    c = aovs.to_c()
    lib().oracle_denoise(C.byref(c), aovs.width, aovs.height, C.byref(params), _p(out), threads or os.cpu_count())
    return out


def instantiate(desc) -> OracleScene:
    """Build a ``sharpray_gb300.synth.SceneDesc`` inside the oracle, using the oracle's own ingest
    (triangle construction + smooth normals) and BVH builds."""
    from sharpray_gb300.api import Material
    s = OracleScene()
    tex = [s.texture(t.texels, t.filter, t.tiling) for t in desc.textures]
    meshes = [s.mesh(triangles_from_corners(m.positions, m.uvs, None, m.smooth_normals)) for m in desc.meshes]
    if desc.sky[0] == "texture":
        s.set_sky_texture(tex[desc.sky[1]], desc.sky[2], desc.sky[3])
    else:
        s.set_sky_procedural(desc.sky[1].to_c())
    if desc.fog is not None:
        s.set_fog(desc.fog.to_c())
    for o in desc.objects:
        s.add_object(o.transform.to_c(), desc.material_c(o, tex), desc.shape_c(o, meshes))
    s.build()
    return s


def render_desc(desc, threads: int = 0, rows=None, counters: bool = False):
    """Render a SceneDesc in the oracle: returns (Aovs, counters-or-None)."""
    from sharpray_gb300.api import render_params
    scene = instantiate(desc)
    return scene.render(desc.view.to_c(), render_params(*desc.render_args()), threads, rows, counters)
