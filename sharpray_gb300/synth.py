"""Seeded synthetic workloads for the render path.

The reference ships its demo assets only as git-LFS pointers, so every input here is generated:
displaced spheres (icosphere or CreateSphere-topology UV spheres with radial fBm value noise), RGBE
HDR environments (vertical gradient + Gaussian sun lobe, optionally a lognormal luminance field),
RGBA8 value-noise albedo textures.  Geometry uses only correctly rounded float64 operations
(+ - * / sqrt floor) before the final float32 rounding, so the same seed yields bit-identical
meshes on x86-64 and aarch64.

A :class:`SceneDesc` is a plain description (corner arrays, texel arrays, object list) that can be
instantiated on the GPU library (:meth:`SceneDesc.instantiate`) or handed to any other consumer of
the same arrays.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _abi
from .api import (AABox, Compositor, Context, Fog, Material, Mesh, Object, Quat, Scene, SkyProcedural,
                  SkyTexture, Sphere, Texture, TextureFilter, Transform, View)

# ---------------------------------------------------------------------------------------------
# noise


def _hash3(ix: np.ndarray, iy: np.ndarray, iz: np.ndarray, seed: int) -> np.ndarray:
    """Lattice hash -> float64 in [0, 1) (integer mixing only)."""
    with np.errstate(over="ignore"):
        h = (ix.astype(np.uint64) * np.uint64(0x9E3779B185EBCA87)) ^ (iy.astype(np.uint64) * np.uint64(0xC2B2AE3D27D4EB4F))
        h ^= iz.astype(np.uint64) * np.uint64(0x165667B19E3779F9)
        h ^= np.uint64((seed * 0x27D4EB2F165667C5) & 0xFFFFFFFFFFFFFFFF)
        h ^= h >> np.uint64(29)
        h *= np.uint64(0xBF58476D1CE4E5B9)
        h ^= h >> np.uint64(32)
        h *= np.uint64(0x94D049BB133111EB)
        h ^= h >> np.uint64(29)
    return (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def value_noise3(p: np.ndarray, seed: int) -> np.ndarray:
    """Trilinear value noise in [0, 1) with smoothstep weights; p is (..., 3) float64."""
    f = np.floor(p)
    t = p - f
    i = f.astype(np.int64)
    w = t * t * (3.0 - 2.0 * t)
    out = np.zeros(p.shape[:-1])
    for dx in (0, 1):
        wx = w[..., 0] if dx else 1.0 - w[..., 0]
        for dy in (0, 1):
            wy = w[..., 1] if dy else 1.0 - w[..., 1]
            for dz in (0, 1):
                wz = w[..., 2] if dz else 1.0 - w[..., 2]
                out = out + wx * wy * wz * _hash3(i[..., 0] + dx, i[..., 1] + dy, i[..., 2] + dz, seed)
    return out


def fbm3(p: np.ndarray, seed: int, octaves: int = 4) -> np.ndarray:
    """Fractal sum of value noise, normalised to about [-1, 1]."""
    total = np.zeros(p.shape[:-1])
    amp, freq, norm = 1.0, 1.0, 0.0
    for o in range(octaves):
        total = total + amp * (2.0 * value_noise3(p * freq, seed + 7919 * o) - 1.0)
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


# ---------------------------------------------------------------------------------------------
# meshes (triangle corners: positions (N, 3, 3) float32, uvs (N, 3, 2) float32)


def icosphere(subdivisions: int):
    """Unit icosphere: vertices (V, 3) float64, faces (F, 3) int (CCW seen from outside)."""
    phi = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, phi, 0), (1, phi, 0), (-1, -phi, 0), (1, -phi, 0), (0, -1, phi), (0, 1, phi), (0, -1, -phi),
             (0, 1, -phi), (phi, 0, -1), (phi, 0, 1), (-phi, 0, -1), (-phi, 0, 1)]
    v = [np.array(p, np.float64) / math.sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]) for p in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        cache: dict = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = (v[a] + v[b]) * 0.5
                v.append(m / math.sqrt(float(m @ m)))
                cache[key] = len(v) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    # The reference's triangles are CCW seen from outside with normal = cross(B-A, C-A); flip to match.
    f = np.array(faces, np.int64)[:, ::-1]
    return np.array(v), np.ascontiguousarray(f)


def displace(verts: np.ndarray, amplitude: float, seed: int, frequency: float = 2.0, octaves: int = 4) -> np.ndarray:
    """Radial fBm displacement r = 1 + amplitude * fbm(frequency * p)."""
    r = 1.0 + amplitude * fbm3(verts * frequency, seed, octaves)
    return verts * r[:, None]


def planar_uv(verts: np.ndarray) -> np.ndarray:
    return np.stack([0.5 + 0.5 * verts[:, 0], 0.5 - 0.5 * verts[:, 1]], axis=1)


def displaced_icosphere(subdivisions: int, amplitude: float, seed: int):
    v, f = icosphere(subdivisions)
    uv = planar_uv(v)
    p = displace(v, amplitude, seed)
    return p[f].astype(np.float32), uv[f].astype(np.float32)


def uv_sphere(rings: int, segments: int, amplitude: float = 0.0, seed: int = 0):
    """CreateSphere topology (mesh.cs:125-165): two triangles per ring/segment quad, uv = (seg, ring)."""
    r = np.arange(rings + 1, dtype=np.float64)
    s = np.arange(segments + 1, dtype=np.float64)
    theta = math.pi * r / rings
    phi = math.pi + 2.0 * math.pi * s / segments
    st, ct = np.sin(theta), np.cos(theta)
    grid = np.stack([st[:, None] * np.cos(phi)[None, :], np.broadcast_to(ct[:, None], (rings + 1, segments + 1)),
                     st[:, None] * np.sin(phi)[None, :]], axis=-1)
    if amplitude:
        flat = grid.reshape(-1, 3)
        grid = displace(flat, amplitude, seed).reshape(grid.shape)
    u = s / segments
    v = r / rings
    uvg = np.stack(np.broadcast_arrays(u[None, :], v[:, None]), axis=-1)
    ri, si = np.meshgrid(np.arange(rings), np.arange(segments), indexing="ij")
    ri, si = ri.ravel(), si.ravel()
    p00, p01, p10, p11 = grid[ri, si], grid[ri, si + 1], grid[ri + 1, si], grid[ri + 1, si + 1]
    t00, t01, t10, t11 = uvg[ri, si], uvg[ri, si + 1], uvg[ri + 1, si], uvg[ri + 1, si + 1]
    tri_a = np.stack([p00, p11, p10], axis=1)
    tri_b = np.stack([p00, p01, p11], axis=1)
    uv_a = np.stack([t00, t11, t10], axis=1)
    uv_b = np.stack([t00, t01, t11], axis=1)
    pos = np.stack([tri_a, tri_b], axis=1).reshape(-1, 3, 3)
    uvs = np.stack([uv_a, uv_b], axis=1).reshape(-1, 3, 2)
    return pos.astype(np.float32), uvs.astype(np.float32)


def ground_quad(half_size: float, y: float):
    s = half_size
    a, b, c, d = (-s, y, -s), (-s, y, s), (s, y, s), (s, y, -s)
    pos = np.array([[a, b, c], [a, c, d]], np.float32)
    uv = np.array([[(0, 1), (0, 0), (1, 0)], [(0, 1), (1, 0), (1, 1)]], np.float32)
    return pos, uv


# ---------------------------------------------------------------------------------------------
# images


def rgbe_encode(rgb: np.ndarray) -> np.ndarray:
    """Radiance RGBE (shared exponent, 8-bit mantissas) of float RGB (H, W, 3)."""
    rgb = np.asarray(rgb, np.float64)
    v = rgb.max(axis=-1)
    m, e = np.frexp(v)
    scale = np.where(v > 1e-32, m * 256.0 / np.where(v > 1e-32, v, 1.0), 0.0)
    out = np.zeros(rgb.shape[:-1] + (4,), np.uint8)
    out[..., :3] = np.clip(np.floor(rgb * scale[..., None]), 0, 255).astype(np.uint8)
    out[..., 3] = np.where(v > 1e-32, e + 128, 0).astype(np.uint8)
    return out


def _equirect_dirs(width: int, height: int) -> np.ndarray:
    """Unit directions of texel centres (Vec3.FromEquirectUv math.cs:493-500), float64."""
    u = (np.arange(width) + 0.5) / width
    v = (np.arange(height) + 0.5) / height
    phi = (u - 0.5) * 2.0 * np.pi
    st, ct = np.sin(np.pi * v), np.cos(np.pi * v)
    return np.stack([st[:, None] * np.cos(phi)[None, :], np.broadcast_to(ct[:, None], (height, width)),
                     st[:, None] * np.sin(phi)[None, :]], axis=-1)


def sky_env(width: int, height: int, seed: int, sun_peak: float = 50.0, sun_sigma_deg: float = 3.0,
            lognormal_sigma: float = 0.0) -> np.ndarray:
    """Equirect HDR sky as RGBE bytes: vertical gradient + Gaussian sun lobe (+ lognormal field)."""
    rng = np.random.default_rng(seed)
    d = _equirect_dirs(width, height)
    y = d[..., 1]
    zenith = np.array([0.25, 0.45, 0.95])
    horizon = np.array([0.85, 0.88, 0.92])
    ground = np.array([0.18, 0.15, 0.12])
    t_up = np.clip(y, 0.0, 1.0) ** 0.5
    sky = horizon * (1.0 - t_up[..., None]) + zenith * t_up[..., None]
    t_dn = np.clip(-y * 4.0, 0.0, 1.0)
    sky = sky * (1.0 - t_dn[..., None]) + ground * t_dn[..., None]
    if lognormal_sigma > 0.0:
        # smooth unit-variance field (fBm on the sphere, evaluated on a coarse grid and bilinearly
        # upsampled), exponentiated: a lognormal luminance field with the requested sigma
        cw, ch = max(4, width // 8), max(2, height // 8)
        f = fbm3(_equirect_dirs(cw, ch) * 3.0, seed + 101, 5)
        z = (f - f.mean()) / max(f.std(), 1e-12)
        gx = (np.arange(width) + 0.5) / width * cw - 0.5
        gy = (np.arange(height) + 0.5) / height * ch - 0.5
        x0 = np.clip(np.floor(gx).astype(int), 0, cw - 1)
        y0 = np.clip(np.floor(gy).astype(int), 0, ch - 1)
        x1, y1 = np.clip(x0 + 1, 0, cw - 1), np.clip(y0 + 1, 0, ch - 1)
        tx = np.clip(gx - x0, 0.0, 1.0)[None, :]
        ty = np.clip(gy - y0, 0.0, 1.0)[:, None]
        zz = ((z[y0][:, x0] * (1 - tx) + z[y0][:, x1] * tx) * (1 - ty) + (z[y1][:, x0] * (1 - tx) + z[y1][:, x1] * tx) * ty)
        sky = sky * np.exp(lognormal_sigma * zz - 0.5 * lognormal_sigma ** 2)[..., None]
    elev = math.radians(rng.uniform(25.0, 55.0))
    azim = rng.uniform(0.0, 2.0 * math.pi)
    sun = np.array([math.cos(elev) * math.cos(azim), math.sin(elev), math.cos(elev) * math.sin(azim)])
    ang = np.arccos(np.clip(d @ sun, -1.0, 1.0))
    sig = math.radians(sun_sigma_deg)
    color = np.array([1.0, 0.92, 0.78])
    color = color / (0.2126 * color[0] + 0.7152 * color[1] + 0.0722 * color[2])
    sky = sky + sun_peak * np.exp(-0.5 * (ang / sig) ** 2)[..., None] * color
    return rgbe_encode(sky)


def value_noise_rgba8(size: int, seed: int, cells: int = 16) -> np.ndarray:
    """RGBA8 value-noise texture (independent noise per channel, alpha 255)."""
    yy, xx = np.meshgrid(np.arange(size) + 0.5, np.arange(size) + 0.5, indexing="ij")
    p = np.stack([xx * cells / size, yy * cells / size, np.zeros_like(xx)], axis=-1)
    out = np.full((size, size, 4), 255, np.uint8)
    for c in range(3):
        n = 0.6 * value_noise3(p, seed + c) + 0.4 * value_noise3(p * 4.0, seed + 10 + c)
        out[..., c] = np.clip(np.floor(n * 255.0 + 0.5), 0, 255).astype(np.uint8)
    return out


# ---------------------------------------------------------------------------------------------
# scene descriptions


@dataclass
class MeshDesc:
    positions: np.ndarray  # (N, 3, 3) float32 triangle corners
    uvs: Optional[np.ndarray]  # (N, 3, 2) float32 or None
    smooth_normals: bool = True


@dataclass
class TextureDesc:
    texels: np.ndarray  # (H, W, 3) float32
    filter: int = 0
    tiling: tuple = (1.0, 1.0)


@dataclass
class ObjectDesc:
    name: str
    transform: Transform
    material: dict  # Material fields; texture fields are indices into SceneDesc.textures
    shape: tuple  # ("mesh", idx) | ("sphere", center, radius) | ("box", min, max)


@dataclass
class SceneDesc:
    name: str = "scene"
    meshes: list = field(default_factory=list)
    textures: list = field(default_factory=list)
    objects: list = field(default_factory=list)
    sky: tuple = ()  # ("texture", tex_idx, multiplier, yaw) | ("procedural", SkyProcedural)
    fog: Optional[Fog] = None
    view: View = field(default_factory=View)
    width: int = 64
    height: int = 64
    spp: int = 4
    bounces: int = 4
    min_samples: Optional[int] = None
    variance_threshold: float = 0.075
    indirect_clamp: float = 10.0
    block_size: int = 32

    @property
    def triangle_count(self) -> int:
        return int(sum(m.positions.shape[0] for m in self.meshes))

    def render_args(self):
        mn = self.min_samples if self.min_samples is not None else self.spp
        return (self.width, self.height, self.block_size, mn, self.spp, self.variance_threshold, self.bounces,
                self.indirect_clamp)

    def material_c(self, obj: ObjectDesc, tex_ids: list):
        m = dict(obj.material)
        kw = {k: m[k] for k in ("albedo", "roughness", "metallic", "transparency", "ior", "radiance") if k in m}
        mat = Material(**kw)
        mc = mat.to_c()
        for key in ("color_texture", "roughness_texture", "metallic_texture", "normal_texture"):
            setattr(mc, key, tex_ids[m[key]] if m.get(key) is not None else -1)
        return mc

    def shape_c(self, obj: ObjectDesc, mesh_ids: list):
        s = _abi.SrShape()
        kind = obj.shape[0]
        if kind == "mesh":
            s.kind, s.mesh = _abi.SR_SHAPE_MESH, mesh_ids[obj.shape[1]]
        elif kind == "sphere":
            s.kind, s.mesh = _abi.SR_SHAPE_SPHERE, -1
            s.params[:4] = [*map(float, obj.shape[1]), float(obj.shape[2])]
        else:
            s.kind, s.mesh = _abi.SR_SHAPE_AABOX, -1
            s.params[:] = [*map(float, obj.shape[1]), *map(float, obj.shape[2])]
        return s

    def instantiate(self, ctx: Context) -> Scene:
        """Build this scene in the GPU library through the public API."""
        textures = [Texture(ctx, t.texels, TextureFilter(t.filter), t.tiling) for t in self.textures]
        meshes = [Mesh.from_corners(ctx, m.positions, m.uvs, None, m.smooth_normals) for m in self.meshes]
        scene = Scene(ctx)
        if self.sky[0] == "texture":
            scene.set_sky(SkyTexture(textures[self.sky[1]], self.sky[2], self.sky[3]))
        else:
            scene.set_sky(self.sky[1])
        if self.fog is not None:
            scene.set_fog(self.fog)
        for o in self.objects:
            m = dict(o.material)
            kw = {k: m[k] for k in ("albedo", "roughness", "metallic", "transparency", "ior", "radiance") if k in m}
            for key in ("color_texture", "roughness_texture", "metallic_texture", "normal_texture"):
                if m.get(key) is not None:
                    kw[key] = textures[m[key]]
            kind = o.shape[0]
            shape = meshes[o.shape[1]] if kind == "mesh" else (
                Sphere(o.shape[1], o.shape[2]) if kind == "sphere" else AABox(o.shape[1], o.shape[2]))
            scene.add_object(Object(o.name, o.transform, Material(**kw), shape))
        scene._keepalive = (textures, meshes)
        return scene


def look_rotation(pos, target) -> Quat:
    """Yaw-then-pitch rotation taking +Z to the direction pos -> target (float32 quaternion)."""
    d = np.asarray(target, np.float64) - np.asarray(pos, np.float64)
    yaw = math.atan2(d[0], d[2])
    pitch = -math.atan2(d[1], math.hypot(d[0], d[2]))
    return Quat.angle_axis(yaw, (0.0, 1.0, 0.0)) * Quat.angle_axis(pitch, (1.0, 0.0, 0.0))


def _rgbe_texels(rgbe: np.ndarray) -> np.ndarray:
    return Texture.rgbe_to_linear(rgbe)


def config_c1(width: int = 256, height: int = 256, spp: int = 16) -> SceneDesc:
    """Plain method, CPU-runnable: 256x256, 16 spp, max depth 4, no fog; ~20k-tri fBm icosphere on a
    ground quad; one GGX material (albedo 0.7, roughness 0.4, metallic 0); 512x256 procedural sky
    (gradient + Gaussian sun, peak luminance 50) from seed 1; 45 degree pinhole camera."""
    pos, uv = displaced_icosphere(5, 0.1, seed=1)
    gpos, guv = ground_quad(8.0, -1.12)
    d = SceneDesc("c1_plain_256_16spp")
    d.meshes = [MeshDesc(pos, uv), MeshDesc(gpos, guv)]
    d.textures = [TextureDesc(_rgbe_texels(sky_env(512, 256, seed=1, sun_peak=50.0)))]
    d.sky = ("texture", 0, 1.0, 0.0)
    mat = {"albedo": (0.7, 0.7, 0.7), "roughness": 0.4, "metallic": 0.0}
    d.objects = [ObjectDesc("sphere", Transform(), mat, ("mesh", 0)),
                 ObjectDesc("ground", Transform(), mat, ("mesh", 1))]
    cam = (0.0, 0.9, -3.6)
    d.view = View(Transform(cam, look_rotation(cam, (0.0, -0.15, 0.0))), math.radians(45.0), 0.1)
    d.width, d.height, d.spp, d.bounces = width, height, spp, 4
    return d


def config_c2(width: int = 1920, height: int = 1080, spp: int = 64, rings: int = 660, rock_rings: int = 50,
              rocks: int = 64, env=(2048, 1024)) -> SceneDesc:
    """Plain GPU vs reference CPU: 1920x1080, 64 spp, depth 8, fog 0.02; fBm sphere (CreateSphere
    topology 660x660 = 871,200 triangles) + 64 instances of one 5,000-triangle rock; per-object
    roughness U[0.05, 1], metallic Bernoulli(0.3), albedo U[0.1, 0.9]^3; 2048x1024 HDR env with a
    lognormal (sigma 1) luminance field and a sun lobe; 512x512 RGBA8 value-noise albedo; seed 2."""
    rng = np.random.default_rng(2)
    pos, uv = uv_sphere(rings, rings, amplitude=0.1, seed=2)
    rpos, ruv = uv_sphere(rock_rings, rock_rings, amplitude=0.3, seed=22)
    d = SceneDesc(f"c2_plain_{width}x{height}_{spp}spp")
    d.meshes = [MeshDesc(pos, uv), MeshDesc(rpos, ruv)]
    d.textures = [TextureDesc(_rgbe_texels(sky_env(env[0], env[1], seed=2, sun_peak=400.0, sun_sigma_deg=1.5,
                                                   lognormal_sigma=1.0))),
                  TextureDesc(Texture.srgb_to_linear(value_noise_rgba8(512, seed=2)), 0, (4.0, 2.0))]
    d.sky = ("texture", 0, 1.0, 0.0)

    def material():
        return {"albedo": tuple(float(x) for x in rng.uniform(0.1, 0.9, 3)),
                "roughness": float(rng.uniform(0.05, 1.0)), "metallic": float(rng.random() < 0.3),
                "color_texture": 1}

    d.objects = [ObjectDesc("sphere", Transform(), material(), ("mesh", 0))]
    for i in range(rocks):
        rad = math.sqrt(rng.uniform(2.0 ** 2, 6.5 ** 2))
        ang = rng.uniform(0.0, 2.0 * math.pi)
        p = (rad * math.cos(ang), -1.0 + rng.uniform(-0.25, 0.25), rad * math.sin(ang))
        axis = rng.normal(size=3)
        axis = axis / np.linalg.norm(axis)
        rot = Quat.angle_axis(float(rng.uniform(0.0, 2.0 * math.pi)), tuple(float(a) for a in axis))
        s = float(rng.uniform(0.18, 0.45))
        d.objects.append(ObjectDesc(f"rock_{i}", Transform(p, rot, (s, s * 0.7, s)), material(), ("mesh", 1)))
    d.fog = Fog(0.02, (0.8, 0.75, 0.6), 0.6, 0.01)
    cam = (0.0, 1.1, -5.0)
    d.view = View(Transform(cam, look_rotation(cam, (0.0, -0.35, 0.0))), math.radians(60.0), 0.1)
    d.width, d.height, d.spp, d.bounces = width, height, spp, 8
    return d


def config_batch(count: int = 32, seed: int = 3) -> list:
    """Batched workload: `count` independent scenes, each one fBm-displaced sphere (CreateSphere
    topology) with a triangle count log-uniform in [1k, 1M], a resolution from {256x256, 512x512,
    1024x768, 1920x1080}, spp from {4, 16, 64}, depth U{4..8}, fog (0.02) on for half; one GGX
    material per scene (roughness U[0.05, 1], metallic Bernoulli(0.3), albedo U[0.1, 0.9]^3) and a
    256x128 HDR env with a sun lobe; seed 3."""
    rng = np.random.default_rng(seed)
    sizes = [(256, 256), (512, 512), (1024, 768), (1920, 1080)]
    out = []
    for i in range(count):
        tris = math.exp(rng.uniform(math.log(1e3), math.log(1e6)))
        rings = max(8, int(round(math.sqrt(tris / 2.0))))
        w, h = sizes[int(rng.integers(len(sizes)))]
        spp = int(rng.choice([4, 16, 64]))
        bounces = int(rng.integers(4, 9))
        fog = bool(rng.random() < 0.5)
        pos, uv = uv_sphere(rings, rings, amplitude=0.1, seed=seed * 1000 + i)
        d = SceneDesc(f"batch{i}_{2 * rings * rings}tris_{w}x{h}_{spp}spp")
        d.meshes = [MeshDesc(pos, uv)]
        d.textures = [TextureDesc(_rgbe_texels(sky_env(256, 128, seed=seed * 1000 + i, sun_peak=200.0,
                                                       sun_sigma_deg=2.0, lognormal_sigma=1.0)))]
        d.sky = ("texture", 0, 1.0, 0.0)
        d.objects = [ObjectDesc("sphere", Transform(),
                                {"albedo": tuple(float(x) for x in rng.uniform(0.1, 0.9, 3)),
                                 "roughness": float(rng.uniform(0.05, 1.0)), "metallic": float(rng.random() < 0.3)},
                                ("mesh", 0))]
        if fog:
            d.fog = Fog(0.02, (0.8, 0.75, 0.6), 0.6, 0.01)
        cam = (0.0, 0.8, -3.0)
        d.view = View(Transform(cam, look_rotation(cam, (0.0, 0.0, 0.0))), math.radians(55.0), 0.1)
        d.width, d.height, d.spp, d.bounces = w, h, spp, bounces
        out.append(d)
    return out


def value_noise_float(size: int, seed: int, lo: float, hi: float, channels: int = 3, cells: int = 16) -> np.ndarray:
    """Float32 value noise in [lo, hi], (size, size, channels) (the same field as value_noise_rgba8,
    unquantised)."""
    yy, xx = np.meshgrid(np.arange(size) + 0.5, np.arange(size) + 0.5, indexing="ij")
    p = np.stack([xx * cells / size, yy * cells / size, np.zeros_like(xx)], axis=-1)
    out = np.empty((size, size, channels), np.float32)
    for c in range(channels):
        n = 0.6 * value_noise3(p, seed + c) + 0.4 * value_noise3(p * 4.0, seed + 10 + c)
        out[..., c] = lo + (hi - lo) * np.clip(n, 0.0, 1.0)
    return out


def config_c4(width: int = 512, height: int = 512, spp: int = 16, rings: int = 316, tex: int = 512,
              seed: int = 4) -> SceneDesc:
    """Differentiable workload: 512x512, 16 spp, depth 6; fBm-displaced sphere (CreateSphere topology
    316x316 = 199,712 triangles) with a 512x512 float RGB albedo texture (value noise in [0.1, 0.9])
    and a 512x512 roughness texture (value noise in [0.05, 1]), metallic 0; 512x256 HDR env with a
    sun lobe; no fog; seed 4.  Texture 1 is the albedo, texture 2 the roughness."""
    pos, uv = uv_sphere(rings, rings, amplitude=0.1, seed=seed)
    d = SceneDesc(f"c4_adjoint_{width}x{height}_{spp}spp")
    d.meshes = [MeshDesc(pos, uv)]
    rough = value_noise_float(tex, seed + 50, 0.05, 1.0, channels=1)
    d.textures = [TextureDesc(_rgbe_texels(sky_env(512, 256, seed=seed, sun_peak=100.0, sun_sigma_deg=3.0,
                                                   lognormal_sigma=0.5))),
                  TextureDesc(value_noise_float(tex, seed, 0.1, 0.9)),
                  TextureDesc(np.repeat(rough, 3, axis=2))]
    d.sky = ("texture", 0, 1.0, 0.0)
    d.objects = [ObjectDesc("sphere", Transform(), {"albedo": (1.0, 1.0, 1.0), "roughness": 1.0, "metallic": 0.0,
                                                    "color_texture": 1, "roughness_texture": 2}, ("mesh", 0))]
    cam = (0.0, 0.4, -2.9)
    d.view = View(Transform(cam, look_rotation(cam, (0.0, 0.0, 0.0))), math.radians(50.0), 0.1)
    d.width, d.height, d.spp, d.bounces = width, height, spp, 6
    d.min_samples = spp
    d.variance_threshold = 0.0
    return d


def config_c5(width: int = 768, height: int = 768, spp: int = 32, rings: int = 500, tex: int = 1024,
              seed: int = 5) -> SceneDesc:
    """Batched + differentiable workload, one view of it: 768x768, 32 spp, depth 8; fBm sphere
    (CreateSphere topology 500x500 = 500,000 triangles) with 1024x1024 albedo (value noise in
    [0.1, 0.9]) and roughness (value noise in [0.05, 1]) textures, metallic 0; near-homogeneous fog
    (density 0.03, falloff 0.01); 1024x512 HDR env; seed 5.  Texture 1 is the albedo, texture 2 the
    roughness; the other views orbit the sphere (bench.py)."""
    pos, uv = uv_sphere(rings, rings, amplitude=0.1, seed=seed)
    d = SceneDesc(f"c5_differentiable_{width}x{height}_{spp}spp")
    d.meshes = [MeshDesc(pos, uv)]
    rough = value_noise_float(tex, seed + 50, 0.05, 1.0, channels=1)
    d.textures = [TextureDesc(_rgbe_texels(sky_env(1024, 512, seed=seed, sun_peak=100.0, sun_sigma_deg=3.0,
                                                   lognormal_sigma=0.5))),
                  TextureDesc(value_noise_float(tex, seed, 0.1, 0.9)),
                  TextureDesc(np.repeat(rough, 3, axis=2))]
    d.sky = ("texture", 0, 1.0, 0.0)
    d.objects = [ObjectDesc("sphere", Transform(), {"albedo": (1.0, 1.0, 1.0), "roughness": 1.0, "metallic": 0.0,
                                                    "color_texture": 1, "roughness_texture": 2}, ("mesh", 0))]
    d.fog = Fog(0.03, (0.8, 0.75, 0.6), 0.6, 0.01)
    cam = (0.0, 0.4, -2.9)
    d.view = View(Transform(cam, look_rotation(cam, (0.0, 0.0, 0.0))), math.radians(50.0), 0.1)
    d.width, d.height, d.spp, d.bounces = width, height, spp, 8
    d.min_samples = spp
    d.variance_threshold = 0.0
    return d


def config_features(width: int = 48, height: int = 40, spp: int = 8, seed: int = 5) -> SceneDesc:
    """Small scene touching every shading branch: textured/normal-mapped/point-filtered materials,
    transparent (refractive) sphere, metal box, emissive object, instanced transformed mesh, fog."""
    rng = np.random.default_rng(seed)
    pos, uv = displaced_icosphere(3, 0.15, seed=seed)
    rpos, ruv = uv_sphere(12, 16, amplitude=0.2, seed=seed + 1)
    gpos, guv = ground_quad(6.0, -1.2)
    d = SceneDesc("features")
    d.meshes = [MeshDesc(pos, uv), MeshDesc(rpos, ruv), MeshDesc(gpos, guv, smooth_normals=False)]
    noise = value_noise_rgba8(64, seed=seed + 3, cells=8)
    d.textures = [TextureDesc(_rgbe_texels(sky_env(128, 64, seed=seed, sun_peak=30.0, sun_sigma_deg=4.0))),
                  TextureDesc(Texture.srgb_to_linear(noise), 0, (3.0, 3.0)),
                  TextureDesc(noise[..., :3].astype(np.float32) / np.float32(255.0), 1, (2.0, 2.0)),
                  TextureDesc(Texture.srgb_to_linear(value_noise_rgba8(32, seed=seed + 4, cells=4)), 0, (1.0, 1.0))]
    d.sky = ("texture", 0, 1.0, 0.7)
    d.objects = [
        ObjectDesc("blob", Transform((0.0, 0.0, 0.0), Quat.angle_axis(0.4, (0.0, 1.0, 0.0)), (1.0, 1.0, 1.0)),
                   {"albedo": (0.8, 0.6, 0.5), "roughness": 0.5, "metallic": 0.0, "color_texture": 1,
                    "normal_texture": 3}, ("mesh", 0)),
        ObjectDesc("glass", Transform(), {"albedo": (0.9, 0.95, 1.0), "roughness": 0.05, "transparency": 0.9,
                                          "ior": 1.5}, ("sphere", (1.6, -0.6, 0.3), 0.55)),
        ObjectDesc("metalbox", Transform((-1.7, -0.7, 0.5), Quat.angle_axis(0.6, (0.0, 1.0, 0.0)), (1.0, 1.0, 1.0)),
                   {"albedo": (0.9, 0.7, 0.3), "roughness": 0.25, "metallic": 1.0, "roughness_texture": 2},
                   ("box", (-0.4, -0.5, -0.4), (0.4, 0.5, 0.4))),
        ObjectDesc("lamp", Transform(), {"albedo": (0.2, 0.2, 0.2), "roughness": 0.9, "radiance": (6.0, 5.0, 3.0)},
                   ("sphere", (0.3, 1.4, 1.5), 0.25)),
        ObjectDesc("ground", Transform(), {"albedo": (0.6, 0.6, 0.6), "roughness": 0.8, "color_texture": 2},
                   ("mesh", 2)),
    ]
    for i in range(3):
        p = (float(rng.uniform(-2.5, 2.5)), -0.9, float(rng.uniform(1.0, 3.0)))
        rot = Quat.angle_axis(float(rng.uniform(0, 6.28)), (0.0, 1.0, 0.0))
        d.objects.append(ObjectDesc(f"rock{i}", Transform(p, rot, (0.3, 0.25, 0.35)),
                                    {"albedo": (0.5, 0.5, 0.45), "roughness": 0.7, "metallic": 0.0},
                                    ("mesh", 1)))
    d.fog = Fog(0.05, (0.8, 0.75, 0.6), 0.6, 0.2)
    cam = (0.0, 0.8, -4.5)
    d.view = View(Transform(cam, look_rotation(cam, (0.0, -0.2, 0.5))), math.radians(60.0), 0.1)
    d.width, d.height, d.spp, d.bounces = width, height, spp, 6
    return d


def config_procedural(width: int = 40, height: int = 32, spp: int = 8) -> SceneDesc:
    """Procedural sky + sun (SkyProcedural) over an icosphere and ground."""
    pos, uv = displaced_icosphere(2, 0.1, seed=9)
    gpos, guv = ground_quad(5.0, -1.1)
    d = SceneDesc("procedural_sky")
    d.meshes = [MeshDesc(pos, uv), MeshDesc(gpos, guv)]
    d.sky = ("procedural", SkyProcedural((0.08, 0.17, 0.70), (0.50, 0.65, 0.90), (0.12, 0.09, 0.07),
                                         tuple(np.array([0.5, 1.0, -0.5]) / math.sqrt(1.5)),
                                         (1000.0, 900.0, 650.0), math.radians(3.0)))
    d.objects = [ObjectDesc("ball", Transform(), {"albedo": (0.7, 0.3, 0.2), "roughness": 0.3}, ("mesh", 0)),
                 ObjectDesc("ground", Transform(), {"albedo": (0.5, 0.5, 0.5), "roughness": 0.9}, ("mesh", 1))]
    cam = (0.0, 0.7, -3.5)
    d.view = View(Transform(cam, look_rotation(cam, (0.0, -0.1, 0.0))), math.radians(50.0), 0.1)
    d.width, d.height, d.spp, d.bounces = width, height, spp, 5
    return d


def default_compositor() -> Compositor:
    """Compositor settings of program.cs:28-40."""
    return Compositor()
