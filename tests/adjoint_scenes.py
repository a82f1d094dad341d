"""Scenes shared by the adjoint tests (GPU: tests/test_adjoint.py; CPU oracle:
tests/test_oracle_adjoint.py)."""
import math

import numpy as np

from sharpray_gb300 import Fog, Quat, Transform, View, synth
from sharpray_gb300.synth import MeshDesc, ObjectDesc, SceneDesc, TextureDesc, look_rotation


def adjoint_scene(fog: bool, bounces: int, clamp: float, w=40, h=30, spp=3, general: bool = False,
                  metal: bool = False) -> SceneDesc:
    """Textured ground and blob sharing one bilinear albedo texture (different material albedos,
    tiling 2 on the blob), a point-filtered texture on a second blob, an untextured rock; `general`
    adds an analytic sphere with the bilinear texture (the kernels' general instantiation); `metal`
    makes the textured blob fully metallic (its albedo then enters through the Fresnel base; the
    lobe probability clamps to a constant, so sampling still does not depend on the albedo)."""
    rng = np.random.default_rng(7)
    gpos, guv = synth.ground_quad(3.0, -1.0)
    bpos, buv = synth.uv_sphere(10, 14, amplitude=0.1, seed=2)
    rpos, ruv = synth.uv_sphere(8, 10, amplitude=0.2, seed=4)
    d = SceneDesc("adjoint")
    d.meshes = [MeshDesc(gpos, guv, smooth_normals=False), MeshDesc(bpos, buv), MeshDesc(rpos, ruv)]
    d.textures = [TextureDesc(synth._rgbe_texels(synth.sky_env(64, 32, seed=3, sun_peak=20.0, sun_sigma_deg=6.0))),
                  TextureDesc(rng.uniform(0.2, 0.9, (6, 8, 3)).astype(np.float32), 0, (1.0, 1.0)),
                  TextureDesc(rng.uniform(0.2, 0.9, (4, 4, 3)).astype(np.float32), 1, (1.0, 1.0))]
    d.sky = ("texture", 0, 1.0, 0.3)
    d.objects = [
        ObjectDesc("ground", Transform(), {"albedo": (0.9, 0.8, 0.7), "roughness": 0.7, "color_texture": 1},
                   ("mesh", 0)),
        ObjectDesc("blob", Transform((-0.6, -0.2, 0.8), Quat.identity(), (0.7, 0.7, 0.7)),
                   {"albedo": (1.0, 0.9, 0.8), "roughness": 0.4, "color_texture": 1}, ("mesh", 1)),
        ObjectDesc("pointblob", Transform((0.9, -0.4, 0.4), Quat.angle_axis(0.5, (0.0, 1.0, 0.0)), (0.5, 0.5, 0.5)),
                   {"albedo": (0.8, 0.8, 0.8), "roughness": 0.5, "color_texture": 2}, ("mesh", 1)),
        ObjectDesc("rock", Transform((0.2, -0.7, -0.6), Quat.identity(), (0.3, 0.3, 0.3)),
                   {"albedo": (0.5, 0.5, 0.45), "roughness": 0.6}, ("mesh", 2)),
    ]
    if metal:
        d.objects[1].material["metallic"] = 1.0
    if general:
        d.objects.append(ObjectDesc("ball", Transform(), {"albedo": (0.7, 0.9, 0.8), "roughness": 0.5,
                                                          "color_texture": 1}, ("sphere", (0.6, -0.75, -0.3), 0.25)))
    # the blob's tiling: a second TextureDesc would be a second texture, so tile through its uvs
    d.meshes[1] = MeshDesc(bpos, buv * np.float32(2.0))
    if fog:
        d.fog = Fog(0.08, (0.8, 0.75, 0.7), 0.5, 0.2)
    cam = (0.0, 0.9, -3.2)
    d.view = View(Transform(cam, look_rotation(cam, (0.0, -0.4, 0.5))), math.radians(55.0), 0.1)
    d.width, d.height, d.spp, d.bounces = w, h, spp, bounces
    d.min_samples = spp
    d.variance_threshold = 0.0  # every pixel takes spp samples (count spp + 1, the loop's off-by-one)
    d.indirect_clamp = clamp
    return d


def roughness_scene(spp: int) -> SceneDesc:
    """adjoint_scene with a 4x4 roughness texture (its red channel) on the ground and the blob."""
    d = adjoint_scene(False, 2, 10.0, w=64, h=48, spp=spp)
    rough = np.random.default_rng(9).uniform(0.25, 0.8, (4, 4, 3)).astype(np.float32)
    d.textures.append(TextureDesc(rough, 0, (1.0, 1.0)))
    for o in d.objects[:2]:
        o.material["roughness"] = 1.0
        o.material["roughness_texture"] = 3
    return d
