"""Oracle pinning (CPU): published known answers, independent restatements, golden fixtures and
analytic cases the reference's arithmetic fixes exactly."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from sharpray_gb300 import synth
from sharpray_gb300.api import Quat, Transform, View, render_params
from tests.golden.make_golden import RNG_SEEDS, rng_reference_python, seeded_rays, sha

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_splitmix64_published_vector(oracle_mod):
    # splitmix64 (Steele/Lea/Flood; Vigna's reference code) from seed 1234567, as published.
    expected = [6457827717110365317, 3203168211198807973, 9817491932198370423, 4593380528125082431,
                16408922859458223821]
    assert [int(v) for v in oracle_mod.splitmix64(1234567, 5)] == expected


@pytest.mark.parametrize("seed", RNG_SEEDS)
def test_rng_matches_independent_restatement(oracle_mod, seed):
    u, f = oracle_mod.rng_stream(seed[0], seed[1], 4096)
    pu, pf = rng_reference_python(seed[0], seed[1], 4096)
    assert np.array_equal(u, pu)
    assert np.array_equal(f.view(np.uint32), pf.view(np.uint32))


def test_rng_golden(oracle_mod):
    fix = json.loads((GOLDEN / "rng.json").read_text())
    for key, want in fix.items():
        a, b = map(int, key.split(","))
        u, f = oracle_mod.rng_stream(a, b, 16)
        assert [int(x) for x in u] == want["uint"]
        assert [int(x) for x in f.view(np.uint32)] == want["float_bits"]


def test_rng_float_range(oracle_mod):
    _, f = oracle_mod.rng_stream(7, 9, 100000)
    assert f.min() >= 0.0 and f.max() < 1.0  # NextFloat is [0, 1): scale 1/(2^32+512)


def test_bvh_and_trace_golden(oracle_mod):
    fix = json.loads((GOLDEN / "hashes.json").read_text())
    d = synth.config_c1(32, 32, 1)
    scene = oracle_mod.instantiate(d)
    b = scene.mesh_bvh(0)
    assert b[0].shape[0] == fix["c1_sphere_bvh_nodes"]
    assert sha(*b) == fix["c1_sphere_bvh"]
    assert sha(*scene.bvh()) == fix["c1_scene_bvh"]
    hits = scene.trace(seeded_rays(4096, seed=7))
    assert int((hits["object"] >= 0).sum()) == fix["c1_trace_hits"]
    assert sha(hits["object"], hits["triangle"], hits["dist"], hits["uv"]) == fix["c1_trace_4096_seed7"]


def test_aov_golden_1spp(oracle_mod):
    g = np.load(GOLDEN / "c1_1spp.npz")
    d = synth.config_c1(32, 32, 1)
    aovs, _ = oracle_mod.render_desc(d)
    assert np.array_equal(aovs.samples, g["samples"])
    # primary hits are exact arithmetic (no transcendental before the first trace)
    assert np.array_equal(np.isinf(aovs.depth), np.isinf(g["depth"]))
    np.testing.assert_allclose(aovs.depth[np.isfinite(aovs.depth)], g["depth"][np.isfinite(g["depth"])], rtol=1e-6)
    np.testing.assert_allclose(aovs.radiance, g["radiance"], rtol=1e-3, atol=1e-5)


def _uniform_sky_desc(value: float, min_spp: int, max_spp: int, threshold: float):
    d = synth.SceneDesc("empty")
    d.textures = [synth.TextureDesc(np.full((8, 16, 3), value, np.float32))]
    d.sky = ("texture", 0, 1.0, 0.0)
    d.view = View(Transform((0.0, 0.0, 0.0)), math.radians(60.0), 0.1)
    d.width, d.height, d.spp, d.bounces = 8, 6, max_spp, 3
    d.min_samples, d.variance_threshold = min_spp, threshold
    return d


def test_empty_scene_sees_sky_exactly(oracle_mod):
    # No objects: every sample returns the sky radiance with MIS weight 1 and energy 1.
    aovs, _ = oracle_mod.render_desc(_uniform_sky_desc(0.75, 4, 8, 0.075))
    assert np.all(aovs.radiance == np.float32(0.75))
    assert np.all(np.isinf(aovs.depth)) and np.all(aovs.normals == 0)
    # zero variance converges at the first check (sampleIndex = minSamples - 1)
    assert np.all(aovs.samples == 4)


def test_unconverged_pixel_off_by_one(oracle_mod):
    # renderer.cs:173-215: a pixel that never converges leaves the loop with sampleIndex ==
    # maxSamples, so it is normalised by maxSamples + 1.
    aovs, _ = oracle_mod.render_desc(_uniform_sky_desc(0.5, 4, 4, -1.0))
    assert np.all(aovs.samples == 5)
    expected = np.float32(np.float32(0.5) * 4) / np.float32(5)
    assert np.all(aovs.radiance == expected)


def test_sphere_distance_analytic(oracle_mod):
    # Analytic sphere, rays aimed at the centre from distance D: t = D - r (within float rounding).
    from sharpray_gb300 import _abi
    s = oracle_mod.OracleScene()
    s.set_sky_texture(s.texture(np.ones((4, 8, 3), np.float32)))
    mat = synth.SceneDesc().material_c(synth.ObjectDesc("s", Transform(), {"albedo": (1, 1, 1), "roughness": 1},
                                                        ("sphere", (0, 0, 0), 1.0)), [])
    sh = _abi.SrShape()
    sh.kind, sh.mesh = _abi.SR_SHAPE_SPHERE, -1
    sh.params[:4] = [0.0, 0.0, 0.0, 1.0]
    s.add_object(Transform().to_c(), mat, sh)
    s.build()
    rng = np.random.default_rng(3)
    dirs = rng.normal(size=(256, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    D = rng.uniform(2.0, 10.0, size=(256, 1))
    rays = np.concatenate([dirs * D, -dirs], axis=1).astype(np.float32)
    hits = s.trace(rays)
    assert np.all(hits["object"] == 0)
    np.testing.assert_allclose(hits["dist"], (D[:, 0] - 1.0), rtol=1e-5)


def test_triangle_hit_barycentrics(oracle_mod):
    # One triangle in a mesh object: hit barycentrics reproduce the aimed point.
    s = oracle_mod.OracleScene()
    s.set_sky_texture(s.texture(np.ones((4, 8, 3), np.float32)))
    pos = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]]], np.float32)
    tris = oracle_mod.triangles_from_corners(pos)
    m = s.mesh(tris)
    from sharpray_gb300 import _abi
    sh = _abi.SrShape()
    sh.kind, sh.mesh = _abi.SR_SHAPE_MESH, m
    mat = synth.SceneDesc().material_c(synth.ObjectDesc("t", Transform(), {"albedo": (1, 1, 1), "roughness": 1},
                                                        ("mesh", 0)), [])
    s.add_object(Transform().to_c(), mat, sh)
    s.build()
    rays = np.array([[0.25, 0.5, -2.0, 0.0, 0.0, 1.0], [0.9, 0.9, -2.0, 0.0, 0.0, 1.0]], np.float32)
    h = s.trace(rays)
    assert h["object"][0] == 0 and h["triangle"][0] == 0 and h["object"][1] == -1
    np.testing.assert_allclose(h["dist"][0], 2.0, rtol=1e-6)
    np.testing.assert_allclose(h["uv"][0], [0.25, 0.5], rtol=1e-6)


def test_oracle_counters_consistent(oracle_mod):
    d = synth.config_c1(24, 24, 2)
    _, c = oracle_mod.render_desc(d, counters=True)
    assert c["sample"] == 24 * 24 * 2
    assert c["scene_trace"] == c["sample_bounce"]
    assert c["blas_node"] % 2 == 0 and c["tlas_node"] % 2 == 0
    assert 0 < c["hit_inflate"] and c["scene_occlude"] <= c["scene_trace"]
