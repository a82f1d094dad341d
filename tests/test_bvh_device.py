"""Device BVH build (SR_BVH_BUILD_DEVICE) against the host build.

The host build is bit-exact to bvh.cs (tests/test_host.py pins it against the oracle); the device
build must give the same tree: node bounds (bits), child/count links, item permutation and node
count -- for the mesh parameters (traverse 1, intersect 0.5, 8 bins) and the scene parameters
(1, 10, 32), on random, clustered, duplicated, flat and signed-zero inputs, the meshes of the
test scenes and the full C2 sphere.
"""
import time

import numpy as np
import pytest

from sharpray_gb300 import Context, Renderer, _abi, synth

pytestmark = pytest.mark.gpu

HOST, DEVICE = _abi.SR_BVH_BUILD_HOST, _abi.SR_BVH_BUILD_DEVICE


def random_bounds(n: int, seed: int, mode: str) -> np.ndarray:
    rng = np.random.default_rng(seed)
    c = rng.uniform(-10.0, 10.0, (n, 3))
    e = rng.uniform(0.0, 0.5, (n, 3))
    if mode == "clustered":
        centers = rng.uniform(-50.0, 50.0, (8, 3))
        c = centers[rng.integers(0, 8, n)] + rng.normal(0.0, 0.3, (n, 3))
    elif mode == "duplicates":
        base = rng.uniform(-5.0, 5.0, (max(1, n // 50), 3))
        c = base[rng.integers(0, len(base), n)]
        e = np.full((n, 3), 0.25)
    elif mode == "flat":
        c[:, 1] = 0.0
        e[:, 1] = 0.0
    elif mode == "signed_zero":
        c = rng.integers(-2, 3, (n, 3)).astype(np.float64)
        e = np.zeros((n, 3))
    lo, hi = (c - e).astype(np.float32), (c + e).astype(np.float32)
    if mode == "signed_zero":
        neg = rng.random((n, 3)) < 0.5
        lo = np.where((lo == 0) & neg, np.float32(-0.0), lo)
        hi = np.where((hi == 0) & ~neg, np.float32(-0.0), hi)
    return np.concatenate([lo, hi], 1).astype(np.float32)


def assert_same_tree(a, b):
    (ba, la, ia), (bb, lb, ib) = a, b
    assert ba.shape == bb.shape, (ba.shape, bb.shape)
    assert np.array_equal(ba.view(np.uint32), bb.view(np.uint32)), "node bounds differ"
    assert np.array_equal(la, lb), "child/count links differ"
    assert np.array_equal(ia, ib), "item permutation differs"


@pytest.mark.parametrize("params", [(1.0, 0.5, 8), (1.0, 10.0, 32)], ids=["mesh", "scene"])
@pytest.mark.parametrize("n,mode", [(0, "uniform"), (1, "uniform"), (2, "uniform"), (3, "flat"), (17, "uniform"),
                                    (1000, "uniform"), (5000, "clustered"), (3000, "duplicates"), (2000, "flat"),
                                    (500, "signed_zero"), (100000, "uniform")])
def test_device_build_matches_host(gpu_ctx, params, n, mode):
    b = random_bounds(n, 11 + n, mode)
    host = gpu_ctx.build_bvh(b, *params, where=HOST)
    dev = gpu_ctx.build_bvh(b, *params, where=DEVICE)
    assert_same_tree(host, dev)
    if n:
        assert sorted(host[2].tolist()) == list(range(n))


def scene_trees(desc, where):
    ctx = Context(0)
    ctx.set_bvh_build(where)
    scene = desc.instantiate(ctx)
    scene.build()
    meshes = scene._keepalive[1]
    return ctx, scene, [m.bvh() for m in meshes], scene.bvh()


@pytest.mark.parametrize("name", ["c1", "features", "c2_reduced"])
def test_scene_meshes_and_tlas_device_build(name):
    desc = {"c1": lambda: synth.config_c1(32, 32, 2), "features": lambda: synth.config_features(32, 24, 2),
            "c2_reduced": lambda: synth.config_c2(48, 27, 2, rings=120, rock_rings=50, env=(128, 64))}[name]()
    ctx_h, scene_h, meshes_h, tlas_h = scene_trees(desc, HOST)
    ctx_d, scene_d, meshes_d, tlas_d = scene_trees(desc, DEVICE)
    for a, b in zip(meshes_h, meshes_d):
        assert_same_tree(a, b)
    assert_same_tree(tlas_h, tlas_d)
    # the same trees render the same image
    ra = Renderer(scene_h, desc.view, *desc.render_args())
    rb = Renderer(scene_d, desc.view, *desc.render_args())
    for plane in ("radiance", "radiance_fog", "normals", "depth", "samples"):
        assert np.array_equal(getattr(ra, plane).view(np.uint32), getattr(rb, plane).view(np.uint32)), plane


def test_c2_sphere_device_build(gpu_ctx):
    """The 871,200-triangle C2 sphere mesh: identical tree, built much faster on the GPU."""
    from sharpray_gb300 import Mesh
    pos, uv = synth.uv_sphere(660, 660, amplitude=0.1, seed=2)
    tris = Mesh.triangles_from_corners(gpu_ctx, pos, uv, None, True)
    lo = np.minimum(np.minimum(tris[:, 0:3], tris[:, 0:3] + tris[:, 3:6]), tris[:, 0:3] + tris[:, 6:9])
    hi = np.maximum(np.maximum(tris[:, 0:3], tris[:, 0:3] + tris[:, 3:6]), tris[:, 0:3] + tris[:, 6:9])
    b = np.concatenate([lo, hi], 1).astype(np.float32)
    t0 = time.perf_counter()
    host = gpu_ctx.build_bvh(b, 1.0, 0.5, 8, where=HOST)
    t1 = time.perf_counter()
    dev = gpu_ctx.build_bvh(b, 1.0, 0.5, 8, where=DEVICE)
    t2 = time.perf_counter()
    assert_same_tree(host, dev)
    print(f"C2 sphere BVH ({len(b)} triangles, {len(host[0])} nodes): host {t1 - t0:.3f} s, device {t2 - t1:.3f} s")
