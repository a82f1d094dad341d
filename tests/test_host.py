"""Host-side logic of the product (CPU, host-only context): triangle ingest and the binned-SAH BVH
builds must be bit-identical to the oracle's restatement of bvh.cs / mesh.cs / math.cs."""
import numpy as np
import pytest

from sharpray_gb300 import Mesh, synth


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _same_bvh(a, b):
    return all(np.array_equal(_bits(x), _bits(y)) for x, y in zip(a, b))


MESHES = {
    "icosphere_s4": lambda: synth.displaced_icosphere(4, 0.1, seed=1),
    "uv_sphere_40": lambda: synth.uv_sphere(40, 40, amplitude=0.2, seed=3),
    "ground": lambda: synth.ground_quad(5.0, -1.0),
}


@pytest.mark.parametrize("name", sorted(MESHES))
@pytest.mark.parametrize("smooth", [True, False])
def test_ingest_bit_exact(host_ctx, oracle_mod, name, smooth):
    pos, uv = MESHES[name]()
    ours = Mesh.triangles_from_corners(host_ctx, pos, uv, None, smooth)
    ref = oracle_mod.triangles_from_corners(pos, uv, None, smooth)
    assert np.array_equal(_bits(ours), _bits(ref))


def test_ingest_with_normals_and_default_uvs(host_ctx, oracle_mod):
    pos, _ = synth.uv_sphere(8, 8)
    rng = np.random.default_rng(0)
    n = rng.normal(size=pos.shape).astype(np.float32)
    ours = Mesh.triangles_from_corners(host_ctx, pos, None, n, True)
    ref = oracle_mod.triangles_from_corners(pos, None, n, True)
    assert np.array_equal(_bits(ours), _bits(ref))


@pytest.mark.parametrize("name", sorted(MESHES))
def test_mesh_bvh_bit_exact(host_ctx, oracle_mod, name):
    pos, uv = MESHES[name]()
    tris = Mesh.triangles_from_corners(host_ctx, pos, uv)
    ours = Mesh(host_ctx, tris).bvh()
    s = oracle_mod.OracleScene()
    ref = s.mesh_bvh(s.mesh(tris))
    assert ours[0].shape == ref[0].shape
    assert _same_bvh(ours, ref)
    # structural invariants of bvh.cs: children consecutive, leaves cover every item once
    bounds, links, items = ours
    assert sorted(items.tolist()) == list(range(len(tris)))


def test_degenerate_and_clustered_meshes(host_ctx, oracle_mod):
    """Edge cases: duplicate triangles, zero-area triangles, a cluster of nearly coincident
    centroids far from the origin (where the split position can round onto the minimum)."""
    rng = np.random.default_rng(11)
    base = rng.normal(size=(50, 3, 3)).astype(np.float32)
    dup = np.repeat(base[:5], 4, axis=0)
    flat = base[5:10].copy()
    flat[:, 2] = flat[:, 0]  # zero area
    cluster = (np.float32(1000.0) + rng.normal(scale=1e-4, size=(40, 3, 3))).astype(np.float32)
    pos = np.concatenate([base, dup, flat, cluster]).astype(np.float32)
    tris = Mesh.triangles_from_corners(host_ctx, pos, None, None, True)
    assert np.array_equal(_bits(tris), _bits(oracle_mod.triangles_from_corners(pos, None, None, True)))
    ours = Mesh(host_ctx, tris).bvh()
    s = oracle_mod.OracleScene()
    assert _same_bvh(ours, s.mesh_bvh(s.mesh(tris)))


def test_empty_and_single_triangle_mesh(host_ctx, oracle_mod):
    s = oracle_mod.OracleScene()
    for n in (0, 1):
        pos = np.zeros((n, 3, 3), np.float32)
        if n:
            pos[0] = [[0, 0, 0], [1, 0, 0], [0, 1, 0]]
        tris = Mesh.triangles_from_corners(host_ctx, pos)
        ours = Mesh(host_ctx, tris).bvh()
        assert _same_bvh(ours, s.mesh_bvh(s.mesh(tris)))
        assert ours[0].shape[0] == n


def test_scene_bvh_bit_exact(host_ctx, oracle_mod):
    d = synth.config_features()
    ours = d.instantiate(host_ctx)
    ours.build()
    ref = oracle_mod.instantiate(d)
    assert _same_bvh(ours.bvh(), ref.bvh())
    for i in range(len(d.meshes)):
        assert _same_bvh(ours._keepalive[1][i].bvh(), ref.mesh_bvh(i))


def test_c2_scene_bvh_reduced(host_ctx, oracle_mod):
    """The 65-object C2 layout (meshes reduced so the check stays fast): the 32-bin scene BVH over
    rotated/scaled instance bounds is bit-identical."""
    d = synth.config_c2(64, 36, 1, rings=40, rock_rings=10, env=(64, 32))
    ours = d.instantiate(host_ctx)
    ours.build()
    ref = oracle_mod.instantiate(d)
    assert _same_bvh(ours.bvh(), ref.bvh())


def test_bvh_build_entry_matches_mesh_build(host_ctx):
    """sr_bvh_build over a mesh's triangle bounds gives the mesh's own tree (host build)."""
    pos, uv = synth.uv_sphere(24, 24, amplitude=0.2, seed=7)
    tris = Mesh.triangles_from_corners(host_ctx, pos, uv)
    a, ab, ac = tris[:, 0:3], tris[:, 0:3] + tris[:, 3:6], tris[:, 0:3] + tris[:, 6:9]
    b = np.concatenate([np.minimum(np.minimum(a, ab), ac), np.maximum(np.maximum(a, ab), ac)], 1)
    assert _same_bvh(host_ctx.build_bvh(b, 1.0, 0.5, 8), Mesh(host_ctx, tris).bvh())


def test_device_bvh_build_needs_a_device(host_ctx):
    from sharpray_gb300 import _abi
    from sharpray_gb300._abi import StateError
    with pytest.raises(StateError):
        host_ctx.set_bvh_build(_abi.SR_BVH_BUILD_DEVICE)
    with pytest.raises(StateError):
        host_ctx.build_bvh(np.zeros((4, 6), np.float32), 1.0, 0.5, 8, where=_abi.SR_BVH_BUILD_DEVICE)


def test_tuning_validation(host_ctx):
    import ctypes as C

    from sharpray_gb300 import Scene, SharpRayError, _abi
    s = Scene(host_ctx)
    s.set_tuning(3, 4, 2, 8)
    t = _abi.SrTuning()
    _abi.check(host_ctx._lib.sr_scene_get_tuning(s.handle, C.byref(t)))
    assert (t.trace_blocks_per_sm, t.fog_shade_blocks_per_sm, t.surface_shade_blocks_per_sm, t.tail_divisor) == (3, 4, 2, 8)
    with pytest.raises(SharpRayError):
        s.set_tuning(-1)


def test_context_outlived_by_scene(native_lib):
    """Destroying a context before its scenes (finalisers run in any order) defers the free."""
    import ctypes as C
    from sharpray_gb300 import _abi
    ctx, sc = C.c_void_p(), C.c_void_p()
    _abi.check(native_lib.sr_ctx_create(-1, C.byref(ctx)))
    _abi.check(native_lib.sr_scene_create(ctx, C.byref(sc)))
    _abi.check(native_lib.sr_ctx_destroy(ctx))
    _abi.check(native_lib.sr_scene_destroy(sc))


def test_progress_adjoint_and_update_validation(host_ctx):
    """Argument and state checks of the progress, adjoint, texture/fog update and float-compose entry
    points (none reaches the GPU)."""
    import ctypes as C

    from sharpray_gb300 import Scene, SharpRayError, StateError, _abi
    lib = host_ctx._lib
    s = Scene(host_ctx)
    assert s.progress() == (0, 0)  # nothing launched
    assert s.seed == 0
    s.set_seed(9)
    assert s.seed == 9
    # the getter reads the C scene, so a direct call through the ABI is seen too
    _abi.check(lib.sr_scene_set_seed(s.handle, 0xFFFFFFFF))
    assert s.get_seed() == 0xFFFFFFFF
    for bad in (-1, 1 << 32):
        with pytest.raises(ValueError):
            s.set_seed(bad)
    assert s.get_seed() == 0xFFFFFFFF
    s.set_seed(0)
    with pytest.raises(SharpRayError):
        _abi.check(lib.sr_scene_set_seed(None, 1))
    with pytest.raises(SharpRayError):
        _abi.check(lib.sr_scene_get_seed(s.handle, None))
    # loop caps round-trip through the tuning (the renders that hit them are GPU tests)
    s.set_tuning(max_bounce_iterations=6, max_traversal_steps=40)
    t = s.get_tuning()
    assert (t["max_bounce_iterations"], t["max_traversal_steps"]) == (6, 40)
    s.set_tuning()
    assert s.get_tuning()["max_traversal_steps"] == 0
    s.set_tuning(trace_block_threads=256)
    assert s.get_tuning()["trace_block_threads"] == 256
    with pytest.raises(SharpRayError):
        s.set_tuning(trace_block_threads=96)
    s.set_tuning()
    d, t = C.c_uint32(), C.c_uint32()
    with pytest.raises(SharpRayError):
        _abi.check(lib.sr_render_progress(s.handle, None, C.byref(t)))
    with pytest.raises(StateError):  # not built
        s.update_fog_density(0.1)
    with pytest.raises(StateError):
        s.update_texture(0, np.zeros((1, 1, 3), np.float32))
    v, p, a = _abi.SrView(), _abi.SrRenderParams(), _abi.SrAovs()
    g = (C.c_float * 3)()
    for call in (lambda: lib.sr_adjoint_texture(s.handle, C.byref(v), C.byref(p), C.byref(a), g, 0, 0, g, None, None),
                 lambda: lib.sr_adjoint_all(s.handle, C.byref(v), C.byref(p), C.byref(a), g, 0, g, -1, None, None,
                                            None, None),
                 lambda: lib.sr_adjoint_texture(s.handle, C.byref(v), C.byref(p), None, g, 0, 0, g, None, None),
                 lambda: lib.sr_adjoint_texture(s.handle, C.byref(v), C.byref(p), C.byref(a), g, 0, 7, g, None,
                                                None),
                 lambda: lib.sr_compose_float_device(host_ctx.handle, C.byref(a), 4, 4, None, None, None, None)):
        with pytest.raises(SharpRayError):
            _abi.check(call())
