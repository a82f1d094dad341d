"""AOV images (program.cs:211-263), the debug overlay (overlay.cs) and image files (image.cs:88-212)
through the C ABI against the oracle (oracle_aov_image / oracle_overlay_draw in sr_oracle.cpp and
the writers in oracle/ingest.py).  Everything here is integer / byte output and compared exactly.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import ingest as ref
from sharpray_gb300 import (AABox, AovKind, Aovs, Font, Overlay, Quat, SharpRayError, Transform, View, _abi,
                            aov_image, load_image, save_image)
from sharpray_gb300.synth import look_rotation


# ---- image files (CPU) ---------------------------------------------------------------------------

@pytest.mark.parametrize("ext", [".tga", ".ppm", ".bmp"])
@pytest.mark.parametrize("shape", [(1, 1), (2, 3), (5, 4), (3, 7), (8, 6)])
def test_save_image_bytes(native_lib, tmp_path, ext, shape):
    rgb = np.random.default_rng(shape[0] * 10 + shape[1]).integers(0, 256, shape + (3,), dtype=np.uint8)
    path = tmp_path / ("img" + ext)
    save_image(path, rgb)
    assert path.read_bytes() == ref.image_bytes(ext, rgb)
    if ext == ".tga":  # the writer's top-left origin reads back unflipped
        assert np.array_equal(load_image(path), rgb)


@pytest.mark.parametrize("name", ["img.png", "img", "img.", "dir.tga/img"])
def test_save_image_rejects(native_lib, tmp_path, name):
    rgb = np.zeros((2, 2, 3), np.uint8)
    with pytest.raises(SharpRayError):
        save_image(tmp_path / name, rgb)


def test_line_box_corners():
    ov = Overlay()
    ov.add_line_box(AABox((-1.0, 0.0, 2.0), (3.0, 1.0, 4.0)), (1, 0, 0))
    assert len(ov.lines) == 12
    pts = {p for line in ov.lines for p in line[:2]}
    assert pts == {(x, y, z) for x in (-1.0, 3.0) for y in (0.0, 1.0) for z in (2.0, 4.0)}
    # corner i has +x when bit 0 is set, +y for bit 1, +z for bit 2 (Box.Corners math.cs:1086-1096)
    assert ov.lines[0][:2] == ((-1.0, 0.0, 2.0), (3.0, 0.0, 2.0))
    assert ov.lines[8][:2] == ((-1.0, 0.0, 2.0), (-1.0, 0.0, 4.0))


# ---- AOV images (GPU) ----------------------------------------------------------------------------

def synthetic_aovs(w, h, seed):
    rng = np.random.default_rng(seed)
    a = Aovs(w, h)
    n = w * h
    a.normals[:] = rng.uniform(-1.2, 1.2, (n, 3)).astype(np.float32)
    a.depth[:] = rng.uniform(-1.0, 40.0, n).astype(np.float32)
    a.depth[::7] = np.inf
    a.depth[3::11] = -np.inf
    a.depth[5::13] = np.nan
    a.variance[:] = rng.uniform(-0.01, 0.3, n).astype(np.float32)
    a.variance[2::9] = np.nan
    a.samples[:] = rng.integers(0, 66, n).astype(np.uint32)
    a.uv[:] = rng.uniform(-5.0, 5.0, (n, 2)).astype(np.float32)
    a.uv[4::10] = 1e30
    a.normals[1::17] = np.nan
    return a


@pytest.mark.gpu
@pytest.mark.parametrize("kind", list(AovKind))
def test_aov_image_matches_oracle(gpu_ctx, oracle_mod, kind):
    a = synthetic_aovs(37, 23, int(kind))
    for thr, lo, hi in ((0.075, 4, 64), (0.01, 1, 1), (0.5, 16, 48)):
        p = _abi.SrAovImageParams(thr, lo, hi)
        # counts the renderer can produce: 0 .. max + 1 (the sample loop's off-by-one)
        a.samples[:] = np.random.default_rng(hi).integers(0, hi + 2, a.samples.shape).astype(np.uint32)
        out = np.zeros((a.height, a.width, 3), np.uint8)
        ca = a.to_c()
        _abi.check(gpu_ctx._lib.sr_aov_image(gpu_ctx.handle, C.byref(ca), a.width, a.height, int(kind), C.byref(p),
                                             out.ctypes.data))
        want = oracle_mod.aov_image(a, int(kind), p)
        assert np.array_equal(out, want), f"{kind}: {(out != want).any(axis=2).sum()} pixels differ"


@pytest.mark.gpu
def test_aov_images_of_a_render(gpu_ctx, oracle_mod):
    from sharpray_gb300 import Renderer, synth
    d = synth.config_features(48, 32, 4)
    d.min_samples = 2
    scene = d.instantiate(gpu_ctx)
    rend = Renderer(scene, d.view, *d.render_args())
    p = _abi.SrAovImageParams(rend.params.variance_threshold, rend.params.min_samples, rend.params.max_samples)
    for kind in AovKind:
        got = aov_image(rend, kind)
        assert np.array_equal(got, oracle_mod.aov_image(rend.aovs, int(kind), p)), kind


@pytest.mark.gpu
def test_aov_image_device_entry(gpu_ctx, oracle_mod):
    torch = pytest.importorskip("torch")
    a = synthetic_aovs(19, 11, 5)
    dev = {k: torch.from_numpy(getattr(a, k).copy()).cuda() for k in ("normals", "uv", "depth", "samples", "variance")}
    da = _abi.SrAovs()
    da.normals, da.uv, da.depth = dev["normals"].data_ptr(), dev["uv"].data_ptr(), dev["depth"].data_ptr()
    da.samples, da.variance = dev["samples"].data_ptr(), dev["variance"].data_ptr()
    p = _abi.SrAovImageParams(0.075, 4, 64)
    for kind in AovKind:
        out = torch.zeros((a.height, a.width, 3), dtype=torch.uint8, device="cuda")
        from sharpray_gb300.autograd import current_stream_handle
        stream = current_stream_handle()
        _abi.check(gpu_ctx._lib.sr_aov_image_device(gpu_ctx.handle, C.byref(da), a.width, a.height, int(kind),
                                                    C.byref(p), out.data_ptr(), C.c_void_p(stream)))
        assert np.array_equal(out.cpu().numpy(), oracle_mod.aov_image(a, int(kind), p)), kind


# ---- overlay (GPU) -------------------------------------------------------------------------------

def random_font(seed=3, first=32, last=126):
    g = np.random.default_rng(seed).integers(0, 256, (last - first + 1, 8), dtype=np.uint8)
    g[0] = 0  # space
    return Font(g, first)


def overlay_case(seed, w, h):
    rng = np.random.default_rng(seed)
    cam = (0.5, 2.0, -6.0)
    view = View(Transform(cam, look_rotation(cam, (0.0, 0.5, 0.0))), np.radians(55.0), 0.1)
    ov = Overlay(random_font(seed))
    for _ in range(40):
        a = rng.uniform(-4, 4, 3)
        b = a + rng.normal(0, 2.5, 3)
        ov.add_line(a, b, rng.uniform(-0.2, 1.5, 3), depth_test=bool(rng.random() < 0.6),
                    depth_bias=float(rng.choice([0.005, 0.0, 0.2])))
    ov.add_line((0, 0, 0), (0, 0, 0), (1, 1, 1))                 # a point
    ov.add_line((-30, 0.5, 3), (30, 0.5, 3), (0, 1, 0))          # leaves the image on both sides
    ov.add_line((0, 0, -5.95), (0, 1, 2), (0, 0, 1))             # one end behind the near plane: skipped
    ov.add_line_box(AABox((-1, 0, -1), (1, 1.5, 1)), (1, 0.5, 0))
    ov.add_line_box(AABox((1, 0, 1), (2, 2, 3)), (0, 1, 1), rot=Quat.angle_axis(0.7, (0.0, 1.0, 0.0)))
    ov.add_text("hello\nworld!", (0.0, 1.0, 0.0), (1, 1, 0))
    ov.add_text("top left é~\x7f", (3, 4), (1, 0, 1))
    ov.add_text("centred\nlines\n\nx", (w // 2, h // 2), (0.5, 0.5, 1), align=Overlay.Center)
    ov.add_text("\n".join("l%d" % i for i in range(70)), (w - 20, 0), (0.2, 1, 0.2))
    ov.add_text("edge", (w - 10, h - 3), (1, 1, 1))
    ov.add_text("behind", (0.0, 0.0, -20.0), (1, 1, 1))
    ov.add_text("overlap", (4, 4), (0, 0, 0))
    img = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
    depth = rng.uniform(2.0, 12.0, (h, w)).astype(np.float32)
    depth[: h // 3] = np.inf
    return ov, view, img, depth


@pytest.mark.gpu
@pytest.mark.parametrize("seed,w,h", [(1, 96, 64), (2, 64, 96), (3, 160, 90)])
def test_overlay_matches_oracle(gpu_ctx, oracle_mod, seed, w, h):
    ov, view, img, depth = overlay_case(seed, w, h)
    lines, texts = ov._c_arrays()
    nl, nt = len(ov.lines), len(ov.texts)
    want = oracle_mod.overlay_draw(img, view.to_c(), depth, (_abi.SrOverlayLine * nl)(*lines[:nl]),
                                   (_abi.SrOverlayText * nt)(*texts[:nt]), ov.font.to_c())
    got = img.copy()
    ov.draw(gpu_ctx, got, view, depth)
    changed = (want != img).any(axis=2).sum()
    assert changed > 200, "the overlay should draw something"
    assert np.array_equal(got, want), f"{(got != want).any(axis=2).sum()} pixels differ"
    # no depth plane: every line drawn
    want_nd = oracle_mod.overlay_draw(img, view.to_c(), None, (_abi.SrOverlayLine * nl)(*lines[:nl]),
                                      (_abi.SrOverlayText * nt)(*texts[:nt]), ov.font.to_c())
    got_nd = img.copy()
    ov.draw(gpu_ctx, got_nd, view, None)
    assert np.array_equal(got_nd, want_nd)


@pytest.mark.gpu
def test_overlay_rejects_huge_lines_and_missing_font(gpu_ctx):
    view = View(Transform((0.0, 0.0, 0.0), Quat.identity()), np.radians(60.0), 0.1)
    img = np.zeros((16, 16, 3), np.uint8)
    ov = Overlay()
    ov.add_line((-1e6, 0.0, 0.1001), (1e6, 0.0, 0.1001), (1, 1, 1))  # projects ~1e10 pixels wide
    with pytest.raises(SharpRayError):
        ov.draw(gpu_ctx, img, view)
    ov = Overlay()
    ov.add_text("x", (1, 1), (1, 1, 1))
    with pytest.raises(SharpRayError):
        ov.draw(gpu_ctx, img, view)
