"""The C ABI library (CPU): it loads, exports every entry point include/sharpray.h declares, and
reports misuse the way the reference does (errors, not crashes).  No compute call needs a GPU here."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from sharpray_gb300 import (Context, Fog, Material, Mesh, Object, Scene, SharpRayError, SkyTexture, StateError,
                            Texture, Transform, _abi)

HEADER = Path(__file__).resolve().parent.parent / "include" / "sharpray.h"


def declared_symbols():
    return sorted(set(re.findall(r"SR_API\s+[\w\s\*]+?\b(sr_\w+)\s*\(", HEADER.read_text())))


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "sr_render" in names and "sr_compose" in names and len(names) >= 25


def test_library_exports_every_declared_symbol(native_lib):
    for name in declared_symbols():
        assert hasattr(native_lib, name), name
        assert name in _abi.PROTOTYPES, f"{name} missing from the ctypes prototypes"


def test_struct_layouts_are_packed_4_byte_fields():
    assert C.sizeof(_abi.SrTriangle) == 144
    assert C.sizeof(_abi.SrTransform) == 40
    assert C.sizeof(_abi.SrMaterial) == 56
    assert C.sizeof(_abi.SrShape) == 32
    assert C.sizeof(_abi.SrView) == 48
    assert C.sizeof(_abi.SrRenderParams) == 32
    assert C.sizeof(_abi.SrComposeParams) == 44


def test_version_and_no_error(native_lib):
    assert b"sm_103a" in native_lib.sr_version()


def _tiny_scene(ctx, with_sky=True):
    s = Scene(ctx)
    tex = Texture(ctx, np.ones((4, 8, 3), np.float32))
    if with_sky:
        s.set_sky(SkyTexture(tex))
    m = Mesh.from_corners(ctx, np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]]], np.float32))
    s.add_object(Object("tri", Transform(), Material((1, 1, 1), 1.0), m))
    return s


def test_scene_requires_sky(host_ctx):
    s = _tiny_scene(host_ctx, with_sky=False)
    with pytest.raises(StateError, match="sky is required"):
        s.build()


def test_no_mutation_after_build(host_ctx):
    s = _tiny_scene(host_ctx)
    s.build()
    with pytest.raises(StateError, match="already built"):
        s.set_fog(Fog(0.1, (1, 1, 1), 0.5, 0.2))
    with pytest.raises(StateError, match="already built"):
        s.add_object(Object("x", Transform(), Material((1, 1, 1), 1.0), s.objects[0].shape))


def test_fog_height_falloff_must_be_positive(host_ctx):
    """Height fog needs falloff > 0 (the reference divides by it); falloff 0 is the homogeneous
    extension, which needs a finite top height."""
    import math
    s = _tiny_scene(host_ctx)
    with pytest.raises(SharpRayError, match="top_height"):
        s.set_fog(Fog(0.02, (1, 1, 1), 0.6, 0.0))
    for bad in (Fog(0.02, (1, 1, 1), 0.6, -0.1), Fog(0.02, (1, 1, 1), 0.6, math.inf), Fog(0.0, (1, 1, 1), 0.6, 0.1),
                Fog(0.02, (1, 1, 1), 1.0, 0.1)):
        with pytest.raises(SharpRayError):
            s.set_fog(bad)
    s.set_fog(Fog(0.02, (1, 1, 1), 0.6, 0.0, 2.5))  # bounded homogeneous medium


def test_bad_ids_and_zero_scale(host_ctx):
    s = _tiny_scene(host_ctx)
    with pytest.raises(SharpRayError, match="Scale"):
        s.add_object(Object("z", Transform(scale=(0, 1, 1)), Material((1, 1, 1), 1.0), s.objects[0].shape))
    lib = host_ctx._lib
    out = C.c_int32()
    assert lib.sr_texture_create(host_ctx.handle, None, 1, 1, 0, 1.0, 1.0, C.byref(out)) == _abi.SR_ERR_INVALID_ARG
    assert b"NULL" in lib.sr_last_error_message()


def test_host_only_context_refuses_device_work(host_ctx):
    s = _tiny_scene(host_ctx)
    s.build()
    with pytest.raises(StateError, match="host-only"):
        s.trace(np.zeros((1, 6), np.float32))


def test_product_never_imports_the_oracle():
    pkg = Path(__file__).resolve().parent.parent / "sharpray_gb300"
    for f in list(pkg.rglob("*.py")) + list(pkg.rglob("*.cu")) + list(pkg.rglob("*.cpp")) + list(pkg.rglob("*.h")):
        text = f.read_text()
        assert "oracle" not in text.lower(), f"{f} references the oracle"
