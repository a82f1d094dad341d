"""sr_compose_device_static: compositing for callers that cannot allocate device memory (a service
whose device memory is committed to its own pools under a quota, or a latency-critical loop that
cannot afford the device-wide synchronisation an allocation may cause).  It keeps its scratch in a
fixed 32 MiB device array instead of allocating, so these checks compare it with the allocating
entry point, sr_compose_device, through the C ABI.

This file is collected last on purpose: it runs after every other test, and it also passes on its
own in a fresh process (`pytest tests/test_zz_no_alloc.py -m gpu`).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_aovs(torch, seed, w, h):
    """Synthetic AOVs on the device: mixed sky / surface pixels with varied normals and depths."""
    rng = np.random.default_rng(seed)
    n = w * h
    sky = rng.random(n) < 0.2
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm[sky] = 0.0
    depth = rng.uniform(1.0, 6.0, n)
    depth[sky] = np.inf
    planes = {
        "radiance": rng.gamma(1.0, 0.5, (n, 3)),
        "radiance_fog": rng.gamma(1.0, 0.05, (n, 3)),
        "normals": nrm,
        "uv": np.zeros((n, 2)),
        "depth": depth,
        "samples": np.ones(n),
        "variance": rng.uniform(0.0, 0.3, n),
    }
    return {k: torch.tensor(v.astype(np.float32).reshape(-1), device="cuda") for k, v in planes.items()}


def _sr_aovs(_abi, t):
    return _abi.SrAovs(*[t[k].data_ptr() for k in ("radiance", "radiance_fog", "normals", "uv", "depth", "samples",
                                                   "variance")])


def _compose(gpu_ctx, fn_name, aovs, w, h, comp, torch):
    from sharpray_gb300 import _abi
    out = torch.zeros(w * h * 3, dtype=torch.uint8, device="cuda")
    a, p = _sr_aovs(_abi, aovs), comp.to_c()
    fn = getattr(gpu_ctx._lib, fn_name)
    _abi.check(fn(gpu_ctx.handle, C.byref(a), w, h, C.byref(p), C.c_void_p(out.data_ptr()), None))
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(h, w, 3).astype(np.int32)


def test_static_compose_matches_allocating_entry_point_twice(gpu_ctx):
    torch = pytest.importorskip("torch")
    from sharpray_gb300 import Compositor, Tonemapper
    # Two different images in a row: the second call reuses the fixed array the first one filled.
    cases = [(960, 540, 1, Compositor()),
             (1280, 720, 2, Compositor(tonemapper=Tonemapper.Reinhard, exposure=1.2))]
    for w, h, seed, comp in cases:
        aovs = _device_aovs(torch, seed, w, h)
        want = _compose(gpu_ctx, "sr_compose_device", aovs, w, h, comp, torch)
        got = _compose(gpu_ctx, "sr_compose_device_static", aovs, w, h, comp, torch)
        diff = np.abs(got - want)
        # same tolerance as the compositor parity tests: one code value on >= 99.9 % of pixels
        assert (diff <= 1).mean() >= 0.999, (w, h, (diff <= 1).mean())
        assert diff.max() <= 3, (w, h, diff.max())


def test_static_compose_rejects_images_wider_than_its_scratch(gpu_ctx):
    torch = pytest.importorskip("torch")
    from sharpray_gb300 import Compositor, _abi
    w, h = 32768, 8  # radius 12 -> 26 rows x 32768 px x 48 B = 40.9 MB > 32 MiB
    comp = Compositor()
    aovs = _device_aovs(torch, 3, w, h)
    out = torch.zeros(w * h * 3, dtype=torch.uint8, device="cuda")
    a, p = _sr_aovs(_abi, aovs), comp.to_c()
    rc = gpu_ctx._lib.sr_compose_device_static(gpu_ctx.handle, C.byref(a), w, h, C.byref(p),
                                               C.c_void_p(out.data_ptr()), None)
    assert rc == _abi.SR_ERR_INVALID_ARG
    assert b"scratch" in gpu_ctx._lib.sr_last_error_message()
