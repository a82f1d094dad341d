"""Batched rendering (sr_render_batch): several scenes of one context in one graph launch, each
scene's AOVs bit-identical to its own sr_render_device render; the cached graph is reused for an
identical batch and rebuilt for a different one; invalid batches are refused."""
import ctypes as C

import numpy as np
import pytest

from sharpray_gb300 import Context, SharpRayError, _abi, render_batch, render_params, synth
from sharpray_gb300.autograd import current_stream_handle

pytestmark = pytest.mark.gpu

PLANES = (("radiance", 3, "float32"), ("radiance_fog", 3, "float32"), ("normals", 3, "float32"), ("uv", 2, "float32"),
          ("depth", 1, "float32"), ("samples", 1, "int32"), ("variance", 1, "float32"))


def device_aovs(torch, n):
    bufs = {k: torch.zeros(n * c, dtype=getattr(torch, t), device="cuda") for k, c, t in PLANES}
    a = _abi.SrAovs(*[bufs[k].data_ptr() for k, _, _ in PLANES])
    return bufs, a


def host(bufs):
    return {k: v.cpu().numpy().copy() for k, v in bufs.items()}


def same(a, b):
    for k in a:
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k


@pytest.fixture(scope="module")
def batch_scenes():
    torch = pytest.importorskip("torch")
    ctx = Context(0)
    descs = [synth.config_c1(40, 32, 4), synth.config_features(36, 28, 3), synth.config_procedural(24, 20, 5),
             synth.config_c2(48, 27, 2, rings=60, rock_rings=20, env=(128, 64))]
    descs[1].min_samples = 1  # adaptive stop in one of them
    scenes = []
    for d in descs:
        s = d.instantiate(ctx)
        s.build()
        scenes.append(s)
    return torch, ctx, descs, scenes


def render_single(torch, ctx, d, s):
    bufs, a = device_aovs(torch, d.width * d.height)
    v, p = d.view.to_c(), render_params(*d.render_args())
    _abi.check(ctx._lib.sr_render_device(s.handle, C.byref(v), C.byref(p), C.byref(a), None))
    torch.cuda.synchronize()  # the device, so also the context's own stream
    return bufs


def test_batch_matches_single_renders(batch_scenes):
    torch, ctx, descs, scenes = batch_scenes
    stream = current_stream_handle()
    singles = []
    for d, s in zip(descs, scenes):
        bufs, a = device_aovs(torch, d.width * d.height)
        v, p = d.view.to_c(), render_params(*d.render_args())
        _abi.check(ctx._lib.sr_render_device(s.handle, C.byref(v), C.byref(p), C.byref(a), C.c_void_p(stream)))
        torch.cuda.synchronize()
        singles.append(host(bufs))
    outs = [device_aovs(torch, d.width * d.height) for d in descs]
    params = [render_params(*d.render_args()) for d in descs]
    for _ in range(2):  # the second launch reuses the cached graph
        for bufs, _a in outs:
            for t in bufs.values():
                t.zero_()
        render_batch(scenes, [d.view for d in descs], params, [a for _b, a in outs], stream=stream)
        torch.cuda.synchronize()
        for (bufs, _a), ref in zip(outs, singles):
            same(host(bufs), ref)
    assert int(singles[1]["samples"].min()) < descs[1].spp  # the adaptive scene did stop early


def test_batch_subset_and_order(batch_scenes):
    """A different batch (other scenes, other order) rebuilds the graph and still matches."""
    torch, ctx, descs, scenes = batch_scenes
    stream = current_stream_handle()
    order = [3, 0]
    outs = [device_aovs(torch, descs[i].width * descs[i].height) for i in order]
    render_batch([scenes[i] for i in order], [descs[i].view for i in order],
                 [render_params(*descs[i].render_args()) for i in order], [a for _b, a in outs], stream=stream)
    torch.cuda.synchronize()
    for i, (bufs, _a) in zip(order, outs):
        ref = render_single(torch, ctx, descs[i], scenes[i])
        same(host(bufs), host(ref))


def test_batch_rejects_duplicates_and_missing_planes(batch_scenes):
    torch, ctx, descs, scenes = batch_scenes
    _b, a = device_aovs(torch, descs[0].width * descs[0].height)
    p = render_params(*descs[0].render_args())
    with pytest.raises(SharpRayError):
        render_batch([scenes[0], scenes[0]], [descs[0].view] * 2, [p, p], [a, a])
    bad = _abi.SrAovs(a.radiance, a.radiance_fog, a.normals, a.uv, a.depth, a.samples, None)
    with pytest.raises(SharpRayError):
        render_batch([scenes[0]], [descs[0].view], [p], [bad])
    other = synth.config_c1(16, 16, 1).instantiate(Context(0))
    other.build()
    with pytest.raises(SharpRayError):
        render_batch([scenes[0], other], [descs[0].view] * 2, [p, p], [a, a])


def test_tuning_leaves_results_unchanged(batch_scenes):
    """Launch geometry (set by hand or by the autotuner) changes timing only, never the AOVs."""
    torch, ctx, descs, scenes = batch_scenes
    d, s = descs[3], scenes[3]
    ref = host(render_single(torch, ctx, d, s))
    for tune in ((3, 4, 2, 8), (1, 1, 1, 64), (0, 0, 0, 0)):
        s.set_tuning(*tune)
        same(host(render_single(torch, ctx, d, s)), ref)
    for threads in (64, 256):  # the traversal kernel's block size
        for per_sm in (0, 2):
            s.set_tuning(trace_blocks_per_sm=per_sm, trace_block_threads=threads)
            same(host(render_single(torch, ctx, d, s)), ref)
    chosen = s.autotune(d.view, render_params(*d.render_args()), trial_spp=2)
    assert chosen["ms"] > 0 and chosen["default_ms"] > 0 and chosen["ms"] <= chosen["default_ms"]
    assert chosen["tail_divisor"] in (8, 16, 32) and chosen["trace_block_threads"] in (64, 128, 256)
    same(host(render_single(torch, ctx, d, s)), ref)
    s.set_tuning()


@pytest.mark.parametrize("index", [1, 3])
def test_fewer_slots_than_pixels_leave_results_unchanged(batch_scenes, index):
    """Slot capacity below the pixel count (slots claim the pixels left over as theirs finish, each
    with the pixel's own random-number stream) gives the same AOVs, in every render mode, with the
    reference's stream and with another one; the adaptive stop of the features scene included."""
    torch, ctx, descs, scenes = batch_scenes
    d, s = descs[index], scenes[index]
    n = d.width * d.height
    try:
        for seed in (0, 7):
            s.set_seed(seed)
            s.set_tuning()
            ref = host(render_single(torch, ctx, d, s))
            for slots in (n // 3, 32, 45):  # a third (rounded up to 32), one warp, a non-multiple of 32
                for mode in (_abi.SR_RENDER_AUTO, _abi.SR_RENDER_WAVEFRONT):
                    s.set_render_mode(mode)
                    s.set_tuning(max_slots=slots)
                    same(host(render_single(torch, ctx, d, s)), ref)
            s.set_render_mode(_abi.SR_RENDER_AUTO)
    finally:
        s.set_seed(0)
        s.set_tuning()
        s.set_render_mode(_abi.SR_RENDER_AUTO)
