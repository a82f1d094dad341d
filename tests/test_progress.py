"""sr_render_progress (Renderer.Tick renderer.cs:98-105, non-blocking): (finished pixels, pixels) of
the last render launch, polled while an asynchronous render runs."""
import ctypes as C
import time

import pytest

from sharpray_gb300 import Context, _abi, render_params, synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [_abi.SR_RENDER_WAVEFRONT_GRAPH, _abi.SR_RENDER_WAVEFRONT, _abi.SR_RENDER_MEGAKERNEL])
def test_progress_during_async_render(mode):
    torch = pytest.importorskip("torch")
    from sharpray_gb300.autograd import current_stream_handle, device_aovs
    ctx = Context(0)
    d = synth.config_c2(256, 144, 16, rings=200, rock_rings=30, env=(256, 128))
    d.min_samples = 2  # adaptive: pixels finish at different bounces
    sc = d.instantiate(ctx)
    sc.build()
    sc.set_render_mode(mode)
    assert sc.progress() == (0, 0)  # nothing launched yet
    _bufs, aovs = device_aovs(d.width, d.height)
    v, p = d.view.to_c(), render_params(*d.render_args())
    torch.cuda.synchronize()
    _abi.check(ctx._lib.sr_render_device(sc.handle, C.byref(v), C.byref(p), C.byref(aovs),
                                         C.c_void_p(current_stream_handle())))
    seen = []
    t0 = time.time()
    while True:
        done, total = sc.progress()
        assert total == d.width * d.height
        seen.append(done)
        if done == total or time.time() - t0 > 60:
            break
    assert seen[-1] == total, seen[-10:]
    assert all(a <= b for a, b in zip(seen, seen[1:])), "progress must not go backwards"
    torch.cuda.synchronize()
    assert sc.progress() == (total, total)
    # the blocking entry point leaves the progress finished
    from sharpray_gb300.api import Aovs
    host = Aovs(d.width, d.height)
    _abi.check(ctx._lib.sr_render(sc.handle, C.byref(v), C.byref(p), C.byref(host.to_c())))
    assert sc.progress() == (total, total)


def test_progress_of_batched_renders():
    """Each scene of an sr_render_batch launch reports its own progress, finished after the graph."""
    torch = pytest.importorskip("torch")
    from sharpray_gb300 import render_batch
    from sharpray_gb300.autograd import current_stream_handle, device_aovs
    ctx = Context(0)
    descs = [synth.config_c1(40, 24, 4), synth.config_procedural(24, 20, 3)]
    scenes, outs, keep = [], [], []
    for d in descs:
        sc = d.instantiate(ctx)
        sc.build()
        bufs, a = device_aovs(d.width, d.height)
        scenes.append(sc)
        outs.append(a)
        keep.append(bufs)
    render_batch(scenes, [d.view for d in descs], [render_params(*d.render_args()) for d in descs], outs,
                 stream=current_stream_handle())
    torch.cuda.synchronize()
    for sc, d in zip(scenes, descs):
        assert sc.progress() == (d.width * d.height, d.width * d.height)
