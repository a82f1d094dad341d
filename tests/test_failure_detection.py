"""Failure detection without a GPU fault: the loop caps of SrTuning.

A render whose bounce loop, or a trace whose traversal, runs past its cap ends early.  The kernel
sets the device error word (2 = loop cap) and returns; the call returns SR_ERR_DEVICE with a
message naming the loop cap; and the context stays usable, so the next render with the default
caps gives the same image as before.  The caps are lowered here far below what the scene needs,
so that they run out on purpose; nothing traps, faults or waits without a bound.  (The reference
has no such guard: Renderer.Tick waits without a timeout, renderer.cs:98-105.)
"""
import numpy as np
import pytest

from sharpray_gb300 import Renderer, SharpRayError, _abi, synth
from tests.golden.make_golden import seeded_rays

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene(gpu_ctx):
    d = synth.config_c1(32, 24, 4)
    g = d.instantiate(gpu_ctx)
    g.build()
    return d, g


def render(d, g):
    return Renderer(g, d.view, *d.render_args())


@pytest.mark.parametrize("mode", [_abi.SR_RENDER_WAVEFRONT_GRAPH, _abi.SR_RENDER_WAVEFRONT])
def test_bounce_loop_cap_reports_and_recovers(scene, mode):
    d, g = scene
    g.set_render_mode(mode)
    try:
        before = render(d, g)
        g.set_tuning(max_bounce_iterations=2)  # 4 spp x 5 segments need ~25 bounces
        with pytest.raises(SharpRayError) as e:
            render(d, g)
        assert e.value.code == _abi.SR_ERR_DEVICE
        assert "loop cap" in str(e.value)
        g.set_tuning()
        after = render(d, g)
    finally:
        g.set_tuning()
        g.set_render_mode(_abi.SR_RENDER_AUTO)
    for plane in ("radiance", "radiance_fog", "samples", "depth"):
        assert np.array_equal(getattr(before, plane).view(np.uint32), getattr(after, plane).view(np.uint32)), plane


def test_traversal_cap_in_trace_and_render(scene, oracle_mod):
    d, g = scene
    rays = seeded_rays(4096, seed=21)
    want = oracle_mod.instantiate(d).trace(rays)
    try:
        g.set_tuning(max_traversal_steps=3)  # fewer actions than any hit needs
        with pytest.raises(SharpRayError) as e:
            g.trace(rays)
        assert e.value.code == _abi.SR_ERR_DEVICE and "loop cap" in str(e.value)
        with pytest.raises(SharpRayError) as e:
            render(d, g)
        assert e.value.code == _abi.SR_ERR_DEVICE
        g.set_tuning()
        got = g.trace(rays)
    finally:
        g.set_tuning()
    assert np.array_equal(got["object"], want["object"]) and np.array_equal(got["triangle"], want["triangle"])
