"""The FP64 path-replay adjoint of the oracle (oracle_adjoint), pinned on the CPU before it serves as the
reference for the GPU adjoint (tests/test_adjoint.py):

* its replay re-renders the oracle's image bit for bit (same random numbers, same paths);
* its albedo-texel gradient -- the exact derivative of the renderer's estimator at fixed random
  numbers for non-metallic and fully metallic surfaces -- matches central finite differences of the
  oracle's own image loss within 1 % (texel channels whose differences at h and 2h disagree saw a
  roulette decision flip and are not scored);
* the fog-density gradient is finite and non-zero in fog, and the roughness gradient lands only on
  the red channel.
The derivatives inside it come from dual numbers through the reference's formulas, not from the
GPU's hand-derived ones, so agreement between the two is a check of both.
"""
import copy

import numpy as np
import pytest

from sharpray_gb300 import render_params
from tests.adjoint_scenes import adjoint_scene


def oracle_loss_and_image(oracle_mod, d, target=None):
    o = oracle_mod.instantiate(d)
    a, _ = o.render(d.view.to_c(), render_params(*d.render_args()))
    img = (a.radiance + a.radiance_fog).reshape(-1).astype(np.float32)
    if target is None:
        return o, a, img
    r = img.astype(np.float64) - target.astype(np.float64)
    return float(np.dot(r, r))


@pytest.mark.parametrize("fog,metal", [(False, False), (True, False), (False, True)])
def test_fp64_adjoint_matches_oracle_finite_differences(oracle_mod, fog, metal):
    d = adjoint_scene(fog=fog, bounces=4, clamp=3.0, w=24, h=18, spp=2, metal=metal)
    o, a, img = oracle_loss_and_image(oracle_mod, d)
    target = (img * np.float32(0.6) + np.float32(0.05)).astype(np.float32)
    d_image = (2.0 * (img.astype(np.float64) - target)).astype(np.float32)
    tex = d.textures[1].texels
    ga, gr, gf, rep = o.adjoint(d.view.to_c(), render_params(*d.render_args()), d_image, a.samples, 1, tex.shape[:2])
    assert np.array_equal(rep.reshape(-1).view(np.uint32), img.view(np.uint32)), "replay must equal the render"
    assert gr is None and np.isfinite(gf)
    scale = float(np.abs(ga).max())
    assert scale > 0.0
    rng = np.random.default_rng(11)
    flat = np.argsort(-np.abs(ga).ravel())[:6].tolist() + rng.choice(ga.size, 4, replace=False).tolist()
    checked = 0
    for f in flat:
        y, x, ch = np.unravel_index(f, ga.shape)
        fds = []
        for h in (1e-3, 2e-3):
            vals = []
            for sgn in (1.0, -1.0):
                dd = copy.deepcopy(d)
                dd.textures[1].texels = tex.copy()
                dd.textures[1].texels[y, x, ch] += np.float32(sgn * h)
                vals.append(oracle_loss_and_image(oracle_mod, dd, target))
            fds.append((vals[0] - vals[1]) / (2.0 * h))
        if abs(fds[0] - fds[1]) > 0.02 * max(abs(fds[0]), 1e-3 * scale):
            continue  # a roulette decision flipped inside the step
        checked += 1
        assert abs(ga[y, x, ch] - fds[0]) <= 0.01 * abs(fds[0]) + 1e-4 * scale, (y, x, ch, ga[y, x, ch], fds)
    assert checked >= 6, f"only {checked} texel channels had stable differences"


def test_fp64_adjoint_all_parameters(oracle_mod):
    d = adjoint_scene(fog=True, bounces=4, clamp=3.0, w=20, h=16, spp=2)
    # the blob's material reads the bilinear texture as its roughness too
    d.objects[1].material["roughness_texture"] = 1
    o, a, img = oracle_loss_and_image(oracle_mod, d)
    d_image = (2.0 * (img - 0.5 * img - 0.02)).astype(np.float32)
    shape = d.textures[1].texels.shape[:2]
    ga, gr, gf, _ = o.adjoint(d.view.to_c(), render_params(*d.render_args()), d_image, a.samples, 1, shape, 1, shape)
    assert np.abs(ga).max() > 0 and np.abs(gr[..., 0]).max() > 0
    assert np.all(gr[..., 1:] == 0.0), "the roughness lookup reads the red channel only"
    assert np.isfinite(gf) and gf != 0.0
