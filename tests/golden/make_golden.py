"""Generates the committed golden fixtures of the oracle and the host path.

Run from the repository root:  python tests/golden/make_golden.py

* rng.json        first 16 NextUInt / NextFloat values of Rng(x, y) (math.cs:1665-1743) for three
                  seeds, computed here by an independent pure-Python restatement;
* hashes.json     sha256 of the oracle's BVH arrays (node bounds, links, item permutation) and of its
                  closest-hit results on a seeded ray set, for the 20k-triangle fBm icosphere scene;
* c1_1spp.npz     oracle AOVs of the 32x32, 1 spp icosphere scene (compared with a tolerance, since
                  they go through the C runtime's transcendentals).

The reference itself cannot be run here (no .NET runtime), so these pin the oracle against
regressions and against the independent restatements, not against the C# binary.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

MASK32 = 0xFFFFFFFF
MASK64 = 0xFFFFFFFFFFFFFFFF


def splitmix64(state: int):
    state = (state + 0x9E3779B97F4A7C15) & MASK64
    r = state
    r = ((r ^ (r >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    r = ((r ^ (r >> 27)) * 0x94D049BB133111EB) & MASK64
    return state, r ^ (r >> 31)


def rng_reference_python(seed_a: int, seed_b: int, n: int):
    """Pure-Python Rng: splitmix64-seeded xorshift with Weyl counter, NextFloat = u * (1/(2^32+512))."""
    st = ((seed_a << 32) | seed_b) & MASK64
    st, v1 = splitmix64(st)
    st, v2 = splitmix64(st)
    s = [v1 & MASK32, v1 >> 32, v2 & MASK32, v2 >> 32, 0]
    out = []
    for _ in range(n):
        t, x0 = s[3], s[0]
        s[3], s[2], s[1] = s[2], s[1], x0
        t ^= t >> 2
        t ^= (t << 1) & MASK32
        t ^= x0 ^ ((x0 << 4) & MASK32)
        s[0] = t
        s[4] = (s[4] + 362437) & MASK32
        out.append((t + s[4]) & MASK32)
    u = np.array(out, np.uint32)
    to_float = np.float32(1.0) / (np.float32(4294967296.0) + np.float32(512.0))
    f = (u.astype(np.float32) * to_float).astype(np.float32)
    return u, f


RNG_SEEDS = [(0, 0), (1, 2), (1919, 1079)]


def sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def seeded_rays(n: int, seed: int) -> np.ndarray:
    """Rays from points around the unit sphere toward jittered points near the origin."""
    rng = np.random.default_rng(seed)
    o = rng.normal(size=(n, 3))
    o = o / np.linalg.norm(o, axis=1, keepdims=True) * rng.uniform(1.5, 4.0, size=(n, 1))
    tgt = rng.uniform(-1.0, 1.0, size=(n, 3)) * 0.8
    d = tgt - o
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([o, d], axis=1).astype(np.float32)
    # renormalise in float32 so every direction is a unit vector at float precision
    dd = rays[:, 3:].astype(np.float64)
    rays[:, 3:] = (dd / np.linalg.norm(dd, axis=1, keepdims=True)).astype(np.float32)
    return rays


def main():
    from oracle import oracle as O
    from sharpray_gb300 import synth
    O.build()
    rng_fix = {}
    for a, b in RNG_SEEDS:
        u, f = rng_reference_python(a, b, 16)
        rng_fix[f"{a},{b}"] = {"uint": [int(x) for x in u], "float_bits": [int(x) for x in f.view(np.uint32)]}
    (HERE / "rng.json").write_text(json.dumps(rng_fix, indent=1) + "\n")

    d = synth.config_c1(32, 32, 1)
    scene = O.instantiate(d)
    mesh_bvh = scene.mesh_bvh(0)
    tlas = scene.bvh()
    rays = seeded_rays(4096, seed=7)
    hits = scene.trace(rays)
    hashes = {
        "c1_sphere_bvh": sha(*mesh_bvh),
        "c1_sphere_bvh_nodes": int(mesh_bvh[0].shape[0]),
        "c1_scene_bvh": sha(*tlas),
        "c1_trace_4096_seed7": sha(hits["object"], hits["triangle"], hits["dist"], hits["uv"]),
        "c1_trace_hits": int((hits["object"] >= 0).sum()),
    }
    (HERE / "hashes.json").write_text(json.dumps(hashes, indent=1) + "\n")

    aovs, _ = scene.render(d.view.to_c(), __import__("sharpray_gb300").render_params(*d.render_args()))
    np.savez_compressed(HERE / "c1_1spp.npz", radiance=aovs.radiance, radiance_fog=aovs.radiance_fog,
                        normals=aovs.normals, uv=aovs.uv, depth=aovs.depth, samples=aovs.samples,
                        variance=aovs.variance)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
