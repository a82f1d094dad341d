"""sharpray_gb300 — SharpRay's render hot path (path loop + denoiser) as CUDA kernels for GB300 (sm_103a).

The native library ``libsharpray_gb300.so`` (C ABI in ``include/sharpray.h``) does all render work;
this package is the Python host side above it, mirroring the reference's Scene / Renderer /
Compositor classes (see :mod:`sharpray_gb300.api`).
"""
from .api import (AABox, AovKind, Aovs, Compositor, Context, Fog, Font, Material, Mesh, Object, Overlay, Quat,
                  Renderer, Scene, SharpRayError, SkyProcedural, SkyTexture, Sphere, StateError, Texture,
                  TextureFilter, Tonemapper, Transform, View, adjoint_albedo, adjoint_texture, aov_image, load_image, mesh_triangles,
                  render_batch, render_compose, render_params, save_image)

__version__ = "0.1.0"
