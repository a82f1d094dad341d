"""The renderer as a differentiable function of an albedo or roughness texture for PyTorch: forward
renders the scene with the given texels (sr_scene_update_texture_device + sr_render_device),
backward runs the path-replay adjoint (sr_adjoint_texture).  All work is issued on torch's current
CUDA stream.

    image = render_albedo(scene, view, params, texture, texels)   # texels: (h, w, 3) float32 cuda
    loss = ((image - target) ** 2).sum()
    loss.backward()                                                 # texels.grad
"""
import ctypes as C

import torch

from . import _abi
from ._abi import check
from .api import Scene, Texture, View, adjoint_texture

_PLANES = (("radiance", 3, torch.float32), ("radiance_fog", 3, torch.float32), ("normals", 3, torch.float32),
           ("uv", 2, torch.float32), ("depth", 1, torch.float32), ("samples", 1, torch.int32),
           ("variance", 1, torch.float32))


def current_stream_handle() -> int:
    """torch's current CUDA stream as a handle for the library.  torch's default stream has handle 0,
    which the library would read as "the context's own stream" (not ordered with torch's work), so it
    is passed as cudaStreamLegacy (1), the stream that handle 0 denotes in the CUDA runtime."""
    return torch.cuda.current_stream().cuda_stream or 1


def device_aovs(width: int, height: int, device=None):
    """Seven zeroed AOV planes on the device and the SrAovs of their pointers."""
    n = width * height
    bufs = {k: torch.zeros(n * c, dtype=t, device=device or "cuda") for k, c, t in _PLANES}
    return bufs, _abi.SrAovs(*[bufs[k].data_ptr() for k, _, _ in _PLANES])


class TextureRender(torch.autograd.Function):
    """I = radiance + radiance_fog (height x width x 3) as a function of the texels of one texture,
    differentiated as the albedo (SR_ADJOINT_ALBEDO) or roughness (SR_ADJOINT_ROUGHNESS: channel 0)
    lookup; the gradient holds the sampling fixed (path replay)."""

    @staticmethod
    def forward(ctx, texels: torch.Tensor, scene: Scene, view: View, params, texture: Texture, parameter: int):
        if not texels.is_cuda or texels.dtype != torch.float32:
            raise TypeError("texels must be a float32 CUDA tensor")
        texels = texels.contiguous()
        if tuple(texels.shape) != (texture.height, texture.width, 3):
            raise ValueError(f"texels must be ({texture.height}, {texture.width}, 3)")
        stream = current_stream_handle()
        scene.update_texture_device(texture, texels.data_ptr(), stream)
        bufs, aovs = device_aovs(params.width, params.height, texels.device)
        v = view.to_c()
        check(scene._lib.sr_render_device(scene.handle, C.byref(v), C.byref(params), C.byref(aovs),
                                          C.c_void_p(stream)))
        ctx.scene, ctx.view, ctx.params, ctx.texture, ctx.parameter = scene, view, params, texture, parameter
        ctx.seed = scene.get_seed()  # the replay must use the forward's random-number stream
        ctx.bufs, ctx.aovs = bufs, aovs
        ctx.save_for_backward(texels)
        return (bufs["radiance"] + bufs["radiance_fog"]).view(params.height, params.width, 3)

    @staticmethod
    def backward(ctx, grad_image: torch.Tensor):
        (texels,) = ctx.saved_tensors
        stream = current_stream_handle()
        # another forward may have replaced the scene's texels since
        ctx.scene.update_texture_device(ctx.texture, texels.data_ptr(), stream)
        g_img = grad_image.contiguous().to(torch.float32)
        grad = torch.zeros_like(texels)
        seed = ctx.scene.get_seed()
        ctx.scene.set_seed(ctx.seed)  # and its random-number stream
        try:
            adjoint_texture(ctx.scene, ctx.view, ctx.params, ctx.aovs, g_img.data_ptr(), ctx.texture,
                            grad.data_ptr(), ctx.parameter, None, stream)
        finally:
            ctx.scene.set_seed(seed)
        return grad, None, None, None, None, None


def render_texture(scene: Scene, view: View, params, texture: Texture, texels: torch.Tensor,
                   parameter: int = _abi.SR_ADJOINT_ALBEDO) -> torch.Tensor:
    """Differentiable render: see TextureRender."""
    if not scene.built:
        scene.build()
    return TextureRender.apply(texels, scene, view, params, texture, parameter)


def render_albedo(scene: Scene, view: View, params, texture: Texture, texels: torch.Tensor) -> torch.Tensor:
    """render_texture with the texture as the albedo lookup."""
    return render_texture(scene, view, params, texture, texels, _abi.SR_ADJOINT_ALBEDO)


def render_roughness(scene: Scene, view: View, params, texture: Texture, texels: torch.Tensor) -> torch.Tensor:
    """render_texture with the texture as the roughness lookup (gradient in channel 0)."""
    return render_texture(scene, view, params, texture, texels, _abi.SR_ADJOINT_ROUGHNESS)
