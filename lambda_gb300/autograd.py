"""torch.autograd binding of the path-replay adjoint (lgpu_adjoint).

`render(scene_fn, camera, opts, params, albedo, scalars)` renders the mean radiance image
(H, W, 3) of the scene that `scene_fn(albedo, roughness, sigma_a, sigma_s)` builds, as a
differentiable function of

* `albedo`: the (h, w, 3) texels of the image texture that `params.texture` names, used as the
  albedo of material `params.tex_material`;
* `scalars`: (roughness of material `params.rough_material`'s first BSDF leaf, sigma_a, sigma_s of
  medium `params.medium`).

Forward: the scene is committed with the given values and rendered on the GPU by the wavefront
(per path the same estimate as the megakernel that the adjoint replays, with the film summed in a
fixed order, so repeated renders are bit-identical); the context is released before returning, so
a graph that is never differentiated holds no device memory.  Backward: the same scene is
committed again from its host-side description (the compile is deterministic) and
`lgpu_adjoint` runs with dLoss/dI = the incoming gradient, on the same seed and samples.  The gradient is that of this Monte Carlo
estimate with its samples held fixed (plus the validity score the adjoint documents), not a
finite difference.  RGB3 only, as lgpu_adjoint.
"""
from collections import namedtuple

import numpy as np
import torch

from . import Renderer

AdjointParams = namedtuple("AdjointParams", "tex_material texture rough_material medium")


class _Render(torch.autograd.Function):
    @staticmethod
    def forward(ctx, albedo, scalars, scene_fn, camera, opts, params):
        a = albedo.detach().to("cpu", torch.float32).numpy()
        r_, sa, ss = (float(x) for x in scalars.detach().cpu().tolist())
        sb = scene_fn(np.ascontiguousarray(a), r_, sa, ss)
        r = Renderer(sb)
        film = torch.zeros((opts.height, opts.width, 4), dtype=torch.float32, device="cuda")
        try:
            r.render_device(camera, opts, film.data_ptr())
            torch.cuda.synchronize()
        finally:
            r.close()
        ctx.scene, ctx.camera, ctx.opts, ctx.params = sb, camera, opts, tuple(params)
        ctx.tex_shape = tuple(albedo.shape)
        ctx.devices = (albedo.device, scalars.device)
        return film[..., :3] / film[..., 3:4]

    @staticmethod
    def backward(ctx, grad_img):
        r = Renderer(ctx.scene)
        h, w = ctx.opts.height, ctx.opts.width
        try:
            dloss = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
            dloss[..., :3] = grad_img.to(torch.float32)
            th, tw = ctx.tex_shape[0], ctx.tex_shape[1]
            gtex = torch.zeros((th, tw, 4), dtype=torch.float32, device="cuda")
            gsc = torch.zeros(3, dtype=torch.float32, device="cuda")
            r.adjoint(ctx.camera, ctx.opts, ctx.params, dloss.data_ptr(), gtex.data_ptr(), gsc.data_ptr())
            torch.cuda.synchronize()
        finally:
            r.close()
        return gtex[..., :3].to(ctx.devices[0]), gsc.to(ctx.devices[1]), None, None, None, None


def render(scene_fn, camera, opts, params, albedo, scalars):
    """Differentiable render: see the module docstring.  opts.kernel_mode is forced to the
    wavefront; opts.spectral_mode must be RGB3."""
    from . import abi
    o = abi.RenderOpts.from_buffer_copy(opts)
    o.kernel_mode = abi.KERNEL_WAVEFRONT
    return _Render.apply(albedo, scalars, scene_fn, camera, o, AdjointParams(*params))
