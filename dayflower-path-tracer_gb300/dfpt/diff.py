"""Differentiable rendering over libdfpt.so's dfpt_diff_* pair (path-replay backpropagation).

DiffRenderer wraps a RendererKernel: forward() renders `spp` samples per pixel with per-primitive
albedo multipliers, added emission and Phong exponents and a sky from (turbidity, sun direction);
backward() takes dLoss/dImage and returns the gradients, replaying the forward's paths from their
RNG keys. RenderFunction exposes the pair to torch.autograd. A backward always refers to the most
recent forward of the same renderer.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, ptr


class DiffRenderer:
    def __init__(self, kernel):
        self.kernel = kernel
        self._lib = _lib.load()
        self.primitives = int(kernel.compiled.primitives.size // 3)
        self._keep = None

    def forward(self, albedo=None, emission=None, phong_exponent=None, turbidity: float = 2.0,
                sun_direction=(0.0, 0.70710677, 0.70710677), spp: int = 16) -> np.ndarray:
        """Returns the film average, shape (height, width, 3), float32."""
        n = self.primitives
        arrays = []

        def arr(x, size):
            if x is None:
                return None
            a = np.ascontiguousarray(np.asarray(x, np.float32).reshape(-1))
            if a.size != size:
                raise ValueError(f"expected {size} values, got {a.size}")
            arrays.append(a)
            return ptr(a, C.c_float)

        p = _lib.DiffParams()
        p.albedo = arr(albedo, 3 * n)
        p.emission = arr(emission, 3 * n)
        p.phong_exponent = arr(phong_exponent, n)
        p.turbidity = float(turbidity)
        for i in range(3):
            p.sun_direction[i] = float(sun_direction[i])
        self._keep = arrays
        k = self.kernel
        img = np.empty(k.resolution_x * k.resolution_y * 3, np.float32)
        check(self._lib.dfpt_diff_forward(k._need(), C.byref(p), int(spp), ptr(img, C.c_float)))
        return img.reshape(k.resolution_y, k.resolution_x, 3)

    def backward(self, dloss_dimage) -> dict:
        k = self.kernel
        g = np.ascontiguousarray(np.asarray(dloss_dimage, np.float32).reshape(-1))
        if g.size != k.resolution_x * k.resolution_y * 3:
            raise ValueError("dloss_dimage must hold 3 values per pixel")
        n = self.primitives
        ga = np.zeros(3 * n, np.float64)
        ge = np.zeros(3 * n, np.float64)
        gx = np.zeros(max(n, 1), np.float64)
        gs = np.zeros(4, np.float64)
        check(self._lib.dfpt_diff_backward(k._need(), ptr(g, C.c_float), ptr(ga, C.c_double), ptr(ge, C.c_double),
                                           ptr(gx, C.c_double), ptr(gs, C.c_double)))
        return {"albedo": ga.reshape(n, 3), "emission": ge.reshape(n, 3), "phong_exponent": gx[:n],
                "turbidity": float(gs[0]), "sun_direction": gs[1:4].copy()}

    def end(self) -> None:
        check(self._lib.dfpt_diff_end(self.kernel._need()))


def render_function():
    """torch.autograd.Function over a DiffRenderer: apply(renderer, spp, albedo (P,3), emission (P,3),
    phong_exponent (P,), turbidity (), sun_direction (3,)) -> image (H, W, 3) on albedo's device."""
    import torch

    class RenderFunction(torch.autograd.Function):
        @staticmethod
        def forward(ctx, renderer, spp, albedo, emission, phong_exponent, turbidity, sun_direction):
            img = renderer.forward(albedo.detach().cpu().numpy(), emission.detach().cpu().numpy(),
                                   phong_exponent.detach().cpu().numpy(), float(turbidity.detach().cpu()),
                                   sun_direction.detach().cpu().numpy().tolist(), spp)
            ctx.renderer = renderer
            ctx.meta = [(t.device, t.dtype) for t in (albedo, emission, phong_exponent, turbidity, sun_direction)]
            return torch.from_numpy(img).to(albedo.device)

        @staticmethod
        def backward(ctx, grad_image):
            g = ctx.renderer.backward(grad_image.detach().float().cpu().numpy())
            vals = [g["albedo"], g["emission"], g["phong_exponent"], np.asarray(g["turbidity"]), g["sun_direction"]]
            out = [torch.as_tensor(v).to(device=d, dtype=t) for v, (d, t) in zip(vals, ctx.meta)]
            return (None, None, *out)

    return RenderFunction
