"""torch.autograd wrapper of the meshify forward/adjoint — test and bench harness.

The product is the C ABI (n2m_meshify_device + n2m_meshify_backward); this
module only lets PyTorch drive it: the forward meshes a CUDA volume and returns
the vertices as a float64 tensor (plus the triangles), the backward hands
dL/dvertex to the library's adjoint kernels and returns dL/dvoxel.

The adjoint uses the state the forward left in the n2m context, so a backward
must follow its own forward on that context with no other meshify call in
between (the usual forward-then-backward step of a fitting loop).
"""
import ctypes as C

import torch

from . import MC33, Context, _lib


class _DeviceView:
    """Zero-copy view of library-owned device memory for torch.as_tensor."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (ptr, False), "version": 2,
                                         "strides": None}


def _device_mesh(ctx, vol, iso, post_smooth):
    vol = vol.contiguous()
    nz, ny, nx = vol.shape
    torch.cuda.current_stream(vol.device).synchronize()
    tp, pp, nt, np_, rep = ctx.meshify_device(vol.data_ptr(), (nx, ny, nz), iso, MC33, pre_smooth=True,
                                              only_largest=False, fill_bubbles=False, post_smooth=post_smooth)
    pts = torch.as_tensor(_DeviceView(pp, (np_, 3), "<f8"), device=vol.device).clone()
    tris = torch.as_tensor(_DeviceView(tp, (nt, 3), "<i4"), device=vol.device).clone()
    return pts, tris, rep


class MeshifyFunction(torch.autograd.Function):
    """vertices, triangles = MeshifyFunction.apply(volume, context, iso, post_smooth)"""

    @staticmethod
    def forward(fctx, vol, ctx, iso, post_smooth):
        pts, tris, rep = _device_mesh(ctx, vol, float(iso), int(post_smooth))
        fctx.n2m = ctx
        fctx.vol_shape = vol.shape
        fctx.report = rep
        fctx.mark_non_differentiable(tris)
        return pts, tris

    @staticmethod
    def backward(fctx, g_pts, g_tris):
        g = g_pts.to(torch.float32).contiguous()
        out = torch.empty(fctx.vol_shape, dtype=torch.float32, device=g.device)
        torch.cuda.current_stream(g.device).synchronize()
        L = _lib.load()
        _lib.check(L.n2m_meshify_backward(fctx.n2m.h, C.c_void_p(g.data_ptr()), C.c_void_p(out.data_ptr())),
                   "n2m_meshify_backward")
        return out, None, None, None


def sphere_loss(pts, center, radius):
    """sum over vertices of (|v - c| - R)^2"""
    c = torch.as_tensor(center, dtype=pts.dtype, device=pts.device)
    return ((pts - c).norm(dim=1) - radius).pow(2).sum()


__all__ = ["MeshifyFunction", "sphere_loss", "Context"]
