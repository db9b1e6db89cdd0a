"""The hand-written adjoint (n2m_meshify_backward) through the torch.autograd
harness: dL/dvoxel against FP64 central finite differences of the exact
forward (relative 1e-3, the spec bar) and against the FP64 host
gradient of the same fixed-topology map."""
import numpy as np
import pytest

from nii2mesh_gb300 import synth
from oracle.adjoint_ref import Problem

pytestmark = pytest.mark.gpu

REL = 1e-3


def gpu_grad(img, iso, iters, center, radius):
    import torch
    from nii2mesh_gb300 import Context
    from nii2mesh_gb300.autograd import MeshifyFunction, sphere_loss
    ctx = Context(0)
    vol = torch.from_numpy(img).cuda().requires_grad_(True)
    pts, tris = MeshifyFunction.apply(vol, ctx, iso, iters)
    loss = sphere_loss(pts, center, radius)
    loss.backward()
    return pts.detach().cpu().numpy(), vol.grad.cpu().numpy(), float(loss)


@pytest.mark.parametrize("iters", [0, 10])
def test_adjoint_vs_finite_differences(oracle, iters):
    img = synth.spheres(n=48, count=4, rmin=6, rmax=10, cmin=14, cmax=34, noise=2.0, seed=12)
    center, radius = (23.5, 23.5, 23.5), 15.0
    pb = Problem(oracle, img, 50.0, iters, center, radius)
    pts, g, loss = gpu_grad(img, 50.0, iters, center, radius)
    assert np.abs(pts - pb.smoothed_positions(img)).max() < 1e-4
    gh = pb.gradient(img)
    assert np.linalg.norm(g - gh) / np.linalg.norm(gh) < REL
    rng = np.random.default_rng(iters)
    cand = np.argwhere(np.abs(gh) > 1e-3 * np.abs(gh).max())
    vox = cand[rng.choice(len(cand), 64, replace=False)]
    fd = pb.central_difference(img, vox, 1e-2)
    rel = np.abs(g[tuple(vox.T)] - fd) / (np.abs(fd) + 1e-3 * np.abs(gh).max())
    assert rel.max() < REL, rel.max()


def test_adjoint_128_workload(oracle):
    """the differentiation workload: 128^3, spheres r 12-28, 10 HC iterations,
    loss to a sphere of radius 40 at the volume centre; the gradient against
    the FP64 host gradient, and against FP64 central finite differences at 64
    random near-surface voxels (voxels whose gradient is at least 1 % of the
    largest: only voxels within the stencil's reach of the surface have one)"""
    img = synth.sphere128()
    center, radius = (63.5, 63.5, 63.5), 40.0
    pb = Problem(oracle, img, 50.0, 10, center, radius)
    pts, g, loss = gpu_grad(img, 50.0, 10, center, radius)
    gh = pb.gradient(img)
    assert np.linalg.norm(g - gh) / np.linalg.norm(gh) < REL
    rng = np.random.default_rng(5)
    cand = np.argwhere(np.abs(gh) > 1e-2 * np.abs(gh).max())
    vox = cand[rng.choice(len(cand), 64, replace=False)]
    fd = pb.central_difference(img, vox, 1e-2)
    rel = np.abs(g[tuple(vox.T)] - fd) / (np.abs(fd) + 1e-3 * np.abs(gh).max())
    assert rel.max() < REL, rel.max()


def test_backward_rejects_clustered_forward(gpu):
    import ctypes as C
    import torch
    ctx = gpu.Context(0)
    img = synth.spheres(n=32, count=2, rmin=5, rmax=8, cmin=10, cmax=22, seed=3)
    d = torch.from_numpy(img).cuda()
    ctx.meshify_device(d.data_ptr(), (32, 32, 32), 50.0, 0, True, True, False)
    g = torch.zeros((10, 3), device="cuda")
    out = torch.zeros_like(d)
    assert gpu.lib().n2m_meshify_backward(ctx.h, C.c_void_p(g.data_ptr()), C.c_void_p(out.data_ptr())) == 4
