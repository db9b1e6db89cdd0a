"""The FP64 host reference of the adjoint checks itself (CPU only): its
analytic gradient must equal FP64 central finite differences of its forward,
and its forward must reproduce the float pipeline's vertices closely."""
import numpy as np

from nii2mesh_gb300 import synth
from oracle.adjoint_ref import Problem


def test_host_gradient_matches_finite_differences(oracle):
    img = synth.spheres(n=32, count=3, rmin=5, rmax=8, cmin=10, cmax=22, noise=2.0, seed=31)
    pb = Problem(oracle, img, 50.0, 4, center=(15.5, 15.5, 15.5), radius=9.0)
    mesh = oracle.meshify(img, 50.0, 0, True, False, False)
    assert np.abs(pb.positions(img) - mesh[1]).max() < 1e-4      # float pipeline vs exact float64
    g = pb.gradient(img)
    rng = np.random.default_rng(0)
    cand = np.argwhere(np.abs(g) > 1e-3 * np.abs(g).max())
    vox = cand[rng.choice(len(cand), 24, replace=False)]
    fd = pb.central_difference(img, vox, 1e-2)
    an = g[tuple(vox.T)]
    rel = np.abs(an - fd) / (np.abs(fd) + 1e-3 * np.abs(g).max())
    assert rel.max() < 1e-5, rel.max()
