"""The allocation-free HC smoothing entry point (n2m_smooth_hc_noalloc).

Some callers cannot allocate device memory (code running inside another
framework's captured or allocation-controlled region, or programs whose device
memory all comes from their own pool).  For them the library offers HC
smoothing with its scratch in a fixed device array.  This file checks, through
the C ABI, that it gives the same vertices as the regular entry point
(n2m_smooth_hc_device) within the smoothing tolerance, on two calls in a row
(the second call must not see the first call's scratch), and that meshes
beyond the fixed limit are rejected.  It is collected last so that a failing
run has already run every other test; it also passes alone.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HC_TOL = 1e-4   # voxels, same bar as the other smoothing tests


def _mesh(gpu, seed):
    from nii2mesh_gb300 import synth
    vol = synth.spheres(n=48, count=6, rmin=5, rmax=11, cmin=10, cmax=38, seed=seed)
    t, p = gpu.meshify(vol, 50.0, pre_smooth=True, only_largest=False, fill_bubbles=False)
    keep = np.ones(len(t), bool)
    keep[::9] = False            # open the surface so border vertices exist
    return t[keep].copy(), p


def test_noalloc_matches_regular_entry_point(gpu):
    import torch
    from nii2mesh_gb300 import _lib
    L = _lib.load()
    L.n2m_smooth_hc_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                        C.c_bool, C.c_void_p]
    L.n2m_smooth_hc_noalloc.restype = C.c_int
    ctx = gpu.Context(0)
    for call, (seed, iters, lock) in enumerate(((10, 5, True), (11, 3, False))):
        t, p = _mesh(gpu, seed)
        assert len(p) <= 131072 and len(t) <= 262144
        dt = torch.from_numpy(t.astype(np.int32)).cuda()
        ref = torch.from_numpy(p).cuda()
        got = ref.clone()
        torch.cuda.synchronize()
        st = L.n2m_smooth_hc_device(ctx.h, C.c_void_p(ref.data_ptr()), C.c_void_p(dt.data_ptr()), len(p), len(t),
                                    0.1, 0.5, iters, lock)
        assert st == 0, L.n2m_last_error()
        st = L.n2m_smooth_hc_noalloc(C.c_void_p(got.data_ptr()), C.c_void_p(dt.data_ptr()), len(p), len(t), 0.1, 0.5,
                                     iters, lock, C.c_void_p(0))
        assert st == 0, L.n2m_last_error()
        torch.cuda.synchronize()
        err = (got - ref).abs().max().item()
        assert err <= HC_TOL, (call, err)
        assert (got - torch.from_numpy(p).cuda()).abs().max().item() > 0   # it did smooth
    # beyond the fixed scratch: rejected with a clear error, nothing queued
    st = L.n2m_smooth_hc_noalloc(C.c_void_p(got.data_ptr()), C.c_void_p(dt.data_ptr()), 131073, len(t), 0.1, 0.5, 1,
                                 True, C.c_void_p(0))
    assert st == 8 and b"exceeds" in L.n2m_last_error()
    # a triangle index outside [0, nvert): the kernels skip that triangle (no
    # access out of bounds, in the scratch array or the caller's arrays), the
    # call fails with N2M_ERR_BAD_ARGS and the vertices stay as they were
    tb = t.astype(np.int32).copy()
    tb[3, 2] = len(p)
    dtb = torch.from_numpy(tb).cuda()
    before = got.clone()
    st = L.n2m_smooth_hc_noalloc(C.c_void_p(got.data_ptr()), C.c_void_p(dtb.data_ptr()), len(p), len(tb), 0.1, 0.5, 3,
                                 True, C.c_void_p(0))
    assert st == 4 and b"outside" in L.n2m_last_error()
    assert torch.equal(got, before)
    ctx.close()
