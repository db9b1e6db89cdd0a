"""NIfTI voxel cast on the device (load_nii, src/nii2mesh.c:160-175) and
meshing straight from raw voxels, against the reference's load_nii output
(tests/golden/nifti.npz) and the float path, bit for bit."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def test_cast_matches_reference_load_nii(gpu):
    import torch
    g = np.load(GOLD / "nifti.npz")
    ctx = gpu.Context(0)
    for k in range(sum(1 for n in g.files if n.startswith("raw"))):
        raw, meta, want = g[f"raw{k}"], g[f"meta{k}"], g[f"out{k}"]
        d_raw = torch.from_numpy(np.ascontiguousarray(raw).view(np.uint8).copy()).cuda()
        d_out = torch.empty(raw.size, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        ctx.cast_voxels_device(d_raw.data_ptr(), raw.dtype, meta[1], meta[2], raw.size, d_out.data_ptr())
        got = d_out.cpu().numpy().reshape(raw.shape)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), k


@pytest.mark.parametrize("dtype,slope,inter", [(np.uint8, 0.0, 0.0), (np.int16, 0.5, -20.0), (np.uint16, 1.0, 3.0),
                                               (np.float32, 2.0, 1.0)])
def test_meshify_typed_equals_float_path(gpu, oracle, dtype, slope, inter):
    from nii2mesh_gb300 import synth
    from oracle.oracle import cast_voxels, canonical
    vol = synth.brain()[::2, ::2, ::2]
    raw = vol.astype(dtype) if dtype != np.int16 else (vol.astype(np.int16) - 60)
    f = cast_voxels(raw, slope, inter)
    iso = float(np.float32(oracle.set_threshold(f, 2)))
    ctx = gpu.Context(0)
    t1, p1, _ = ctx.meshify_typed(raw, slope, inter, iso, pre_smooth=True, only_largest=True, fill_bubbles=True)
    t2, p2, _ = ctx.meshify(f, iso, pre_smooth=True, only_largest=True, fill_bubbles=True)
    assert np.array_equal(t1, t2) and np.array_equal(p1.view(np.uint64), p2.view(np.uint64))
    ot, op = oracle.meshify(f, iso, 0, True, True, True)
    a, b = canonical(t1, p1), canonical(ot, op)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_meshify_typed_rejects_unknown_datatype(gpu):
    import ctypes as C
    L = gpu.lib()
    ctx = gpu.Context(0)
    o = gpu.Options(0, 0.5, True, False, False, 0, False)
    tp, pp, nt, np_ = C.c_void_p(), C.c_void_p(), C.c_int(), C.c_int()
    buf = np.zeros(8 * 8 * 8, np.float64)
    s = L.n2m_meshify_typed(ctx.h, buf.ctypes.data, 64, 1.0, 0.0, (C.c_int * 3)(8, 8, 8), C.byref(o), C.byref(tp),
                            C.byref(pp), C.byref(nt), C.byref(np_), None)
    assert s != 0
