"""GPU results against the reference's own golden outputs (tests/golden/)
and against the oracle, through the C ABI: meshify, marchingCubes (exact
vertex/triangle order), bwlabel, laplacian_smoothHC, apply_sform."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import MC_CLASSIC_TABLE, OLDCUBES, canonical

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
G = json.loads((GOLD / "golden.json").read_text())
INPUTS = dict(np.load(GOLD / "inputs.npz"))
HC_TOL = 1e-4     # smoothed positions, voxels (spec bar)


def mesh_hash(tris, pts):
    ct, cp = canonical(tris, pts)
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(ct, np.int64).tobytes())
    h.update(np.ascontiguousarray(cp, np.float64).tobytes())
    return h.hexdigest()


def raw_hash(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("e", G["meshify"], ids=lambda e: f"{e['input']}-v{e['variant']}-"
                         f"{int(e['pre_smooth'])}{int(e['only_largest'])}{int(e['fill_bubbles'])}")
def test_meshify_golden(gpu, e):
    m = gpu.meshify(INPUTS[e["input"]], e["iso"], original_mc=1 if e["variant"] == MC_CLASSIC_TABLE else 0,
                    pre_smooth=e["pre_smooth"], only_largest=e["only_largest"], fill_bubbles=e["fill_bubbles"],
                    oldcubes=e["variant"] == OLDCUBES)
    if e.get("result", 1) is None:
        assert m is None
        return
    assert (len(m[1]), len(m[0])) == (e["nvert"], e["ntri"])
    assert mesh_hash(*m) == e["sha256"]


def test_marching_cubes_dropin_exact_order(gpu):
    """marchingCubes() returns the un-welded mesh in the reference's exact
    vertex and triangle order"""
    v = INPUTS["sphere48"]
    for e in G["marching_cubes"]:
        t, p = gpu.marching_cubes(v, e["lo"], e["hi"], 50.0, original_mc=e["original_mc"])
        assert (len(p), len(t)) == (e["nvert"], e["ntri"])
        assert raw_hash(t.astype(np.int32), p.astype(np.float64)) == e["sha256"]


def test_bwlabel_golden(gpu):
    for e in G["bwlabel"]:
        lab, n = gpu.bwlabel(INPUTS["blobs40"], e["conn"], e["only_largest"], e["fill_bubbles"])
        assert n == e["n"], e
        assert raw_hash(lab.astype(np.float32)) == e["sha256"], e


def test_bwlabel_vs_oracle_random(gpu, oracle):
    rng = np.random.default_rng(4)
    for shape, p in (((30, 41, 37), 0.35), ((12, 64, 50), 0.55), ((2, 9, 70), 0.5)):
        img = (rng.random(shape) < p).astype(np.float32)
        for conn in (6, 18, 26):
            for ol, fb in ((False, False), (True, False), (False, True), (True, True)):
                a, na = gpu.bwlabel(img, conn, ol, fb)
                b, nb = oracle.bwlabel(img, conn, ol, fb)
                assert na == nb and np.array_equal(a, b), (shape, conn, ol, fb)


def test_bwlabel_vs_oracle_ct_mask(gpu, oracle):
    """a 200^3 CT-like mask (hundreds of thousands of components, one
    background component spanning the volume, rows of 7 words): every
    connectivity and option set equals the oracle, on repeated calls (a race
    in the labelling would show as a few voxels that differ between calls)"""
    from nii2mesh_gb300 import synth
    img = (synth.ct512(n=200) >= 300.0).astype(np.float32)
    for conn in (6, 18, 26):
        for ol, fb in ((False, False), (True, False), (False, True), (True, True)):
            b, nb = oracle.bwlabel(img, conn, ol, fb)
            for _ in range(2):
                a, na = gpu.bwlabel(img, conn, ol, fb)
                assert na == nb and np.array_equal(a, b), (conn, ol, fb, int((a != b).sum()))


def test_hc_golden(gpu):
    hc = np.load(GOLD / "hc.npz")
    t, p = hc["tris"], hc["pts"]
    for it in (1, 5, 20):
        got = gpu.laplacian_smoothHC(p, t, 0.1, 0.5, it, True)
        err = np.abs(got - hc[f"smoothed_{it}"]).max()
        assert err <= HC_TOL, (it, err)
    got = gpu.laplacian_smoothHC(p, hc["open_tris"], 0.1, 0.5, 5, True)
    err = np.abs(got - hc["open_smoothed_5"]).max()
    assert err <= HC_TOL, err


def test_hc_unlocked_and_isolated(gpu, oracle):
    hc = np.load(GOLD / "hc.npz")
    t, p = hc["tris"], hc["pts"]
    p2 = np.vstack([p, [[1.0, 2.0, 3.0]]])   # an isolated vertex keeps its position
    got = gpu.laplacian_smoothHC(p2, t[::2], 0.1, 0.5, 7, False)
    want = oracle.laplacian_smoothHC(p2, t[::2], 0.1, 0.5, 7, False)
    assert np.abs(got - want).max() <= HC_TOL
    assert np.array_equal(got[-1], p2[-1])


def test_sform_golden(gpu):
    hc = np.load(GOLD / "hc.npz")
    t, p = hc["tris"], hc["pts"]
    for e in G["sform"]:
        tt, pp = gpu.apply_sform(p, t, *e["rows"])
        assert raw_hash(tt.astype(np.int32), pp.astype(np.float64)) == e["sha256"]


def test_hc_rejects_out_of_range_index(gpu):
    """a triangle index outside [0, nvert) (past the end, or negative) fails
    with N2M_ERR_BAD_ARGS through the device entry point and leaves the
    vertices unchanged; the drop-in laplacian_smoothHC leaves the caller's
    vertices unchanged; the next call on the same context is correct again"""
    import ctypes as C
    import torch
    hc = np.load(GOLD / "hc.npz")
    t, p = hc["tris"].astype(np.int32), hc["pts"]
    L = gpu.lib()
    ctx = gpu.Context(0)
    for bad in (len(p), -1, 1 << 30):
        tb = t.copy()
        tb[len(tb) // 2, 1] = bad
        dt = torch.from_numpy(tb).cuda()
        dp = torch.from_numpy(p).cuda()
        st = L.n2m_smooth_hc_device(ctx.h, C.c_void_p(dp.data_ptr()), C.c_void_p(dt.data_ptr()), len(p), len(tb),
                                    0.1, 0.5, 3, True)
        assert st == 4, st
        assert b"outside" in L.n2m_last_error()
        assert np.array_equal(dp.cpu().numpy(), p)
        assert np.array_equal(gpu.laplacian_smoothHC(p, tb, 0.1, 0.5, 3, True), p)
    got = gpu.laplacian_smoothHC(p, t, 0.1, 0.5, 1, True)
    assert np.abs(got - hc["smoothed_1"]).max() <= 1e-4
    ctx.close()
