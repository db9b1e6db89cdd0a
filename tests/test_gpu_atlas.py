"""Atlas meshing (src/nii2mesh.c:492-583): the batched all-labels path against
the per-label loop (identical meshes) and against the oracle run label by
label on the binarised volume (connectivity exact; positions exact without
post-smoothing, within 1e-4 voxels after HC)."""
import numpy as np
import pytest

from nii2mesh_gb300 import synth
from oracle.oracle import mesh_equal, smoothed_equal

pytestmark = pytest.mark.gpu


def small_atlas(seed=3, n=64, labels=24):
    return synth.atlas256(seed=seed, n=n, labels=labels)


@pytest.mark.parametrize("flags", [(True, True, True, 5), (True, False, False, 0), (False, True, False, 0),
                                   (True, False, True, 2)])
def test_batched_equals_loop_and_oracle(gpu, oracle, flags):
    smooth, largest, bubbles, iters = flags
    lab = small_atlas()
    ctx = gpu.Context(0)
    kw = dict(pre_smooth=smooth, only_largest=largest, fill_bubbles=bubbles, post_smooth=iters)
    batched = ctx.atlas(lab, mode=gpu.ATLAS_BATCHED, **kw)
    loop = ctx.atlas(lab, mode=gpu.ATLAS_LOOP, **kw)
    raw = ctx.atlas(lab, mode=gpu.ATLAS_BATCHED, **dict(kw, post_smooth=0)) if iters else batched
    present = sorted(set(np.unique(lab)) - {0})
    assert [m[0] for m in batched] == [m[0] for m in loop] == present
    img = lab.astype(np.float32)
    for (l, sb, tb, pb), (_, sl, tl, pl), (_, _, tr, pr) in zip(batched, loop, raw):
        assert sb == sl, l
        if sb:
            continue
        assert np.array_equal(tb, tl) and np.array_equal(pb, pl), f"label {l}: batched != loop"
        binimg, n = oracle.binarize_label(img, int(l))
        want = oracle.meshify(binimg, 0.5, 0, smooth, largest, bubbles)
        assert want is not None, l
        if iters:
            ws = oracle.laplacian_smoothHC(want[1], want[0], 0.1, 0.5, iters, True)
            ok, d, msg = smoothed_equal((tr, pr), pb, want, ws, 1e-4)
        else:
            ok, d, msg = mesh_equal((tb, pb), want, 0.0)
        assert ok, f"label {l}: {msg}"
    ctx.close()


def test_atlas_labels_touching_faces(gpu, oracle):
    """labels that reach the volume faces (edge darkening, row wrap, clipped sub-boxes)"""
    rng = np.random.default_rng(9)
    lab = np.zeros((20, 24, 28), np.int16)
    lab[:, :, -4:] = 1
    lab[:3, :, :] = 2
    lab[8:14, 5:15, 0:6] = 3
    lab[rng.random(lab.shape) < 0.01] = 4
    ctx = gpu.Context(0)
    batched = ctx.atlas(lab, mode=gpu.ATLAS_BATCHED, pre_smooth=True, only_largest=False, fill_bubbles=True,
                        post_smooth=0)
    img = lab.astype(np.float32)
    for l, st, t, p in batched:
        binimg, _ = oracle.binarize_label(img, int(l))
        want = oracle.meshify(binimg, 0.5, 0, True, False, True)
        if st:
            assert want is None
            continue
        ok, d, msg = mesh_equal((t, p), want, 0.0)
        assert ok, f"label {l}: {msg}"
    ctx.close()


def test_atlas256_full_size(gpu, oracle):
    """the benchmark workload at full size (256^3 int16, ~250 power-law labels,
    -p 1 -l 1 -b 1 -s 5): batched equals the per-label loop on every label;
    eight labels from the smallest to the largest against the oracle (raw
    meshes bit for bit, HC within 1e-4 voxels)"""
    lab = synth.atlas256()
    ctx = gpu.Context(0)
    kw = dict(pre_smooth=True, only_largest=True, fill_bubbles=True)
    batched = ctx.atlas(lab, mode=gpu.ATLAS_BATCHED, post_smooth=5, **kw)
    loop = ctx.atlas(lab, mode=gpu.ATLAS_LOOP, post_smooth=5, **kw)
    raw = {m[0]: m for m in ctx.atlas(lab, mode=gpu.ATLAS_BATCHED, post_smooth=0, **kw)}
    assert len(batched) == len(loop) > 200
    for (l, sb, tb, pb), (l2, sl, tl, pl) in zip(batched, loop):
        assert (l, sb) == (l2, sl) and np.array_equal(tb, tl) and np.array_equal(pb, pl), l
    ids, counts = np.unique(lab[lab > 0], return_counts=True)
    sample = [int(ids[i]) for i in np.argsort(counts)[np.linspace(0, len(ids) - 1, 8).astype(int)]]
    img = lab.astype(np.float32)
    by_label = {m[0]: m for m in batched}
    for l in sample:
        binimg, _ = oracle.binarize_label(img, l)
        want = oracle.meshify(binimg, 0.5, 0, True, True, True)
        _, st, t, p = by_label[l]
        if want is None:
            assert st != 0
            continue
        _, _, tr, pr = raw[l]
        ok, d, msg = mesh_equal((tr, pr), want, 0.0)
        assert ok, f"label {l}: {msg}"
        ws = oracle.laplacian_smoothHC(want[1], want[0], 0.1, 0.5, 5, True)
        ok, d, msg = smoothed_equal((tr, pr), p, want, ws, 1e-4)
        assert ok, f"label {l} (HC): {msg}"
    ctx.close()
