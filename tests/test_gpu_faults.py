"""Host-side fault injection: a device allocation that fails (n2m_debug_fail_
allocations) at every point of a call in turn.  Each call must return
N2M_ERR_OOM without a crash, and the same context must then produce the
correct result.  No GPU fault is involved: the failing allocation is refused on
the host before cudaMalloc is called."""
import numpy as np
import pytest

from nii2mesh_gb300 import synth

pytestmark = pytest.mark.gpu

OOM = 3


def _walk(gpu, run, check, limit=150):
    """for k = 0, 1, ...: a fresh context whose k-th allocation fails; the call
    must fail with N2M_ERR_OOM and the context then work; stops at the first k
    the call no longer reaches (every allocation point covered).  Returns the
    number of allocation points."""
    L = gpu.lib()
    try:
        for k in range(limit):
            ctx = gpu.Context(0)
            L.n2m_debug_fail_allocations(k)
            try:
                out = run(ctx)
            except gpu.N2MError as e:
                assert e.status == OOM, (k, str(e))
                L.n2m_debug_fail_allocations(-1)
                check(run(ctx))
                ctx.close()
                continue
            L.n2m_debug_fail_allocations(-1)
            check(out)
            ctx.close()
            return k
    finally:
        L.n2m_debug_fail_allocations(-1)
    raise AssertionError("more allocation points than the limit")


def test_meshify_survives_allocation_failures(gpu):
    vol = synth.spheres(n=40, count=4, rmin=4, rmax=9, cmin=9, cmax=31, seed=4)
    want = gpu.Context(0).meshify(vol, 50.0, gpu.MC33, True, True, True, 2)[:2]

    def check(out):
        assert np.array_equal(out[0], want[0]) and np.array_equal(out[1], want[1])

    assert _walk(gpu, lambda ctx: ctx.meshify(vol, 50.0, gpu.MC33, True, True, True, 2)[:2], check) >= 10


def test_meshify_into_and_atlas_survive_allocation_failures(gpu):
    vol = synth.ct512(seed=2, n=48, count=6)
    want = gpu.Context(0).meshify(vol, 300.0, gpu.MC33, True, False, False)[:2]
    tb, pb = np.empty((len(want[0]) + 8, 3), np.int32), np.empty((len(want[1]) + 8, 3), np.float64)

    def run_into(ctx):
        nt, nv, _ = ctx.meshify_into(vol, tb, pb, 300.0, gpu.MC33, True, False, False)
        return tb[:nt].copy(), pb[:nv].copy()

    def check(out):
        assert np.array_equal(out[0], want[0]) and np.array_equal(out[1], want[1])

    assert _walk(gpu, run_into, check) >= 5

    lab = synth.atlas256(n=48, labels=12)
    want_a = gpu.Context(0).atlas(lab)

    def check_a(out):
        assert len(out) == len(want_a)
        for (l1, s1, t1, p1), (l2, s2, t2, p2) in zip(out, want_a):
            assert (l1, s1) == (l2, s2) and np.array_equal(t1, t2) and np.array_equal(p1, p2)

    assert _walk(gpu, lambda ctx: ctx.atlas(lab), check_a) >= 5


def test_writers_survive_allocation_failures(gpu):
    from oracle import writers as W
    vol = synth.spheres(n=40, count=4, rmin=4, rmax=9, cmin=9, cmax=31, seed=5)
    t, p, _ = gpu.Context(0).meshify(vol, 50.0, gpu.MC33, True, False, False)
    want = W.normalize(W.encode(W.FMT_GII, t, p, True))

    def check(b):
        assert W.normalize(b) == want

    # GIfTI with zlib: mesh upload, packing, two deflate streams, base64
    assert _walk(gpu, lambda ctx: ctx.encode_mesh(gpu.FMT_GII, t, p, True), check) >= 5
