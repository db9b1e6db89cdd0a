"""GPU parity of meshify (src/meshify.c:286-389) against the oracle.

Every case runs the CUDA path through the C ABI and the CPU oracle on the same
seeded input.  The bar: identical vertex and triangle counts, identical
triangle connectivity after canonical sorting, vertex positions bit-identical
(tolerance 0.0; the path reproduces the reference's float arithmetic).
"""
import numpy as np
import pytest

from nii2mesh_gb300 import synth
from oracle.oracle import MC33, MC_CLASSIC_TABLE, OLDCUBES, mesh_equal, smoothed_equal

pytestmark = pytest.mark.gpu

POS_TOL = 0.0   # raw vertices are bit-exact (spec bar: 1e-5 voxels)
HC_TOL = 1e-4   # HC-smoothed vertices, voxels (spec bar)


def small_spheres(seed=10, n=48):
    return synth.spheres(n=n, count=6, rmin=5, rmax=11, cmin=10, cmax=n - 10, seed=seed)


def run_both(gpu, oracle, vol, iso, variant, smooth, largest, bubbles):
    got = gpu.meshify(vol, iso, original_mc=1 if variant == MC_CLASSIC_TABLE else 0, pre_smooth=smooth,
                      only_largest=largest, fill_bubbles=bubbles, oldcubes=variant == OLDCUBES)
    want = oracle.meshify(vol, iso, variant, smooth, largest, bubbles)
    return got, want


@pytest.mark.parametrize("variant", [MC33, MC_CLASSIC_TABLE, OLDCUBES])
@pytest.mark.parametrize("flags", [(True, True, False), (True, False, False), (False, False, False),
                                   (True, True, True), (False, True, True), (True, False, True)])
def test_spheres_all_options(gpu, oracle, variant, flags):
    vol = small_spheres()
    got, want = run_both(gpu, oracle, vol, 50.0, variant, *flags)
    assert want is not None and got is not None
    ok, d, msg = mesh_equal(got, want, POS_TOL)
    assert ok, msg


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_sphere64_config(gpu, oracle, seed):
    """the 64^3 workload (-p 1 -l 1 -b 0 -o 0)"""
    vol = synth.spheres(seed=seed)
    got, want = run_both(gpu, oracle, vol, 50.0, MC33, True, True, False)
    ok, d, msg = mesh_equal(got, want, POS_TOL)
    assert ok, msg


@pytest.mark.parametrize("variant", [MC33, MC_CLASSIC_TABLE, OLDCUBES])
def test_ct_like(gpu, oracle, variant):
    """CT-like values (negative background, salt noise), iso 300, no clustering"""
    vol = synth.ct512(seed=5, n=96, count=12)
    got, want = run_both(gpu, oracle, vol, 300.0, variant, True, False, False)
    ok, d, msg = mesh_equal(got, want, POS_TOL)
    assert ok, msg


def test_brain_u8(gpu, oracle):
    """brain-sized u8 volume, Otsu iso, -p 1 -l 1 -b 1, both cube tables"""
    vol = synth.brain().astype(np.float32)
    iso = oracle.set_threshold(vol, 2)
    for variant in (MC33, MC_CLASSIC_TABLE):
        got, want = run_both(gpu, oracle, vol, iso, variant, True, True, True)
        ok, d, msg = mesh_equal(got, want, POS_TOL)
        assert ok, msg


@pytest.mark.parametrize("variant", [MC33, MC_CLASSIC_TABLE, OLDCUBES])
def test_brain182_full_options(gpu, oracle, variant):
    """the brain-sized workload with every option it names: 182x218x182 uint8
    cast to float32, the Otsu 'medium' isolevel of the raw volume, -p 1 -l 1
    -b 1 with the Lewiner (-o 0) and classic (-o 1) tables and the classic
    build's oldcubes, then -s 20 HC
    smoothing as nii2 runs it (alpha 0.1, beta 0.5, borders locked;
    src/nii2mesh.c:326-331).  The isolevel and the raw mesh must equal the
    oracle's bit for bit; the smoothed vertices, through the drop-in
    laplacian_smoothHC and through n2m_meshify's own post-smooth, must lie
    within 1e-4 voxels of the oracle's FP64 HC (src/quadric.c:343-394)"""
    vol = synth.brain().astype(np.float32)
    iso = oracle.set_threshold(vol, 2)
    assert gpu.set_threshold(vol, 2) == iso
    got, want = run_both(gpu, oracle, vol, iso, variant, True, True, True)
    ok, d, msg = mesh_equal(got, want, POS_TOL)
    assert ok, msg
    assert len(want[0]) > 100_000
    want_s = oracle.laplacian_smoothHC(want[1], want[0], 0.1, 0.5, 20, True)
    got_s = gpu.laplacian_smoothHC(got[1], got[0], 0.1, 0.5, 20, True)
    ok, d, msg = smoothed_equal(got, got_s, want, want_s, HC_TOL)
    assert ok, msg
    ctx = gpu.Context(0)
    cubes = {MC33: gpu.MC33, MC_CLASSIC_TABLE: gpu.CLASSIC_TABLE, OLDCUBES: gpu.OLDCUBES}[variant]
    t, p, _ = ctx.meshify(vol, iso, cubes, True, True, True, post_smooth=20)
    assert np.array_equal(t, got[0])
    assert np.abs(p - got_s).max() <= HC_TOL
    ctx.close()


@pytest.mark.parametrize("variant", [MC33, OLDCUBES])
def test_ct_labelling_256(gpu, oracle, variant):
    """-p 1 -l 1 -b 1 on a 256^3 CT-like volume through the device entry
    point, three calls in a row: the oracle's mesh every time"""
    vol = synth.ct512(n=256)
    want = oracle.meshify(vol, 300.0, variant, True, True, True)
    ctx = gpu.Context(0)
    cubes = gpu.OLDCUBES if variant == OLDCUBES else gpu.MC33
    for _ in range(3):
        got = device_mesh(gpu, ctx, vol, 300.0, cubes, True, True)
        ok, d, msg = mesh_equal(got, want, POS_TOL)
        assert ok, msg
    ctx.close()


def test_selftest_fields_meshify(gpu, oracle):
    """the reference's analytic self-test fields through the whole pipeline"""
    for obj in range(10):
        f = oracle.selftest_field(obj)
        for variant in (MC33, MC_CLASSIC_TABLE):
            got, want = run_both(gpu, oracle, f, 0.001, variant, False, False, False)
            if want is None:
                assert got is None
                continue
            ok, d, msg = mesh_equal(got, want, POS_TOL)
            assert ok, f"object {obj} variant {variant}: {msg}"


def test_iso_out_of_range(gpu, oracle):
    vol = small_spheres()
    for iso in (-1e6, 1e6, float(vol.max()) + 1):
        got, want = run_both(gpu, oracle, vol, iso, MC33, True, True, False)
        ok, d, msg = mesh_equal(got, want, POS_TOL)
        assert ok, msg


def test_failures(gpu, oracle):
    flat = np.full((16, 16, 16), 3.0, np.float32)
    assert gpu.meshify(flat, 1.0) is None
    assert oracle.meshify(flat, 1.0) is None


def test_small_dims_skip_smoothing(gpu, oracle):
    vol = small_spheres()[:4, :, :].copy()   # nz < 5: the reference skips the pre-smooth
    got, want = run_both(gpu, oracle, vol, 50.0, MC33, True, False, False)
    ok, d, msg = mesh_equal(got, want, POS_TOL)
    assert ok, msg


def test_ragged_dims(gpu, oracle):
    rng = np.random.default_rng(7)
    for shape in ((37, 5, 61), (5, 33, 7), (70, 19, 33)):
        vol = (rng.random(shape) * 100).astype(np.float32)
        got, want = run_both(gpu, oracle, vol, 50.0, MC33, True, False, False)
        if want is None:
            assert got is None
            continue
        ok, d, msg = mesh_equal(got, want, POS_TOL)
        assert ok, f"{shape}: {msg}"


def test_bbox_touches_volume_faces(gpu, oracle):
    """bright voxels on the faces exercise the padded grid and its row wrap"""
    rng = np.random.default_rng(3)
    vol = rng.normal(0, 1, (20, 24, 28)).astype(np.float32)
    vol[:, :, -3:] += 10
    vol[-2:, :, :] += 10
    for variant in (MC33, OLDCUBES):
        got, want = run_both(gpu, oracle, vol, 4.0, variant, True, False, False)
        ok, d, msg = mesh_equal(got, want, POS_TOL)
        assert ok, msg


@pytest.mark.parametrize("shape", [(48, 52, 64), (96, 96, 96), (40, 33, 36), (64, 64, 128)])
@pytest.mark.parametrize("variant", [MC33, OLDCUBES])
@pytest.mark.parametrize("bubbles", [False, True])
def test_device_path_on_demand_labelling(gpu, oracle, shape, variant, bubbles):
    """-l 1 (with and without -b 1) on device-resident volumes whose rows
    allow the on-demand pre-smooth: the mask is pass A's sign bitmap, the
    exact values at the marching cubes' corners get the clustering's fill and
    mask-out; equal to the oracle bit for bit.  The last volume masks nothing
    out (its one component's dilation covers it), which takes the exact
    three passes instead"""
    ctx = gpu.Context(0)
    nz, ny, nx = shape
    cubes = gpu.OLDCUBES if variant == OLDCUBES else gpu.MC33
    full = np.full(shape, 100.0, np.float32) + synth.spheres(n=max(shape), count=3, seed=3)[:nz, :ny, :nx]
    full[nz // 2 - 1:nz // 2 + 2, ny // 2 - 1:ny // 2 + 2, nx // 2 - 1:nx // 2 + 2] = 0.0
    vols = [(synth.ct512(seed=sum(shape), n=max(shape), count=10)[:nz, :ny, :nx].copy(), 300.0),
            (synth.spheres(n=max(shape), count=6, rmin=5, rmax=12, cmin=10, cmax=max(shape) - 10, noise=20.0,
                           seed=nx)[:nz, :ny, :nx].copy(), 50.0),
            (full, 50.0)]
    for vol, iso in vols:
        want = oracle.meshify(vol, iso, variant, True, True, bubbles)
        got = device_mesh(gpu, ctx, vol, iso, cubes, True, bubbles)
        ok, d, msg = mesh_equal(got, want, POS_TOL)
        assert ok, (shape, iso, msg)
    ctx.close()


def test_meshify_into_caller_buffers(gpu):
    """n2m_meshify_into writes the same mesh as n2m_meshify into reused caller
    arrays (pageable and pinned), staged and unstaged uploads, with and without
    HC post-smoothing; a mesh that does not fit fails with N2M_ERR_TOO_LARGE
    and reports the room it needs"""
    import torch
    ctx = gpu.Context(0)
    vol = synth.ct512(seed=6, n=80, count=10)
    for smooth, post in ((True, 0), (False, 0), (True, 3)):
        t, p, _ = ctx.meshify(vol, 300.0, gpu.MC33, smooth, False, False, post)
        for pinned in (False, True):
            if pinned:
                tb = torch.empty((len(t) + 100, 3), dtype=torch.int32, pin_memory=True).numpy()
                pb = torch.empty((len(p) + 100, 3), dtype=torch.float64, pin_memory=True).numpy()
            else:
                tb, pb = np.empty((len(t) + 100, 3), np.int32), np.empty((len(p) + 100, 3), np.float64)
            for _ in range(2):
                nt, nv, rep = ctx.meshify_into(vol, tb, pb, 300.0, gpu.MC33, smooth, False, False, post)
                assert (nt, nv) == (len(t), len(p))
                assert np.array_equal(tb[:nt], t) and np.array_equal(pb[:nv], p)
    small_t, small_p = np.empty((10, 3), np.int32), np.empty((len(p), 3), np.float64)
    with pytest.raises(gpu.N2MError) as e:
        ctx.meshify_into(vol, small_t, small_p, 300.0, gpu.MC33, True, False, False, 3)
    assert e.value.status == 8 and e.value.needed == (len(t), len(p))


@pytest.mark.parametrize("shape", [(23, 29, 37), (40, 48, 64), (17, 61, 33)])
@pytest.mark.parametrize("variant", [MC33, MC_CLASSIC_TABLE])
def test_ragged_shapes_no_clustering(gpu, oracle, shape, variant):
    """pre-smoothing without clustering on shapes whose rows and slices are not
    multiples of 32 voxels (MC words straddle rows of the volume), host (staged
    upload) and device paths against the oracle, with an isolevel in range and
    one that falls back to mid-range"""
    import torch
    rng = np.random.default_rng(sum(shape))
    vol = (rng.normal(0, 30, shape) + 100 * (rng.random(shape) < 0.3)).astype(np.float32)
    for iso in (40.0, 1e6):   # 1e6: out of range, the isolevel falls back
        got, want = run_both(gpu, oracle, vol, iso, variant, True, False, False)
        ok, d, msg = mesh_equal(got, want, POS_TOL)
        assert ok, (iso, msg)
        ctx = gpu.Context(0)
        dv = torch.from_numpy(vol).cuda()
        nz, ny, nx = shape
        cubes = gpu.CLASSIC_TABLE if variant == MC_CLASSIC_TABLE else gpu.MC33
        dt, dp, nt, nv, _ = ctx.meshify_device(dv.data_ptr(), (nx, ny, nz), iso, cubes, True, False, False)
        assert (nt, nv) == (len(want[0]), len(want[1]))


def test_ct512_full_size_bit_exact(gpu, oracle):
    """the benchmark workload at full size (512^3 CT-like, iso 300, -p 1 -l 0
    -b 0, Lewiner; 7.1 M triangles): the host-memory call, the caller-buffer
    call and the oracle give the same mesh, connectivity and every vertex"""
    vol = synth.ct512()
    got = gpu.meshify(vol, 300.0, pre_smooth=True, only_largest=False, fill_bubbles=False)
    want = oracle.meshify(vol, 300.0, MC33, True, False, False)
    assert len(got[0]) > 7_000_000
    ok, d, msg = mesh_equal(got, want, POS_TOL)
    assert ok, msg
    ctx = gpu.Context(0)
    tb, pb = np.empty((len(got[0]), 3), np.int32), np.empty((len(got[1]), 3), np.float64)
    nt, nv, _ = ctx.meshify_into(vol, tb, pb, 300.0, gpu.MC33, True, False, False)
    assert np.array_equal(tb[:nt], got[0]) and np.array_equal(pb[:nv], got[1])
    # the device-resident call (pre-smooth with exact rounding on demand) gives the same mesh
    dt, dp = device_mesh(gpu, ctx, vol, 300.0, gpu.MC33)
    assert np.array_equal(dt, got[0]) and np.array_equal(dp, got[1])


def device_mesh(gpu, ctx, vol, iso, cubes, largest=False, bubbles=False):
    """n2m_meshify_device on a CUDA copy of vol; the mesh copied back to host arrays"""
    import torch
    from nii2mesh_gb300.autograd import _DeviceView
    d = torch.from_numpy(vol).cuda()
    nz, ny, nx = vol.shape
    tp, pp, nt, nv, _ = ctx.meshify_device(d.data_ptr(), (nx, ny, nz), iso, cubes, True, largest, bubbles)
    t = torch.as_tensor(_DeviceView(tp, (nt, 3), "<i4"), device="cuda").cpu().numpy().copy()
    p = torch.as_tensor(_DeviceView(pp, (nv, 3), "<f8"), device="cuda").cpu().numpy().copy()
    return t, p


@pytest.mark.parametrize("shape", [(48, 52, 64), (96, 96, 96), (40, 33, 36), (64, 64, 128), (31, 29, 37)])
@pytest.mark.parametrize("variant", [MC33, MC_CLASSIC_TABLE, OLDCUBES])
def test_device_path_on_demand_smoothing(gpu, oracle, shape, variant):
    """device-resident volumes whose rows are a multiple of 4 voxels take the
    pre-smooth with exact rounding on demand (pass A over TMA tiles, exact
    values only where marching cubes reads them); rows of other lengths the
    exact three passes: either way the oracle's mesh, bit for bit, on CT-like
    data, on spheres with noise around the isolevel and on an isolevel that
    falls back to mid-range"""
    ctx = gpu.Context(0)
    nz, ny, nx = shape
    cubes = {MC33: gpu.MC33, MC_CLASSIC_TABLE: gpu.CLASSIC_TABLE, OLDCUBES: gpu.OLDCUBES}[variant]
    vols = [(synth.ct512(seed=sum(shape), n=max(shape), count=10)[:nz, :ny, :nx].copy(), 300.0),
            (synth.spheres(n=max(shape), count=6, rmin=5, rmax=12, cmin=10, cmax=max(shape) - 10, noise=20.0,
                           seed=nx)[:nz, :ny, :nx].copy(), 50.0)]
    vols.append((vols[1][0], 1e6))
    for vol, iso in vols:
        want = oracle.meshify(vol, iso, variant, True, False, False)
        got = device_mesh(gpu, ctx, vol, iso, cubes)
        ok, d, msg = mesh_equal(got, want, POS_TOL)
        assert ok, (shape, iso, msg)
    ctx.close()
