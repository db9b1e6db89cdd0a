"""Pin the CPU oracle against the reference (CPU only).

The golden fixtures in tests/golden/ were produced by the reference nii2mesh
itself (tests/golden/make_golden.py).  The oracle must reproduce every one of
them bit for bit; where the reference build (oracle/_ref) is present, the
oracle is also compared with it directly on further seeded inputs.
"""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import MC33, MC_CLASSIC_TABLE, OLDCUBES, Reference, canonical, mesh_equal, reference_available
from oracle.refpath import reference_data

GOLD = Path(__file__).resolve().parent / "golden"
G = json.loads((GOLD / "golden.json").read_text())
INPUTS = dict(np.load(GOLD / "inputs.npz"))

# MC self-test known answers (vertices, triangles) of the reference's ten
# analytic 60^3 fields (src/MarchingCubes.c:1282-1405), Lewiner, iso 0
KNOWN_SELFTEST = {0: (302, 600), 1: (792, 1572), 2: (7038, 13720), 3: (554, 1104), 4: (2168, 4352),
                  5: (5304, 10616), 6: (13196, 25834), 7: (11333, 22620), 8: (10800, 20886), 9: (5789, 11298)}


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
def test_meshify_matches_reference(oracle, e):
    m = oracle.meshify(INPUTS[e["input"]], e["iso"], e["variant"], e["pre_smooth"], e["only_largest"],
                       e["fill_bubbles"])
    if e.get("result", 1) is None:
        assert m is None
        return
    assert (len(m[1]), len(m[0])) == (e["nvert"], e["ntri"])
    assert mesh_hash(*m) == e["sha256"]


def test_selftest_known_answers(oracle):
    for obj, (nv, nt) in KNOWN_SELFTEST.items():
        f = oracle.selftest_field(obj)
        assert raw_hash(f) == G["selftest"][str(obj)]["field_sha256"]
        t, v = oracle.mc_raw(f, 0)
        assert (len(v), len(t)) == (nv, nt) == (G["selftest"][str(obj)]["nvert"], G["selftest"][str(obj)]["ntri"])


# The self-test fields written as N.nii (src/MarchingCubes.c:1355-1360) and meshed
# by the reference's whole nii2mesh program with -p 0 -l 0 -b 0 -r 1 -i 0.001:
# (triangles, vertices) after the weld and the degenerate filter, per cube
# variant, read from the .mz3 files it wrote (tests/golden/make_golden.py
# records each command beside its counts).
KNOWN_MCTEST_CLI = {(e["object"], e["variant"]): (e["ntri"], e["nvert"]) for e in G["cli"] if e["input"] == "selftest"}


@pytest.mark.parametrize("obj,variant", [(0, MC33), (1, MC33), (2, MC33), (5, MC33), (8, MC33),
                                         (8, MC_CLASSIC_TABLE), (8, OLDCUBES)])
def test_mctest_cli_known_answers(oracle, obj, variant):
    t, p = oracle.meshify(oracle.selftest_field(obj), 0.001, variant, False, False, False)[:2]
    assert (len(t), len(p)) == KNOWN_MCTEST_CLI[(obj, variant)]


def test_thresholds(oracle):
    for key, val in G["threshold"].items():
        name, mode = key.split(":")
        assert oracle.set_threshold(INPUTS[name], int(mode)) == pytest.approx(val, abs=0, rel=0)


TH = json.loads((GOLD / "threshold.json").read_text())
TH_INPUTS = dict(np.load(GOLD / "threshold_inputs.npz"))


@pytest.mark.parametrize("case", sorted(TH))
def test_threshold_edge_cases(oracle, case):
    """setThreshold edge cases (constant, all-NaN, < 100 voxels, NaNs, zero
    background, ties, outliers, heavy tails) — reference values from
    tests/golden/make_threshold_golden.py, modes 1-3, bit for bit."""
    for mode, val in TH[case].items():
        assert oracle.set_threshold(TH_INPUTS[case], int(mode)) == val


def test_nifti_cast():
    """the oracle's voxel cast equals the reference's load_nii output
    (tests/golden/make_nifti_golden.py) bit for bit on all four datatypes"""
    from oracle.oracle import cast_voxels
    g = np.load(GOLD / "nifti.npz")
    for k in range(sum(1 for n in g.files if n.startswith("raw"))):
        meta = g[f"meta{k}"]
        assert np.array_equal(cast_voxels(g[f"raw{k}"], meta[1], meta[2]).view(np.uint32), g[f"out{k}"].view(np.uint32))


def test_bwlabel(oracle):
    for e in G["bwlabel"]:
        lab, n = oracle.bwlabel(INPUTS["blobs40"], e["conn"], e["only_largest"], e["fill_bubbles"])
        assert n == e["n"]
        assert raw_hash(lab.astype(np.float32)) == e["sha256"]


def test_marching_cubes_order(oracle):
    v = INPUTS["sphere48"]
    for e in G["marching_cubes"]:
        t, p = oracle.marching_cubes(v, e["lo"], e["hi"], e["original_mc"], 50.0)
        assert raw_hash(t.astype(np.int32), p.astype(np.float64)) == e["sha256"]


def test_hc_and_sform(oracle):
    hc = np.load(GOLD / "hc.npz")
    t, p = hc["tris"], hc["pts"]
    for it in (1, 5, 20):
        assert np.array_equal(oracle.laplacian_smoothHC(p, t, 0.1, 0.5, it, True), hc[f"smoothed_{it}"])
    assert np.array_equal(oracle.laplacian_smoothHC(p, hc["open_tris"], 0.1, 0.5, 5, True), hc["open_smoothed_5"])
    for e in G["sform"]:
        tt, pp = oracle.apply_sform(p, t, *e["rows"])
        assert raw_hash(tt.astype(np.int32), pp.astype(np.float64)) == e["sha256"]


@pytest.mark.skipif(not reference_available(), reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("seed", [21, 22, 23])
def test_oracle_vs_reference_random(oracle, seed):
    from nii2mesh_gb300 import synth
    rl, rc = Reference(False), Reference(True)
    vol = synth.spheres(n=40, count=5, rmin=3, rmax=9, cmin=8, cmax=32, noise=12.0, seed=seed)
    for variant, ref in ((MC33, rl), (MC_CLASSIC_TABLE, rl), (OLDCUBES, rc)):
        for flags in ((True, True, True), (False, False, False), (True, False, True)):
            a, b = oracle.meshify(vol, 50.0, variant, *flags), ref.meshify(vol, 50.0, variant, *flags)
            ok, d, msg = mesh_equal(a, b, 0.0)
            assert ok, msg


WRITER_EXTS = ["mz3", "gii", "inflated", "pial", "json", "off", "obj", "ply", "stl", "vtk", "xyz"]


@pytest.mark.parametrize("case", ["sphere", "special", "empty"])
def test_writers_match_reference(case):
    """oracle/writers.py writes the reference's files (tests/golden/writers.npz,
    made by the reference's own save_mesh): every format, with and without
    isGz; compressed sections and the FreeSurfer time stamp compared after
    normalisation; an unknown extension gets .mz3 appended."""
    from oracle import writers as W
    g = np.load(GOLD / "writers.npz")
    t, p = g[f"tris_{case}"], g[f"pts_{case}"]
    for ext in WRITER_EXTS:
        for gz in (False, True):
            want = g[f"{case}_{ext}{'_gz' if gz else ''}"].tobytes()
            fmt = W.format_of(f"{case}.{ext}")
            assert (fmt < 0) == (ext == "xyz")
            got = W.encode(W.FMT_MZ3 if fmt < 0 else fmt, t, p, gz)
            assert W.normalize(got) == W.normalize(want), (case, ext, gz)



REF_DATA = reference_data() or Path("/nonexistent")


def _load_reference_volume(name):
    """a volume of the reference's data/ folder read by its own load_nii
    (oracle/_ref/libn2m_ref_cli.so): float32 (nz, ny, nx) and the header"""
    import ctypes as C
    from oracle.oracle import REF_DIR
    lib = C.CDLL(str(REF_DIR / "libn2m_ref_cli.so"))
    lib.load_nii.restype = C.c_void_p
    lib.load_nii.argtypes = [C.c_char_p, C.c_void_p]
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    hdr = C.create_string_buffer(348)
    p = lib.load_nii(str(REF_DATA / name).encode(), hdr)
    assert p, name
    dims = np.frombuffer(hdr.raw, np.int16, 8, 40)
    nx, ny, nz = (int(d) for d in dims[1:4])
    vol = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_float)), shape=(nx * ny * nz,)).copy()
    libc.free(p)
    srow = np.frombuffer(hdr.raw, np.float32, 12, 280).reshape(3, 4)
    return vol.reshape(nz, ny, nx), srow


# bet.nii.gz through the reference's nii2mesh program with its defaults (Otsu
# medium, -p 1 -l 1 -b 0) and -r 1: (triangles, vertices) per cube variant as its
# .mz3 output holds them (make_golden.py records the commands); the reference's
# meshify called directly must give the same counts
KNOWN_BET = {("bet.nii.gz", e["variant"]): (e["ntri"], e["nvert"]) for e in G["cli"] if e["input"] == "bet.nii.gz"}


@pytest.mark.skipif(not ((REF_DATA / "bet.nii.gz").exists() and reference_available() and reference_available(True)),
                    reason="needs the reference tree (its data/ images and oracle/_ref)")
@pytest.mark.parametrize("name", ["bet.nii.gz", "pve_1.nii.gz", "pve_2.nii.gz"])
def test_real_images_oracle_vs_reference(oracle, name):
    """The reference's own images (data/, read by its load_nii): the default
    isolevel (Otsu medium, src/nii2mesh.c:586) bit for bit, then meshify with
    the CLI defaults (-p 1 -l 1 -b 0), Lewiner and classic tables and the
    oldcubes build, oracle against the reference mesh for mesh; with -b 1 and
    HC post-smoothing plus the header's sform on the Lewiner mesh."""
    vol, srow = _load_reference_volume(name)
    ref, refc = Reference(False), Reference(True)
    iso = ref.set_threshold(vol, 2)
    assert oracle.set_threshold(vol, 2) == iso
    for variant, r in ((MC33, ref), (MC_CLASSIC_TABLE, ref), (OLDCUBES, refc)):
        want = r.meshify(vol, iso, variant, True, True, False)
        got = oracle.meshify(vol, iso, variant, True, True, False)
        ok, d, msg = mesh_equal(got, want, 0.0)
        assert ok, (name, variant, msg)
        if (name, variant) in KNOWN_BET:
            assert (len(got[0]), len(got[1])) == KNOWN_BET[(name, variant)]
    want = ref.meshify(vol, iso, MC33, True, True, True)
    got = oracle.meshify(vol, iso, MC33, True, True, True)
    ok, d, msg = mesh_equal(got, want, 0.0)
    assert ok, (name, "fill bubbles", msg)
    t, p = want
    ps_r, ps_o = ref.laplacian_smoothHC(p, t, iters=5), oracle.laplacian_smoothHC(p, t, iters=5)
    assert np.array_equal(ps_r, ps_o)
    tr, pr = ref.apply_sform(ps_r, t, *srow)
    to, po = oracle.apply_sform(ps_o, t, *srow)
    assert np.array_equal(tr, to) and np.array_equal(pr, po)


@pytest.mark.skipif(not ((REF_DATA / "D99_atlas_v2.0_right.nii.gz").exists() and reference_available()),
                    reason="needs the reference tree (its data/ images and oracle/_ref)")
def test_real_atlas_labels_oracle_vs_reference(oracle):
    """D99 atlas labels (data/, read by load_nii) binarised as the atlas loop
    does (src/nii2mesh.c:555-563) and meshed at iso 0.5 with -l 1 -b 1: a large
    and a small label, oracle against the reference"""
    vol, _ = _load_reference_volume("D99_atlas_v2.0_right.nii.gz")
    labels, counts = np.unique(vol[vol > 0].astype(np.int32), return_counts=True)
    ref = Reference(False)
    for lab in (labels[np.argmax(counts)], labels[np.argmin(counts)]):
        m, _ = oracle.binarize_label(vol, int(lab))
        want = ref.meshify(m, 0.5, MC33, True, True, True)
        got = oracle.meshify(m, 0.5, MC33, True, True, True)
        if want is None:
            assert got is None
            continue
        ok, d, msg = mesh_equal(got, want, 0.0)
        assert ok, (int(lab), msg)
