"""CPU-only checks of the product's host side: the exact smoothing arithmetic
(compiled for the host), the C ABI exports, and the workload generators."""
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle.refpath import reference_src

ROOT = Path(__file__).resolve().parents[1]


def test_exact_tap_sum_matches_double(tmp_path):
    """tap5_fast and tap5_split (nii2mesh_gb300/csrc/exact.cuh) never disagree
    with the reference's double sequence, over 8M random taps of 16 value
    families (arbitrary finite bit patterns, signed zeros, subnormals, mixed
    signs, cancellation, any binade scale included); tap5_fast decides more
    than 95 % of the taps on ordinary data and tap5_split more than 95 % on
    CT-like data by themselves."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "exact_check"
    subprocess.run([cxx, "-O2", "-ffp-contract=off", "-o", str(exe), str(ROOT / "tests/cpu_harness/exact_check.cpp")],
                   check=True)
    out = subprocess.run([str(exe), "8000000", "11"], capture_output=True, text=True)
    bad, frac, split = out.stdout.split()[-3:]
    assert out.returncode == 0 and int(bad) == 0, out.stdout
    assert float(frac) > 0.95 and float(split) > 0.95


def test_text_formatter_matches_printf(tmp_path):
    """The device %g / %d formatter of the text mesh writers
    (nii2mesh_gb300/csrc/fmt.cuh, compiled for the host) prints exactly what the
    C library's printf prints (src/meshify.c:683-723 call fprintf "%g"): any bit
    pattern, mesh coordinates, float grids, exact ties at the seventh digit,
    powers of ten and their neighbours; its wide path on every value too."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "fmt_check"
    subprocess.run([cxx, "-O2", "-ffp-contract=off", "-o", str(exe), str(ROOT / "tests/cpu_harness/fmt_check.cpp")],
                   check=True)
    out = subprocess.run([str(exe), "600000", "5"], capture_output=True, text=True)
    cases, bad = out.stdout.split()[-2:]
    assert out.returncode == 0 and int(bad) == 0 and int(cases) > 1000000, out.stdout


def test_abi_exports_every_declared_symbol():
    """libn2m_gpu.so loads without a GPU and exports every entry point that
    include/n2m_gpu.h declares (no compute call is made)."""
    from nii2mesh_gb300 import _lib
    if not _lib.LIB_PATH.exists():
        pytest.fail("libn2m_gpu.so not built (run __graft_entry__.build())")
    L = _lib.load()
    hdr = (ROOT / "include" / "n2m_gpu.h").read_text()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    declared = set(re.findall(r"^[A-Za-z_][\w\s\*]*?\b(\w+)\s*\([^;{]*\)\s*;", hdr, flags=re.M))
    declared -= {"if", "while"}
    assert {"meshify", "laplacian_smoothHC", "marchingCubes", "bwlabel", "n2m_meshify"} <= declared
    for name in sorted(declared | set(_lib.SYMBOLS)):
        assert hasattr(L, name), f"missing export {name}"


def test_generators_deterministic():
    from nii2mesh_gb300 import synth
    a, b = synth.spheres(n=32, count=3, rmin=3, rmax=6, cmin=8, cmax=24, seed=3), \
        synth.spheres(n=32, count=3, rmin=3, rmax=6, cmin=8, cmax=24, seed=3)
    assert a.dtype == np.float32 and a.shape == (32, 32, 32) and np.array_equal(a, b)
    c = synth.ct512(seed=5, n=40, count=4)
    assert c.dtype == np.float32 and c.shape == (40, 40, 40)
    assert (c == 2000.0).mean() == pytest.approx(0.01, abs=0.003)
    at = synth.atlas256(n=48, labels=20)
    assert at.dtype == np.int16 and at.max() <= 20 and at.min() >= 0


def test_mesh_format_rule_matches_reference_rule():
    """n2m_mesh_format_of (host code of the library, no GPU call) picks the
    format save_mesh picks (strip_ext + strstr, src/meshify.c:973-1019), as
    restated in oracle/writers.py, on awkward names"""
    from nii2mesh_gb300 import _lib
    from oracle import writers as W
    if not _lib.LIB_PATH.exists():
        pytest.fail("libn2m_gpu.so not built (run __graft_entry__.build())")
    L = _lib.load()
    names = ["a.mz3", "a.gii", "a.obj", "a.OBJ", "lh.pial", "lh.inflated", "x.json", "x.off", "x.ply", "x.stl",
             "x.vtk", "x.xyz", "x", "", ".obj", "dir.obj/file", "dir/.obj", "a.b.stl", "a.stl.gz", "a.gii.mz3",
             "a.mz3x", "a.xmz3", "a.json5", "a.vtkx", "C:\\dir.obj\\f", "a.obj.", "a..obj", "./a.ply", "a.inflatedx",
             "mesh.pial.gz", "m.offset", "a/b.c/d.gii"]
    for n in names:
        assert L.n2m_mesh_format_of(n.encode()) == W.format_of(n), n


REF_SRC = reference_src() or Path("/nonexistent")


@pytest.mark.skipif(not (REF_SRC / "nii2mesh.c").exists() or shutil.which("gcc") is None,
                    reason="needs the reference tree and gcc")
def test_reference_program_links_against_library(tmp_path):
    """The reference's own program (its nii2mesh.c, with quadric.c for the
    decimation and base64.c) links against libn2m_gpu.so in place of
    meshify.o, isolevel.o, MarchingCubes.o, bwlabel.o and radixsort.o: every
    symbol it takes from those objects is exported with the same signature
    (include/n2m_gpu.h).  Compiled in a temporary directory; it runs and prints
    its usage."""
    from nii2mesh_gb300 import _lib
    if not _lib.LIB_PATH.exists():
        pytest.fail("libn2m_gpu.so not built (run __graft_entry__.build())")
    probe = subprocess.run(["gcc", "-x", "c", "-", "-lz", "-o", str(tmp_path / "z")], input="#include <zlib.h>\nint main(void){return 0;}\n",
                           capture_output=True, text=True)
    zl = ["-DHAVE_ZLIB"] if probe.returncode == 0 else []
    objs = []
    for src, extra in (("nii2mesh.c", []), ("base64.c", []), ("quadric.c", ["-Dlaplacian_smoothHC=ref_laplacian_smoothHC"])):
        o = tmp_path / (src + ".o")
        subprocess.run(["gcc", "-O1", "-w", "-DNII2MESH", "-DHAVE_FORMATS", *zl, *extra, "-I", str(ROOT / "include"),
                        "-I", str(REF_SRC), "-c", str(REF_SRC / src), "-o", str(o)], check=True)
        objs.append(str(o))
    exe = tmp_path / "nii2mesh"
    lib_dir = str(_lib.LIB_PATH.parent)
    r = subprocess.run(["gcc", "-o", str(exe), *objs, "-L", lib_dir, "-ln2m_gpu", f"-Wl,-rpath,{lib_dir}", "-lm"] +
                       (["-lz"] if zl else []), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert "Usage" in out.stdout


# SHA-256 of the reference's marching-cubes tables (the LookUpTable.h tables in
# process_cube's order, then oldcubes.c's edgeTable and triTable), each element
# a little-endian int32, as tests/cpu_harness/table_check.c writes them: taken
# from the reference's own files where they are present (the test below checks
# it there), and compared with the packed tables everywhere.
MC_TABLES_SHA256 = "c6dc08cd3fc42588817af879b104779dbee4e8e96aac983914f5e523203e6e94"


def _classic_tables_inc(src_text):
    """oldcubes.c's edgeTable / triTable declarations with their initialisers,
    cut verbatim out of the function that holds them"""
    out = []
    for decl in (r"int\s+edgeTable\s*\[256\]\s*=", r"int\s+triTable\s*\[256\]\s*\[16\]\s*="):
        i = re.search(decl, src_text).start()
        j = src_text.index("};", i) + 2
        out.append(src_text[i:j])
    return "\n".join(out) + "\n"


def test_mc_tables_match_reference(tmp_path):
    """every entry of the packed tables (nii2mesh_gb300/csrc/mc_tables.h) equals
    the reference's, read by the C compiler from LookUpTable.h and oldcubes.c
    (not by the script that generated the packed copy); without the reference
    tree, the packed tables' stream must hash to the reference's committed hash"""
    import hashlib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("needs a C compiler")
    csrc = ROOT / "nii2mesh_gb300" / "csrc"
    exe = tmp_path / "tc_ours"
    subprocess.run([cc, "-O1", "-fsigned-char", "-I", str(csrc), "-o", str(exe),
                    str(ROOT / "tests/cpu_harness/table_check.c")], check=True)
    ours = subprocess.run([str(exe), "ours"], check=True, capture_output=True).stdout
    assert hashlib.sha256(ours).hexdigest() == MC_TABLES_SHA256
    src = reference_src()
    if src is None:
        return
    (tmp_path / "classic_tables.inc").write_text(_classic_tables_inc((src / "oldcubes.c").read_text()))
    exe = tmp_path / "tc_ref"
    subprocess.run([cc, "-O1", "-fsigned-char", "-w", "-DWITH_REFERENCE", "-I", str(csrc), "-I", str(src),
                    "-I", str(tmp_path), "-o", str(exe), str(ROOT / "tests/cpu_harness/table_check.c")], check=True)
    r = subprocess.run([str(exe), "ref"], capture_output=True)
    assert r.returncode == 0, r.stderr.decode()[-2000:]
    assert r.stdout == ours
    assert hashlib.sha256(r.stdout).hexdigest() == MC_TABLES_SHA256
