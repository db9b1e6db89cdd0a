"""CPU-only checks of the product's host side: the exact smoothing arithmetic
(compiled for the host), the C ABI exports, and the workload generators."""
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_exact_tap_sum_matches_double(tmp_path):
    """tap5_fast (nii2mesh_gb300/csrc/exact.cuh) never disagrees with the
    reference's double sequence, over 4M random taps of 12 value families
    (arbitrary finite bit patterns, signed zeros and subnormals included), and
    decides more than 95 % of the taps on ordinary data by itself."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "exact_check"
    subprocess.run([cxx, "-O2", "-ffp-contract=off", "-o", str(exe), str(ROOT / "tests/cpu_harness/exact_check.cpp")],
                   check=True)
    out = subprocess.run([str(exe), "4000000", "11"], capture_output=True, text=True)
    bad, frac = out.stdout.split()[-2:]
    assert out.returncode == 0 and int(bad) == 0, out.stdout
    assert float(frac) > 0.95


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
