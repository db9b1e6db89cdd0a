#!/usr/bin/env python3
"""Generate the mesh-writer fixtures (save_mesh, src/meshify.c:984-1019) from
the reference nii2mesh itself: every format it writes, plain and with isGz,
for three meshes, written by the reference's own save_mesh
(oracle/_ref/libn2m_ref_cli.so, built from its sources with HAVE_FORMATS and
zlib).

Run where the reference tree exists:  python tests/golden/make_writer_golden.py

Writes writers.npz:
  tris_<case>, pts_<case>         the input meshes
  <case>_<ext>[_gz]               the bytes of the reference's file (uint8);
                                  for .mz3 with isGz the gunzipped bytes (the
                                  compressed bytes depend on the deflate search)
"""
import ctypes as C
import gzip
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from nii2mesh_gb300 import synth  # noqa: E402
from oracle.oracle import Oracle  # noqa: E402

from oracle.refpath import reference_src  # noqa: E402

SRC = reference_src()   # N2M_REFERENCE, or a `reference` checkout beside this repository
EXTS = ["mz3", "gii", "inflated", "pial", "json", "off", "obj", "ply", "stl", "vtk"]


def meshes():
    o = Oracle()
    vol = synth.spheres(n=24, count=2, rmin=4, rmax=7, cmin=7, cmax=17, seed=11)
    tris, pts = o.meshify(vol, 50.0, pre_smooth=True, only_largest=False)[:2]
    # scanner-like affine: mm coordinates with long decimal expansions
    A = np.array([[0.9375, 0.0123, 0.0, -90.5], [0.0, 1.1, 0.0207, -126.25], [0.0, -0.004, 1.2, -72.0]])
    pts = pts @ A[:, :3].T + A[:, 3]
    rng = np.random.default_rng(5)
    special = np.array([0.0, -0.0, 1e-5, 9.99995e-5, 9.999949e-5, 0.0001, 123456.5, 123457.5, 999999.5, 1234567.0,
                        -1e-20, 1e22, 3.0000001, 1.0 / 3.0, -2.5e-5, 100000.0, 1e6, 5e-324, 1.7976931348623157e308,
                        -0.1, 65504.0, 1e-300, 2.0 ** -30, 7.0, -1234.5678])
    sp = np.concatenate([special, rng.normal(0, 300, 3 * 30 - len(special))]).reshape(30, 3)
    st = rng.integers(0, 30, (17, 3)).astype(np.int32)
    return {"sphere": (np.ascontiguousarray(tris, np.int32), np.ascontiguousarray(pts, np.float64)),
            "special": (st, sp),
            "empty": (np.zeros((0, 3), np.int32), np.zeros((0, 3), np.float64))}


def main():
    subprocess.run(["sh", str(ROOT / "oracle" / "build_ref.sh"), str(SRC)], check=True, stdout=subprocess.DEVNULL)
    lib = C.CDLL(str(ROOT / "oracle" / "_ref" / "libn2m_ref_cli.so"))
    lib.save_mesh.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_bool]
    out = {}
    with tempfile.TemporaryDirectory() as td:
        for name, (t, p) in meshes().items():
            out[f"tris_{name}"] = t
            out[f"pts_{name}"] = p
            for ext in EXTS + ["xyz"]:
                for gz in (False, True):
                    f = Path(td) / f"{name}.{ext}"
                    r = lib.save_mesh(str(f).encode(), t.ctypes.data, p.ctypes.data, len(t), len(p), gz)
                    assert r == 0, (name, ext, gz)
                    if ext == "xyz":   # unknown extension: the reference appends .mz3
                        f = Path(td) / f"{name}.xyz.mz3"
                    data = f.read_bytes()
                    if ext in ("mz3", "xyz") and gz:
                        data = gzip.decompress(data)
                    out[f"{name}_{ext}{'_gz' if gz else ''}"] = np.frombuffer(data, np.uint8)
                    f.unlink()
    np.savez_compressed(HERE / "writers.npz", **out)
    print(f"wrote {len(out)} arrays, {sum(v.nbytes for v in out.values())} bytes")


if __name__ == "__main__":
    main()
