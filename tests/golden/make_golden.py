#!/usr/bin/env python3
"""Generate the golden fixtures from the reference nii2mesh itself.

Run where the reference tree exists (it builds oracle/_ref from the
reference's own sources):  python tests/golden/make_golden.py

Writes
  inputs.npz    the small seeded input volumes (stored, so that every machine
                meshes bit-identical inputs)
  golden.json   reference results: counts and SHA-256 of canonical meshes,
                label volumes, thresholds, self-test known answers, and the
                counts the reference's nii2mesh program writes for the
                self-test volumes and data/bet.nii.gz (with each command)
  hc.npz        reference HC-smoothed vertices (compared with a tolerance)
"""
import gzip
import hashlib
import json
import re
import struct
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from nii2mesh_gb300 import synth  # noqa: E402
from oracle.oracle import MC33, MC_CLASSIC_TABLE, OLDCUBES, Reference, canonical  # noqa: E402

from oracle.refpath import reference_src  # noqa: E402

SRC = reference_src()   # N2M_REFERENCE, or a `reference` checkout beside this repository
OPTION_SETS = [(True, True, False), (True, False, False), (False, False, False), (True, True, True),
               (False, True, True), (True, False, True)]


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


def inputs():
    rng = np.random.default_rng(40)
    blobs = np.zeros((40, 40, 40), np.float32)
    z, y, x = np.ogrid[0:40, 0:40, 0:40]
    for _ in range(14):
        c = rng.uniform(4, 36, 3)
        r = rng.uniform(2, 7)
        d = np.sqrt((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2)
        blobs[d <= r] = 1
        if rng.random() < 0.5:
            blobs[d <= r * 0.5] = 0   # hollow: a bubble
    return {
        "sphere48": synth.spheres(n=48, count=6, rmin=5, rmax=11, cmin=10, cmax=38, seed=10),
        "ct48": synth.ct512(seed=5, n=48, count=6),
        "brain_small": synth.brain()[::4, ::4, ::4].astype(np.float32),
        "blobs40": blobs,
    }


def run_cli(d, name, obj, src, variant, args):
    """Run the reference's nii2mesh program (oracle/_ref: nii2mesh = `make lewiner`,
    nii2mesh_classic = the default oldcubes build) and read the triangle and vertex
    counts from the header of the .mz3 it writes (gzip, the default quality)."""
    exe = "nii2mesh_classic" if variant == OLDCUBES else "nii2mesh"
    opts = (["-o", "1"] if variant == MC_CLASSIC_TABLE else []) + list(args)
    out = Path(d) / "cli_out.mz3"
    subprocess.run([str(ROOT / "oracle" / "_ref" / exe), str(src), *opts, str(out)], check=True, cwd=d,
                   capture_output=True)
    raw = out.read_bytes()
    if raw[:2] == b"\x1f\x8b":
        raw = gzip.decompress(raw)
    sig, _, nface, nvert, _ = struct.unpack("<HHIII", raw[:16])
    assert sig == 23117, "not an mz3 file"
    out.unlink()
    return {"input": name, "object": obj, "variant": variant, "ntri": nface, "nvert": nvert,
            "command": " ".join([exe, Path(src).name if obj is None else f"{obj}.nii", *opts, "out.mz3"])}


def main():
    subprocess.run(["sh", str(ROOT / "oracle" / "build_ref.sh"), str(SRC)], check=True, stdout=subprocess.DEVNULL)
    vols = inputs()
    np.savez_compressed(HERE / "inputs.npz", **vols)
    rl, rc = Reference(False), Reference(True)
    g = {"meshify": [], "bwlabel": [], "threshold": {}, "selftest": {}, "marching_cubes": [], "sform": []}
    isos = {"sphere48": 50.0, "ct48": 300.0, "brain_small": None, "blobs40": 0.5}
    for name in ("sphere48", "ct48", "brain_small", "blobs40"):
        vol = vols[name]
        iso = isos[name] if isos[name] is not None else rl.set_threshold(vol, 2)
        for variant, ref in ((MC33, rl), (MC_CLASSIC_TABLE, rl), (OLDCUBES, rc)):
            for flags in OPTION_SETS:
                m = ref.meshify(vol, iso, variant, *flags)
                e = {"input": name, "iso": iso, "variant": variant, "pre_smooth": flags[0], "only_largest": flags[1],
                     "fill_bubbles": flags[2]}
                if m is None:
                    e["result"] = None
                else:
                    e.update(nvert=len(m[1]), ntri=len(m[0]), sha256=mesh_hash(*m))
                g["meshify"].append(e)
        for mode in (1, 2, 3):
            g["threshold"][f"{name}:{mode}"] = rl.set_threshold(vol, mode)
    # HC smoothing of a reference mesh, 5 iterations, edges locked (nii2mesh -s 5)
    t, p = rl.meshify(vols["sphere48"], 50.0, MC33, True, False, False)
    hc = {"tris": t, "pts": p}
    for it in (1, 5, 20):
        hc[f"smoothed_{it}"] = rl.laplacian_smoothHC(p, t, 0.1, 0.5, it, True)
    # an open mesh (border vertices): drop a band of triangles
    keep = np.ones(len(t), bool)
    keep[::7] = False
    hc["open_tris"] = t[keep]
    hc["open_smoothed_5"] = rl.laplacian_smoothHC(p, t[keep], 0.1, 0.5, 5, True)
    np.savez_compressed(HERE / "hc.npz", **hc)
    # bwlabel on the blob volume
    for conn in (6, 18, 26):
        for ol, fb in ((False, False), (True, False), (False, True), (True, True)):
            lab, n = rl.bwlabel(vols["blobs40"], conn, ol, fb)
            g["bwlabel"].append({"conn": conn, "only_largest": ol, "fill_bubbles": fb, "n": n,
                                 "sha256": raw_hash(lab.astype(np.float32))})
    # marchingCubes() on an explicit box: the un-welded mesh in the reference's order
    v = vols["sphere48"]
    for lo, hi in (((3, 4, 5), (40, 44, 47)), ((0, 0, 0), (48, 48, 48)), ((10, 0, 7), (48, 30, 48))):
        for omc in (0, 1):
            m = rl.marching_cubes(v, lo, hi, omc, 50.0)
            g["marching_cubes"].append({"lo": lo, "hi": hi, "original_mc": omc, "nvert": len(m[1]), "ntri": len(m[0]),
                                        "sha256": raw_hash(m[0].astype(np.int32), m[1].astype(np.float64))})
    # apply_sform with a mirrored affine (negative determinant flips winding)
    for rows in (((1, 0, 0, 0), (0, 1, 0, 0), (0, 0, 1, 0)), ((-0.9, 0.1, 0, 90.5), (0.05, 1.1, 0.02, -126), (0, 0.1, 1.2, -72.25))):
        tt, pp = rl.apply_sform(p, t, *rows)
        g["sform"].append({"rows": rows, "sha256": raw_hash(tt.astype(np.int32), pp.astype(np.float64))})
    # the reference's MC self-test: known answers and the generated fields
    with tempfile.TemporaryDirectory() as d:
        out = subprocess.run([str(ROOT / "oracle" / "_ref" / "mctest")], cwd=d, capture_output=True, text=True).stdout
        counts = [tuple(map(int, x)) for x in re.findall(r"output mesh vert: (\d+) tris: (\d+)", out)]
        for obj in range(10):
            raw = (Path(d) / f"{obj}.nii").read_bytes()
            field = np.frombuffer(raw, np.float32, 60 ** 3, 352)
            g["selftest"][str(obj)] = {"nvert": counts[obj][0], "ntri": counts[obj][1], "field_sha256": raw_hash(field)}
        # whole-program known answers: the reference's nii2mesh program run on the self-test
        # volumes it wrote (N.nii) and on its own data/bet.nii.gz
        g["cli"] = []
        for obj in (0, 1, 2, 5, 8):
            for variant in ((MC33, MC_CLASSIC_TABLE, OLDCUBES) if obj == 8 else (MC33,)):
                g["cli"].append(run_cli(d, "selftest", obj, Path(d) / f"{obj}.nii", variant,
                                        ["-p", "0", "-l", "0", "-b", "0", "-r", "1", "-i", "0.001"]))
        bet = SRC.parent / "data" / "bet.nii.gz"
        for variant in (MC33, MC_CLASSIC_TABLE, OLDCUBES):
            g["cli"].append(run_cli(d, "bet.nii.gz", None, bet, variant, ["-r", "1"]))
    (HERE / "golden.json").write_text(json.dumps(g, indent=1))
    print("wrote", HERE / "golden.json")


if __name__ == "__main__":
    main()
