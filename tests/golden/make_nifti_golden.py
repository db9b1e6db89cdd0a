#!/usr/bin/env python3
"""Generate the NIfTI voxel-cast fixtures (load_nii, src/nii2mesh.c:53-175)
from the reference nii2mesh itself: small .nii files of the four datatypes it
reads, with and without scl_slope/scl_inter, loaded by the reference's own
load_nii (oracle/_ref/libn2m_ref_cli.so, built from its sources).

Run where the reference tree exists:  python tests/golden/make_nifti_golden.py

Writes nifti.npz: for case k, raw{k} (the voxels as stored), meta{k}
[datatype, scl_slope, scl_inter] (float64) and out{k} (the reference's float32
volume).
"""
import ctypes as C
import struct
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
from oracle.refpath import reference_src  # noqa: E402

SRC = reference_src()   # N2M_REFERENCE, or a `reference` checkout beside this repository
DT = {np.uint8: 2, np.int16: 4, np.float32: 16, np.uint16: 512}


def nifti_bytes(raw, slope, inter):
    """a single-file NIfTI-1 (.nii): 348-byte header, 4 bytes of extension flag, voxels"""
    nz, ny, nx = raw.shape
    h = bytearray(352)
    struct.pack_into("<i", h, 0, 348)
    struct.pack_into("<8h", h, 40, 3, nx, ny, nz, 1, 1, 1, 1)
    struct.pack_into("<h", h, 70, DT[raw.dtype.type])
    struct.pack_into("<h", h, 72, raw.dtype.itemsize * 8)
    struct.pack_into("<8f", h, 76, 1, 1, 1, 1, 1, 1, 1, 1)
    struct.pack_into("<f", h, 108, 352.0)
    struct.pack_into("<f", h, 112, slope)
    struct.pack_into("<f", h, 116, inter)
    h[344:348] = b"n+1\0"
    return bytes(h) + np.ascontiguousarray(raw).tobytes()


def cases():
    rng = np.random.default_rng(91)
    shape = (12, 17, 23)
    n = int(np.prod(shape))
    return [
        (rng.integers(0, 256, n).astype(np.uint8).reshape(shape), 0.0, 0.0),        # slope 0 means 1
        (rng.integers(0, 256, n).astype(np.uint8).reshape(shape), 0.37, -12.5),
        (rng.integers(-32768, 32768, n).astype(np.int16).reshape(shape), 1.0, -1024.0),
        (rng.integers(-32768, 32768, n).astype(np.int16).reshape(shape), 0.0123, 3.75),
        (rng.integers(0, 65536, n).astype(np.uint16).reshape(shape), 2.5, 0.0),
        (rng.integers(0, 65536, n).astype(np.uint16).reshape(shape), 1.0e-3, -7.0),
        (rng.normal(0, 1000, n).astype(np.float32).reshape(shape), 1.0, 0.0),
        (rng.normal(0, 1000, n).astype(np.float32).reshape(shape), 0.3, 100.125),
    ]


def main():
    subprocess.run(["sh", str(ROOT / "oracle" / "build_ref.sh"), str(SRC)], check=True, stdout=subprocess.DEVNULL)
    lib = C.CDLL(str(ROOT / "oracle" / "_ref" / "libn2m_ref_cli.so"))
    lib.load_nii.restype = C.c_void_p
    lib.load_nii.argtypes = [C.c_char_p, C.c_void_p]
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    out = {}
    with tempfile.TemporaryDirectory() as td:
        for k, (raw, slope, inter) in enumerate(cases()):
            f = Path(td) / f"c{k}.nii"
            f.write_bytes(nifti_bytes(raw, slope, inter))
            hdr = C.create_string_buffer(348)
            p = lib.load_nii(str(f).encode(), hdr)
            assert p, f"load_nii failed on case {k}"
            vol = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_float)), shape=(raw.size,)).copy()
            libc.free(p)
            out[f"raw{k}"] = raw
            out[f"meta{k}"] = np.array([DT[raw.dtype.type], slope, inter], np.float64)
            out[f"out{k}"] = vol.reshape(raw.shape)
    np.savez_compressed(HERE / "nifti.npz", **out)
    print(f"wrote {len(cases())} cases")


if __name__ == "__main__":
    main()
