"""Mesh writers (save_mesh, src/meshify.c:984-1019) and the deflate streams on
the GPU, against the reference's own files (tests/golden/writers.npz, written
by its save_mesh) and against the oracle's restatement (oracle/writers.py) on
larger meshes.  Compressed files are compared after decompression (the deflate
search differs from zlib's; the bytes it encodes may not)."""
import gzip
import zlib
from pathlib import Path

import numpy as np
import pytest

from oracle import writers as W

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
WG = dict(np.load(GOLD / "writers.npz"))
EXTS = ["mz3", "gii", "inflated", "pial", "json", "off", "obj", "ply", "stl", "vtk", "xyz"]
WBITS = {0: -15, 1: 15, 2: 31}   # raw deflate, zlib, gzip


def _dev_bytes(data, offset=0):
    import torch
    buf = bytearray(offset) + bytearray(data) + bytearray(1)
    t = torch.frombuffer(buf, dtype=torch.uint8).cuda()
    torch.cuda.synchronize()
    return t, t.data_ptr() + offset


@pytest.mark.parametrize("case", ["sphere", "special", "empty"])
def test_encode_matches_reference_files(gpu, case):
    ctx = gpu.Context(0)
    t, p = WG[f"tris_{case}"], WG[f"pts_{case}"]
    for ext in EXTS:
        fmt = gpu.mesh_format_of(f"{case}.{ext}")
        assert fmt == W.format_of(f"{case}.{ext}")
        for gz in (False, True):
            want = WG[f"{case}_{ext}{'_gz' if gz else ''}"].tobytes()
            got = ctx.encode_mesh(gpu.FMT_MZ3 if fmt < 0 else fmt, t, p, gz)
            if gz and fmt in (gpu.FMT_MZ3, -1):
                assert got[:3] == b"\x1f\x8b\x08"
            assert W.normalize(got) == W.normalize(want), (case, ext, gz)


def test_save_mesh_writes_reference_files(gpu, tmp_path):
    """the drop-in save_mesh() and n2m_save_mesh write the same files as the
    reference's save_mesh, including the ".mz3" it appends to unknown names"""
    ctx = gpu.Context(0)
    t, p = WG["tris_sphere"], WG["pts_sphere"]
    for ext in EXTS:
        for gz in (False, True):
            want = W.normalize(WG[f"sphere_{ext}{'_gz' if gz else ''}"].tobytes())
            f1, f2 = tmp_path / f"a_{int(gz)}.{ext}", tmp_path / f"b_{int(gz)}.{ext}"
            assert gpu.save_mesh(f1, t, p, gz) == 0
            ctx.save_mesh(f2, t, p, gz)
            if ext == "xyz":
                assert not f1.exists() and not f2.exists()
                f1, f2 = Path(str(f1) + ".mz3"), Path(str(f2) + ".mz3")
            assert W.normalize(f1.read_bytes()) == want, (ext, gz)
            assert W.normalize(f2.read_bytes()) == want, (ext, gz)
    assert gpu.save_mesh(tmp_path / "missing_dir" / "x.mz3", t, p) == 1   # EXIT_FAILURE, like fopen failing


def test_device_mesh_matches_oracle(gpu):
    """a mesh straight from n2m_meshify_device (75k triangles, scanner-like
    coordinates after apply_sform) in every format, against the oracle"""
    import torch
    from nii2mesh_gb300 import synth
    ctx = gpu.Context(0)
    vol = synth.ct512(seed=3, n=96, count=14)
    t, p, _ = ctx.meshify(vol, 300.0, gpu.MC33, True, False, False)
    d = torch.from_numpy(vol).cuda()
    dt, dp, nt, np_, _ = ctx.meshify_device(d.data_ptr(), (96, 96, 96), 300.0, gpu.MC33, True, False, False)
    assert (nt, np_) == (len(t), len(p)) and nt > 20000
    for fmt in range(9):
        for gz in (False, True):
            got = ctx.encode_mesh_device(fmt, dt, dp, nt, np_, gz)
            assert W.normalize(got) == W.normalize(W.encode(fmt, t, p, gz)), (fmt, gz)
    # awkward coordinates for %g: an sform to millimetres
    t2, p2 = gpu.apply_sform(p, t, [0.9375, 0.0123, 0.0, -90.5], [0.0, 1.1, 0.0207, -126.25], [0.0, -0.004, 1.2, -72.0])
    for fmt in (gpu.FMT_OBJ, gpu.FMT_OFF, gpu.FMT_JSON):
        assert ctx.encode_mesh(fmt, t2, p2) == W.encode(fmt, t2, p2), fmt


def test_deflate_round_trips(gpu):
    """raw / zlib / gzip streams decompress (zlib) to the input: empty, one
    byte, chunk-boundary sizes, incompressible data (stored blocks), zeros
    (258-byte matches), text, mesh bytes; unaligned source pointers"""
    ctx = gpu.Context(0)
    rng = np.random.default_rng(3)
    t, p = WG["tris_sphere"], WG["pts_sphere"]
    datas = {
        "empty": b"",
        "one": b"\x07",
        "three": b"abc",
        "zeros": bytes(1 << 20),
        "random": rng.bytes(100_003),
        "text": b"the quick brown fox jumps over the lazy dog " * 3000,
        "chunk_edge_lo": rng.integers(0, 4, 32768, dtype=np.uint8).tobytes(),
        "chunk_edge_hi": rng.integers(0, 4, 3 * 32768 + 1, dtype=np.uint8).tobytes(),
        "mesh": W.mz3(t, p) * 40,
        "runs": np.repeat(rng.integers(0, 256, 5000, dtype=np.uint8), rng.integers(1, 300, 5000)).tobytes(),
    }
    for name, data in datas.items():
        for container in (0, 1, 2):
            for off in (0, 1, 3):
                keep, ptr = _dev_bytes(data, off)
                out = ctx.deflate_device(ptr, len(data), container)
                assert zlib.decompress(out, WBITS[container]) == data, (name, container, off)
                nblocks = max(1, (len(data) + 16383) // 16384)   # 16 KB blocks, 5 bytes each when stored
                assert len(out) <= len(data) + 5 * nblocks + 18, (name, container)
    gz = ctx.deflate_device(_dev_bytes(datas["text"])[1], len(datas["text"]), 2)
    assert gzip.decompress(gz) == datas["text"] and len(gz) < len(datas["text"]) // 20


def test_deflate_ratio_close_to_zlib(gpu):
    """on mesh bytes (the mz3 body of a 220k-triangle mesh) the GPU stream is
    at most 8 % larger than zlib's at level 6, the level gzopen uses"""
    from nii2mesh_gb300 import synth
    ctx = gpu.Context(0)
    vol = synth.ct512(seed=8, n=128, count=30)
    t, p, _ = ctx.meshify(vol, 300.0, gpu.MC33, True, False, False)
    body = W.mz3(t, p)
    keep, ptr = _dev_bytes(body)
    ours = ctx.deflate_device(ptr, len(body), 2)
    ref = zlib.compress(body, 6)
    assert gzip.decompress(ours) == body
    assert len(ours) <= 1.08 * len(ref), (len(ours), len(ref), len(body))
