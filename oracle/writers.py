"""CPU restatement of the reference's mesh writers (src/meshify.c:391-1019).

Test infrastructure only (the product encodes on the GPU,
nii2mesh_gb300/csrc/writers.cu): the GPU tests compare the product with it on
meshes larger than the fixtures, and bench.py times it as the CPU baseline of
the writer.  It is pinned against the reference's own files in
tests/golden/writers.npz (tests/test_oracle_golden.py).

Python's "%g" is correctly rounded with ties to even, as glibc's printf is;
gzip/zlib streams use zlib at level 6, what gzopen(fnm, "w") and compress()
use in the reference.
"""
import base64
import gzip
import re
import struct
import zlib

import numpy as np

FMT_MZ3, FMT_GII, FMT_FREESURFER, FMT_JSON, FMT_OFF, FMT_OBJ, FMT_PLY, FMT_STL, FMT_VTK = range(9)


def format_of(fnm):
    """strip_ext + the strstr chain of save_mesh (src/meshify.c:973-1019); -1 = append ".mz3"."""
    def ch(i):
        return fnm[i] if i < len(fnm) else "\0"

    p = len(fnm)   # from the terminating NUL back to a '.', '\\' or '/'
    while p > 0 and ch(p) not in ".\\/":
        p -= 1
    ext = fnm[p:] if (p > 0 and ch(p) == "." and fnm[p - 1] not in "\\/") else ""
    for fmt, keys in ((FMT_MZ3, (".mz3",)), (FMT_GII, (".gii",)), (FMT_FREESURFER, (".inflated", ".pial")),
                      (FMT_JSON, (".json",)), (FMT_OFF, (".off",)), (FMT_OBJ, (".obj",)), (FMT_PLY, (".ply",)),
                      (FMT_STL, (".stl",)), (FMT_VTK, (".vtk",))):
        if any(k in ext for k in keys):
            return fmt
    return -1


def _f32(pts):
    with np.errstate(over="ignore"):   # out-of-range doubles become +-inf, as the C cast does
        return np.ascontiguousarray(pts, np.float64).astype(np.float32)


def _tris(tris):
    return np.ascontiguousarray(tris, np.int32).reshape(-1, 3)


def mz3(tris, pts, gz=False):
    """save_mz3 (src/meshify.c:602-679): 16-byte header, int32 faces, float32 vertices (little-endian)."""
    t, p = _tris(tris), _f32(pts)
    body = struct.pack("<HHIII", 0x5A4D, 3, len(t), len(p), 0) + t.astype("<i4").tobytes() + p.astype("<f4").tobytes()
    return gzip.compress(body, 6, mtime=0) if gz else body


def gii(tris, pts, gz=False):
    """save_gii (src/meshify.c:819-930)."""
    t, p = _tris(tris), _f32(pts)

    def data(raw):
        return base64.b64encode(zlib.compress(raw, 6) if gz else raw).decode()

    enc = "GZipBase64Binary" if gz else "Base64Binary"

    def head(is_tri, dim0):
        s = ('   <DataArray  ArrayIndexingOrder="RowMajorOrder"\n'
             f'               DataType="{"NIFTI_TYPE_INT32" if is_tri else "NIFTI_TYPE_FLOAT32"}"\n'
             f'               Dim0="{dim0}"\n'
             '               Dim1="3"\n'
             '               Dimensionality="2"\n'
             f'               Encoding="{enc}"\n'
             '               Endian="LittleEndian"\n'
             '               ExternalFileName=""\n'
             '               ExternalFileOffset=""\n'
             f'               Intent="{"NIFTI_INTENT_TRIANGLE" if is_tri else "NIFTI_INTENT_POINTSET"}">\n'
             '      <MetaData>\n'
             '      </MetaData>\n')
        if not is_tri:
            s += ('      <CoordinateSystemTransformMatrix>\n'
                  '         <DataSpace><![CDATA[NIFTI_XFORM_UNKNOWN]]></DataSpace>\n'
                  '         <TransformedSpace><![CDATA[NIFTI_XFORM_UNKNOWN]]></TransformedSpace>\n'
                  '         <MatrixData>' + "".join(f"{v:.6f} " for v in np.eye(4).ravel()) + '</MatrixData>\n'
                  '      </CoordinateSystemTransformMatrix>\n')
        return s + '      <Data>'

    s = ('<?xml version="1.0" encoding="UTF-8"?>\n'
         '<!DOCTYPE GIFTI SYSTEM "http://www.nitrc.org/frs/download.php/115/gifti.dtd">\n'
         '<GIFTI Version="1.0"  NumberOfDataArrays="2">\n'
         '   <MetaData>\n'
         '      <MD>\n'
         '          <Name><![CDATA[nii2mesh-version]]></Name>\n'
         '          <Value><![CDATA[nii2mesh, 1 Jan 2022]]></Value>\n'
         '      </MD>\n'
         '   </MetaData>\n'
         '   <LabelTable/>\n')
    s += head(True, len(t)) + data(t.astype("<i4").tobytes()) + "</Data>\n   </DataArray>\n"
    s += head(False, len(p)) + data(p.astype("<f4").tobytes()) + "</Data>\n   </DataArray>\n</GIFTI>\n"
    return s.encode()


def freesurfer(tris, pts, stamp="created by niimath on Thu Jan  1 00:00:00 1970\n\n"):
    """save_freesurfer (src/meshify.c:418-459): big-endian counts, float32 vertices, int32 faces."""
    t, p = _tris(tris), _f32(pts)
    return (b"\xff\xff\xfe" + stamp.encode() + struct.pack(">ii", len(p), len(t)) + p.astype(">f4").tobytes() +
            t.astype(">i4").tobytes())


def _lines(fmt_v, fmt_t, tris, pts):
    p = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
    t = _tris(tris) + 1
    return "".join(fmt_v % tuple(r) for r in p.tolist()), "".join(fmt_t % tuple(r) for r in t.tolist())


def json_(tris, pts):
    """save_json (src/meshify.c:683-698)."""
    v, f = _lines("[%g,\t%g,\t%g],\n", "[%d,\t%d,\t%d],\n", tris, pts)
    return ("{\n\t\"_DataInfo_\":{\n\t\t\"JMeshVersion\":\"0.5\",\n\t\t\"Comment\":\"Created by nii2mesh\"\n\t},\n"
            "\t\"MeshVertex3\":[\n" + v + "\t],\n\t\"MeshTri3\":[\n" + f + "\t]\n}\n").encode()


def off(tris, pts):
    """save_off (src/meshify.c:700-711); faces are written 1-based like the reference."""
    v, f = _lines("%g %g %g\n", "%d %d %d\n", tris, pts)
    return (f"OFF\n{len(np.asarray(pts).reshape(-1, 3))}\t{len(_tris(tris))}\t0\n" + v + f).encode()


def obj(tris, pts):
    """save_obj (src/meshify.c:713-723)."""
    v, f = _lines("v %g %g %g\n", "f %d %d %d\n", tris, pts)
    return (v + f).encode()


def ply(tris, pts):
    """save_ply (src/meshify.c:764-817): binary little-endian, faces as (uint8 3, int32 x3) packed."""
    t, p = _tris(tris), _f32(pts)
    h = ("ply\nformat binary_little_endian 1.0\ncomment niimath\n"
         f"element vertex {len(p)}\nproperty float x\nproperty float y\nproperty float z\n"
         f"element face {len(t)}\nproperty list uchar int vertex_indices\nend_header\n").encode()
    faces = np.zeros(len(t), dtype=[("n", "u1"), ("i", "<i4", 3)])
    faces["n"] = 3
    faces["i"] = t
    return h + p.astype("<f4").tobytes() + faces.tobytes()


def stl(tris, pts):
    """save_stl (src/meshify.c:725-762): 80-byte header, count, 50-byte facets with zero normals."""
    t, p = _tris(tris), _f32(pts)
    fac = np.zeros(len(t), dtype=[("n", "<f4", 3), ("v", "<f4", (3, 3)), ("s", "<u2")])
    if len(t):
        fac["v"] = p[t]
    return b"\0" * 80 + struct.pack("<i", len(t)) + fac.tobytes()


def vtk(tris, pts):
    """save_vtk (src/meshify.c:932-971): legacy binary (big-endian) polydata."""
    t, p = _tris(tris), _f32(pts)
    polys = np.concatenate([np.full((len(t), 1), 3, np.int64), t], axis=1).astype(">u4")
    return (b"# vtk DataFile Version 3.0\nthis file was written using niimath\nBINARY\nDATASET POLYDATA\n" +
            f"POINTS {len(p)} float\n".encode() + p.astype(">f4").tobytes() +
            f"POLYGONS {len(t)} {4 * len(t)}\n".encode() + polys.tobytes())


def encode(fmt, tris, pts, gz=False, stamp=None):
    """The bytes save_mesh writes for format `fmt` (FMT_*)."""
    if fmt == FMT_MZ3:
        return mz3(tris, pts, gz)
    if fmt == FMT_GII:
        return gii(tris, pts, gz)
    if fmt == FMT_FREESURFER:
        return freesurfer(tris, pts, stamp) if stamp else freesurfer(tris, pts)
    return {FMT_JSON: json_, FMT_OFF: off, FMT_OBJ: obj, FMT_PLY: ply, FMT_STL: stl, FMT_VTK: vtk}[fmt](tris, pts)


def normalize(data):
    """Comparable form of a mesh file: a gzip body gunzipped, zlib-compressed
    GIfTI arrays decompressed (and re-encoded in base64), the FreeSurfer time
    stamp blanked.  Files that differ only in how they were deflated (or when
    they were written) normalize to the same bytes."""
    data = bytes(data)
    if data[:2] == b"\x1f\x8b":
        return gzip.decompress(data)
    if data[:3] == b"\xff\xff\xfe":
        return data[:3] + b"<stamp>" + data[data.index(b"\n\n", 3) + 2:]
    if data.startswith(b"<?xml") and b"GZipBase64Binary" in data:
        def plain(m):
            return b"<Data>" + base64.b64encode(zlib.decompress(base64.b64decode(m.group(1)))) + b"</Data>"
        return re.sub(rb"<Data>(.*?)</Data>", plain, data, flags=re.S)
    return data

