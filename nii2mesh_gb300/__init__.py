"""nii2mesh_gb300 — GB300-native volume->mesh path of nii2mesh.

The product is libn2m_gpu.so (C ABI in include/n2m_gpu.h): the reference's own
entry points (meshify, laplacian_smoothHC, marchingCubes, bwlabel,
apply_sform) plus n2m_* calls with explicit status codes, device-resident
variants, the adjoint and the batched atlas.  This module is a thin numpy /
torch front end over that ABI, mirroring the reference's functions
(src/meshify.h:9, src/quadric.h:7, src/MarchingCubes.h:19, src/bwlabel.h:10):
same argument meaning, same failure behaviour (None where the reference
returns EXIT_FAILURE).

Volumes are numpy float32 arrays shaped (nz, ny, nx) — x fastest, exactly the
reference's memory layout.  Meshes are (tris int32 (nt,3), pts float64 (np,3)).
"""
import ctypes as C
import queue
import threading
import weakref

import numpy as np

from . import _lib
from ._lib import AtlasMesh, N2MError, Options, Report, vec3d, vec3i

MC33, CLASSIC_TABLE, OLDCUBES = 0, 1, 2
# NIfTI datatype codes of the voxel types load_nii reads (src/nii2mesh.c:114-117)
_NIFTI_DT = {np.dtype(np.uint8): 2, np.dtype(np.int16): 4, np.dtype(np.float32): 16, np.dtype(np.uint16): 512}
ATLAS_BATCHED, ATLAS_LOOP = 0, 1
# mesh file formats (n2m_mesh_format) and deflate containers
FMT_MZ3, FMT_GII, FMT_FREESURFER, FMT_JSON, FMT_OFF, FMT_OBJ, FMT_PLY, FMT_STL, FMT_VTK = range(9)
DEFLATE_RAW, DEFLATE_ZLIB, DEFLATE_GZIP = 0, 1, 2

__all__ = ["Context", "meshify", "laplacian_smoothHC", "marching_cubes", "bwlabel", "apply_sform", "set_threshold",
           "save_mesh", "mesh_format_of", "N2MError",
           "MC33", "CLASSIC_TABLE", "OLDCUBES", "lib"]


def lib():
    return _lib.load()


def _vol(img):
    a = np.ascontiguousarray(img, dtype=np.float32)
    if a.ndim != 3:
        raise ValueError("volume must be 3-D (nz, ny, nx)")
    return a


class _Reaper:
    """Frees large result buffers on a background thread.  Releasing a
    pre-faulted mesh of a few hundred MB unmaps every page (~1.4 ms for the
    170 MB of a 512^3 CT mesh); done here it overlaps the caller's next call
    instead of blocking the thread that dropped the arrays."""

    BIG = 8 << 20

    def __init__(self):
        self.q = None
        self.lock = threading.Lock()

    def free(self, L, addr, nbytes):
        if nbytes < self.BIG:
            L.libc_free(addr)
            return
        with self.lock:
            if self.q is None:
                self.q = queue.SimpleQueue()
                threading.Thread(target=self._run, args=(L, self.q), name="n2m-free", daemon=True).start()
        self.q.put(addr)

    @staticmethod
    def _run(L, q):
        while True:
            L.libc_free(q.get())   # ctypes releases the GIL for the call


_reaper = _Reaper()


def _owned(L, ptr, n, ctype, dtype):
    """numpy (n, 3) view of library-malloc'd memory, freed with libc free()
    once the last array referring to it is gone (no copy of the mesh)."""
    addr = ptr.value if isinstance(ptr, C.c_void_p) else ptr
    if not n:
        L.libc_free(addr)
        return np.zeros((0, 3), dtype)
    buf = (ctype * (3 * n)).from_address(addr)
    weakref.finalize(buf, _reaper.free, L, addr, 3 * n * C.sizeof(ctype))
    return np.frombuffer(buf, dtype).reshape(n, 3)


def _take(L, tp, pp, nt, np_):
    return _owned(L, tp, nt, C.c_int, np.int32), _owned(L, pp, np_, C.c_double, np.float64)


class Context:
    """A CUDA stream + device workspace (n2m_context)."""

    def __init__(self, device=0):
        L = _lib.load()
        self._L = L
        h = C.c_void_p()
        _lib.check(L.n2m_context_create(C.byref(h), device), "n2m_context_create")
        self.h = h

    def close(self):
        if self.h:
            self._L.n2m_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self):
        return self._L.n2m_context_stream(self.h)

    @staticmethod
    def _opts(iso, cubes, pre_smooth, only_largest, fill_bubbles, post_smooth, verbose):
        return Options(int(cubes), float(iso), bool(pre_smooth), bool(only_largest), bool(fill_bubbles),
                       int(post_smooth), bool(verbose))

    def meshify(self, img, iso, cubes=MC33, pre_smooth=True, only_largest=True, fill_bubbles=False, post_smooth=0,
                verbose=False):
        """Host volume in, host mesh out (n2m_meshify).  Raises N2MError."""
        a = _vol(img)
        nz, ny, nx = a.shape
        dims = (C.c_int * 3)(nx, ny, nz)
        o = self._opts(iso, cubes, pre_smooth, only_largest, fill_bubbles, post_smooth, verbose)
        tp, pp, nt, np_ = C.c_void_p(), C.c_void_p(), C.c_int(), C.c_int()
        rep = Report()
        _lib.check(self._L.n2m_meshify(self.h, a.ctypes.data, dims, C.byref(o), C.byref(tp), C.byref(pp), C.byref(nt),
                                       C.byref(np_), C.byref(rep)), "n2m_meshify")
        t, p = _take(self._L, tp, pp, nt.value, np_.value)
        return t, p, rep.as_dict()

    def meshify_into(self, img, tris_out, pts_out, iso, cubes=MC33, pre_smooth=True, only_largest=True,
                     fill_bubbles=False, post_smooth=0, verbose=False):
        """n2m_meshify_into: the mesh goes into caller-owned arrays (int32 (T, 3)
        and float64 (V, 3), C-contiguous; pinned memory copies fastest) that can
        be reused from call to call.  Returns (nt, np, report); the mesh is
        tris_out[:nt], pts_out[:np].  Raises N2MError (N2M_ERR_TOO_LARGE, with
        .needed = (nt, np)) when it does not fit."""
        a = _vol(img)
        nz, ny, nx = a.shape
        for arr, dt in ((tris_out, np.int32), (pts_out, np.float64)):
            if arr.dtype != dt or arr.ndim != 2 or arr.shape[1] != 3 or not arr.flags.c_contiguous:
                raise ValueError("outputs must be C-contiguous int32 (T, 3) and float64 (V, 3) arrays")
        o = self._opts(iso, cubes, pre_smooth, only_largest, fill_bubbles, post_smooth, verbose)
        nt, np_ = C.c_int(), C.c_int()
        rep = Report()
        st = self._L.n2m_meshify_into(self.h, a.ctypes.data, (C.c_int * 3)(nx, ny, nz), C.byref(o),
                                      tris_out.ctypes.data, len(tris_out), pts_out.ctypes.data, len(pts_out),
                                      C.byref(nt), C.byref(np_), C.byref(rep))
        if st != 0:
            try:
                _lib.check(st, "n2m_meshify_into")
            except N2MError as e:
                e.needed = (nt.value, np_.value)
                raise
        return nt.value, np_.value, rep.as_dict()

    def meshify_device(self, d_img_ptr, dims_xyz, iso, cubes=MC33, pre_smooth=True, only_largest=True,
                       fill_bubbles=False, post_smooth=0):
        """Device volume (pointer) in; mesh stays on the device.  Returns
        (d_tris_ptr, d_pts_ptr, nt, np, report)."""
        dims = (C.c_int * 3)(*dims_xyz)
        o = self._opts(iso, cubes, pre_smooth, only_largest, fill_bubbles, post_smooth, False)
        tp, pp, nt, np_ = C.c_void_p(), C.c_void_p(), C.c_int(), C.c_int()
        rep = Report()
        _lib.check(self._L.n2m_meshify_device(self.h, C.c_void_p(d_img_ptr), dims, C.byref(o), C.byref(tp), C.byref(pp),
                                              C.byref(nt), C.byref(np_), C.byref(rep)), "n2m_meshify_device")
        return tp.value, pp.value, nt.value, np_.value, rep.as_dict()


    def meshify_typed(self, raw, scl_slope, scl_inter, iso, cubes=MC33, pre_smooth=True, only_largest=True,
                      fill_bubbles=False, post_smooth=0, verbose=False):
        """n2m_meshify_typed: raw NIfTI voxels (uint8, int16, uint16 or float32
        numpy array shaped (nz, ny, nx)) sent as they are and cast on the device
        as load_nii does (src/nii2mesh.c:160-175)."""
        a = np.ascontiguousarray(raw)
        if a.ndim != 3 or a.dtype not in _NIFTI_DT:
            raise ValueError("raw must be a 3-D uint8/int16/uint16/float32 array")
        nz, ny, nx = a.shape
        o = self._opts(iso, cubes, pre_smooth, only_largest, fill_bubbles, post_smooth, verbose)
        tp, pp, nt, np_ = C.c_void_p(), C.c_void_p(), C.c_int(), C.c_int()
        rep = Report()
        _lib.check(self._L.n2m_meshify_typed(self.h, a.ctypes.data, _NIFTI_DT[a.dtype], float(scl_slope), float(scl_inter),
                                             (C.c_int * 3)(nx, ny, nz), C.byref(o), C.byref(tp), C.byref(pp),
                                             C.byref(nt), C.byref(np_), C.byref(rep)), "n2m_meshify_typed")
        t, p = _take(self._L, tp, pp, nt.value, np_.value)
        return t, p, rep.as_dict()

    def cast_voxels_device(self, d_raw_ptr, dtype, scl_slope, scl_inter, nvox, d_out_ptr):
        """n2m_cast_voxels_device: device raw voxels -> device float32."""
        _lib.check(self._L.n2m_cast_voxels_device(self.h, C.c_void_p(d_raw_ptr), _NIFTI_DT[np.dtype(dtype)],
                                                  float(scl_slope), float(scl_inter), int(nvox), C.c_void_p(d_out_ptr)),
                   "n2m_cast_voxels_device")

    def set_threshold(self, img, mode=2):
        """Otsu isolevel of a host volume (n2m_set_threshold); mode 1 dark, 2 medium, 3 bright."""
        a = np.ascontiguousarray(img, dtype=np.float32)
        out = C.c_float()
        _lib.check(self._L.n2m_set_threshold(self.h, a.ctypes.data, a.size, int(mode), C.byref(out)), "n2m_set_threshold")
        return out.value

    def set_threshold_device(self, d_img_ptr, nvox, mode=2):
        """Otsu isolevel of a device volume (n2m_set_threshold_device)."""
        out = C.c_float()
        _lib.check(self._L.n2m_set_threshold_device(self.h, C.c_void_p(d_img_ptr), int(nvox), int(mode), C.byref(out)),
                   "n2m_set_threshold_device")
        return out.value

    def _bytes(self, ptr, n):
        """bytes of library-malloc'd memory, released afterwards"""
        try:
            return C.string_at(ptr, n) if n else b""
        finally:
            self._L.libc_free(ptr)

    def encode_mesh(self, fmt, tris, pts, gz=False):
        """The file save_mesh() writes in format `fmt` (FMT_* or a file name),
        encoded on the GPU, as bytes (n2m_encode_mesh)."""
        if isinstance(fmt, str):
            fmt = mesh_format_of(fmt)
        t = np.ascontiguousarray(tris, dtype=np.int32)
        p = np.ascontiguousarray(pts, dtype=np.float64)
        out, n = C.c_void_p(), C.c_size_t()
        _lib.check(self._L.n2m_encode_mesh(self.h, int(fmt), t.ctypes.data, p.ctypes.data, len(t), len(p), int(gz),
                                           C.byref(out), C.byref(n)), "n2m_encode_mesh")
        return self._bytes(out, n.value)

    def encode_mesh_device(self, fmt, d_tris_ptr, d_pts_ptr, ntri, npt, gz=False):
        """encode_mesh of a mesh in device memory (n2m_encode_mesh_device)."""
        if isinstance(fmt, str):
            fmt = mesh_format_of(fmt)
        out, n = C.c_void_p(), C.c_size_t()
        _lib.check(self._L.n2m_encode_mesh_device(self.h, int(fmt), C.c_void_p(d_tris_ptr), C.c_void_p(d_pts_ptr),
                                                  int(ntri), int(npt), int(gz), C.byref(out), C.byref(n)),
                   "n2m_encode_mesh_device")
        return self._bytes(out, n.value)

    def encode_mesh_to_device(self, fmt, d_tris_ptr, d_pts_ptr, ntri, npt, gz=False):
        """encode_mesh leaving the bytes in device memory (n2m_encode_mesh_to_device):
        returns (device pointer, length), valid until the next call on this context."""
        if isinstance(fmt, str):
            fmt = mesh_format_of(fmt)
        out, n = C.c_void_p(), C.c_size_t()
        _lib.check(self._L.n2m_encode_mesh_to_device(self.h, int(fmt), C.c_void_p(d_tris_ptr), C.c_void_p(d_pts_ptr),
                                                     int(ntri), int(npt), int(gz), C.byref(out), C.byref(n)),
                   "n2m_encode_mesh_to_device")
        return out.value, n.value

    def save_mesh(self, fnm, tris, pts, gz=False):
        """save_mesh() with a status (n2m_save_mesh)."""
        t = np.ascontiguousarray(tris, dtype=np.int32)
        p = np.ascontiguousarray(pts, dtype=np.float64)
        _lib.check(self._L.n2m_save_mesh(self.h, str(fnm).encode(), t.ctypes.data, p.ctypes.data, len(t), len(p),
                                         int(gz)), "n2m_save_mesh")

    def save_mesh_device(self, fnm, d_tris_ptr, d_pts_ptr, ntri, npt, gz=False):
        """save_mesh() of a mesh in device memory (n2m_save_mesh_device)."""
        _lib.check(self._L.n2m_save_mesh_device(self.h, str(fnm).encode(), C.c_void_p(d_tris_ptr), C.c_void_p(d_pts_ptr),
                                                int(ntri), int(npt), int(gz)), "n2m_save_mesh_device")

    def deflate_device(self, d_ptr, nbytes, container=DEFLATE_GZIP):
        """Deflate nbytes of device memory (n2m_deflate_device) -> bytes."""
        out, n = C.c_void_p(), C.c_size_t()
        _lib.check(self._L.n2m_deflate_device(self.h, C.c_void_p(d_ptr), int(nbytes), int(container), C.byref(out),
                                              C.byref(n)), "n2m_deflate_device")
        return self._bytes(out, n.value)

    def atlas(self, labels, cubes=MC33, pre_smooth=True, only_largest=True, fill_bubbles=True, post_smooth=5,
              mode=ATLAS_BATCHED):
        """Mesh every label of an int16 label volume (n2m_atlas).  Returns a
        list of (label, status, tris, pts) — tris local to each mesh."""
        a = np.ascontiguousarray(labels, dtype=np.int16)
        nz, ny, nx = a.shape
        o = self._opts(0.5, cubes, pre_smooth, only_largest, fill_bubbles, post_smooth, False)
        nm = C.c_int()
        mp, pp, tp = C.c_void_p(), C.c_void_p(), C.c_void_p()
        npts, ntri = C.c_int64(), C.c_int64()
        _lib.check(self._L.n2m_atlas(self.h, a.ctypes.data, (C.c_int * 3)(nx, ny, nz), C.byref(o), int(mode),
                                     C.byref(nm), C.byref(mp), C.byref(pp), C.byref(tp), C.byref(npts),
                                     C.byref(ntri)), "n2m_atlas")
        ms = C.cast(mp, C.POINTER(AtlasMesh))
        pts = np.ctypeslib.as_array(C.cast(pp, C.POINTER(C.c_double)), shape=(max(npts.value, 1), 3))[:npts.value].copy()
        tri = np.ctypeslib.as_array(C.cast(tp, C.POINTER(C.c_int)), shape=(max(ntri.value, 1), 3))[:ntri.value].copy()
        out = []
        for i in range(nm.value):
            m = ms[i]
            out.append((m.label, m.status, tri[m.tri_offset:m.tri_offset + m.ntri],
                        pts[m.vert_offset:m.vert_offset + m.nvert]))
        for ptr in (mp, pp, tp):
            self._L.libc_free(ptr)
        return out

    def atlas_device(self, d_labels_ptr, dims_xyz, cubes=MC33, pre_smooth=True, only_largest=True, fill_bubbles=True,
                     post_smooth=5, mode=ATLAS_BATCHED):
        """Device label volume in; meshes stay on the device.  Returns
        (number of meshes, total vertices, total triangles, report)."""
        o = self._opts(0.5, cubes, pre_smooth, only_largest, fill_bubbles, post_smooth, False)
        nm = C.c_int()
        mp = C.POINTER(AtlasMesh)()
        pp, tp = C.c_void_p(), C.c_void_p()
        npts, ntri = C.c_int64(), C.c_int64()
        rep = Report()
        _lib.check(self._L.n2m_atlas_device(self.h, C.c_void_p(d_labels_ptr), (C.c_int * 3)(*dims_xyz), C.byref(o),
                                            int(mode), C.byref(nm), C.byref(mp), C.byref(pp), C.byref(tp),
                                            C.byref(npts), C.byref(ntri), C.byref(rep)), "n2m_atlas_device")
        ok = sum(1 for i in range(nm.value) if mp[i].status == 0)
        return nm.value, ok, npts.value, ntri.value, rep.as_dict()


# ---- the reference's entry points, through the drop-in C symbols -----------------
def meshify(img, isolevel, original_mc=0, pre_smooth=True, only_largest=True, fill_bubbles=False, verbose=False,
            oldcubes=False):
    """meshify() (src/meshify.h:9).  Returns (tris, pts) or None on failure."""
    L = _lib.load()
    a = _vol(img)
    nz, ny, nx = a.shape
    dims = (C.c_short * 3)(nx, ny, nz)
    tp, pp, nt, np_ = C.c_void_p(), C.c_void_p(), C.c_int(), C.c_int()
    prev = L.n2m_set_oldcubes(1 if oldcubes else 0)
    try:
        r = L.meshify(a.ctypes.data, dims, int(original_mc), float(isolevel), C.byref(tp), C.byref(pp), C.byref(nt),
                      C.byref(np_), pre_smooth, only_largest, fill_bubbles, verbose)
    finally:
        L.n2m_set_oldcubes(prev)
    if r != 0:
        return None
    return _take(L, tp, pp, nt.value, np_.value)


def laplacian_smoothHC(pts, tris, alpha=0.1, beta=0.5, iters=1, lock_edges=True):
    """laplacian_smoothHC() (src/quadric.h:7); returns the smoothed vertices."""
    L = _lib.load()
    p = np.ascontiguousarray(pts, dtype=np.float64).copy()
    t = np.ascontiguousarray(tris, dtype=np.int32)
    L.laplacian_smoothHC(p.ctypes.data, t.ctypes.data, len(p), len(t), alpha, beta, iters, lock_edges)
    return p


def marching_cubes(img, lo, hi, isolevel, original_mc=0, oldcubes=False):
    """marchingCubes() (src/MarchingCubes.h:19): mesh of the padded box lo..hi
    before any weld.  Returns (tris, pts) or None."""
    L = _lib.load()
    a = _vol(img)
    nz, ny, nx = a.shape
    dims = (C.c_short * 3)(nx, ny, nz)
    tp, pp, nv, nt = C.c_void_p(), C.c_void_p(), C.c_int(), C.c_int()
    prev = L.n2m_set_oldcubes(1 if oldcubes else 0)
    try:
        r = L.marchingCubes(a.ctypes.data, dims, (C.c_int * 3)(*lo), (C.c_int * 3)(*hi), int(original_mc),
                            float(isolevel), C.byref(pp), C.byref(tp), C.byref(nv), C.byref(nt))
    finally:
        L.n2m_set_oldcubes(prev)
    if r != 0:
        return None
    return _take(L, tp, pp, nt.value, nv.value)


def bwlabel(img, conn=18, only_largest=False, fill_bubbles=False):
    """bwlabel() (src/bwlabel.h:10): returns (labelled volume, number of labels)."""
    L = _lib.load()
    a = _vol(img).copy()
    nz, ny, nx = a.shape
    n = L.bwlabel(a.ctypes.data, conn, (C.c_size_t * 3)(nx, ny, nz), only_largest, fill_bubbles)
    return a, n


def apply_sform(pts, tris, srow_x, srow_y, srow_z):
    """apply_sform() (src/meshify.h:10): returns (tris, pts)."""
    L = _lib.load()
    p = np.ascontiguousarray(pts, dtype=np.float64).copy()
    t = np.ascontiguousarray(tris, dtype=np.int32).copy()
    f = lambda r: (C.c_float * 4)(*r)
    L.apply_sform(t.ctypes.data, p.ctypes.data, len(t), len(p), f(srow_x), f(srow_y), f(srow_z))
    return t, p


def set_threshold(img, mode=2):
    """setThreshold() (src/isolevel.h:7): Otsu isolevel on the robust range;
    mode 1 dark, 2 medium, 3 bright."""
    L = _lib.load()
    a = np.ascontiguousarray(img, dtype=np.float32).ravel()
    return float(L.setThreshold(a.ctypes.data, a.size, int(mode)))


def mesh_format_of(fnm):
    """The format save_mesh() picks for a file name (FMT_*); -1 when it appends ".mz3"."""
    return int(_lib.load().n2m_mesh_format_of(str(fnm).encode()))


def save_mesh(fnm, tris, pts, is_gz=False):
    """save_mesh() (src/meshify.h:8): writes the mesh in the format of the file
    name's extension.  Returns 0 (EXIT_SUCCESS) or 1 (EXIT_FAILURE)."""
    L = _lib.load()
    t = np.ascontiguousarray(tris, dtype=np.int32)
    p = np.ascontiguousarray(pts, dtype=np.float64)
    return int(L.save_mesh(str(fnm).encode(), t.ctypes.data, p.ctypes.data, len(t), len(p), bool(is_gz)))

