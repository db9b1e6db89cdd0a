"""ctypes front end of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module; it is the checker, never part of the product path.

Two back ends share one numpy-facing interface:
  * ``Oracle()``      — the C restatement in n2m_oracle.c, built by
                        oracle/Makefile into oracle/_build/ (available on any
                        machine with a C compiler);
  * ``Reference()``   — the reference nii2mesh compiled from its own sources by
                        oracle/build_ref.sh into oracle/_ref/ (available only
                        where the reference tree is present).
Volumes are numpy float32 arrays of shape (nz, ny, nx) (x fastest, the
reference's layout).  Meshes are (tris int32 (nt,3), pts float64 (np,3)).
"""
import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OR_LIB = HERE / "_build" / "libn2m_oracle.so"
REF_DIR = HERE / "_ref"

MC33, MC_CLASSIC_TABLE, OLDCUBES = 0, 1, 2

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")


def build_oracle():
    """Compile the oracle library (idempotent)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return OR_LIB


def _as_vol(img):
    a = np.ascontiguousarray(img, dtype=np.float32)
    if a.ndim != 3:
        raise ValueError("volume must be 3-D (nz, ny, nx)")
    return a


def _dims(a):
    nz, ny, nx = a.shape
    return (C.c_short * 3)(nx, ny, nz)


def _take_mesh(lib, tp, pp, nt, np_):
    tris = np.ctypeslib.as_array(C.cast(tp, C.POINTER(C.c_int)), shape=(nt, 3)).copy() if nt else np.zeros((0, 3), np.int32)
    pts = np.ctypeslib.as_array(C.cast(pp, C.POINTER(C.c_double)), shape=(np_, 3)).copy() if np_ else np.zeros((0, 3))
    lib.free_(tp)
    lib.free_(pp)
    return tris.astype(np.int32), pts


class Oracle:
    """The C restatement (n2m_oracle.c)."""

    def __init__(self, path=None):
        path = Path(path) if path else OR_LIB
        if not path.exists():
            build_oracle()
        L = C.CDLL(str(path))
        self.lib = L
        L.or_quick_smooth.argtypes = [_f32p, C.c_int, C.c_int, C.c_int]
        L.or_bwlabel.argtypes = [_f32p, C.c_int, C.POINTER(C.c_size_t), C.c_bool, C.c_bool]
        L.or_prepare_volume.argtypes = [_f32p, C.POINTER(C.c_short), C.POINTER(C.c_float), C.c_bool, C.c_bool, C.c_bool,
                                        C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_float)]
        L.or_marching_cubes.argtypes = [_f32p, C.POINTER(C.c_short), C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int,
                                        C.c_float, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_int),
                                        C.POINTER(C.c_int)]
        L.or_meshify.argtypes = [_f32p, C.POINTER(C.c_short), C.c_int, C.c_float, C.POINTER(C.c_void_p),
                                 C.POINTER(C.c_void_p), C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_bool, C.c_bool, C.c_bool]
        L.or_marching_cubes_sources.argtypes = [_f32p, C.POINTER(C.c_short), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                                C.c_int, C.c_float, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                                C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_void_p)]
        L.or_mc_raw.argtypes = [_f32p, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.or_laplacian_smoothHC.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_bool]
        L.or_border_vertices.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        L.or_apply_sform.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_float),
                                     C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.or_set_threshold.argtypes = [_f32p, C.c_int, C.c_int]
        L.or_set_threshold.restype = C.c_float
        L.or_binarize_label.argtypes = [_f32p, C.c_int, C.c_int, _f32p]
        L.or_selftest_field.argtypes = [C.c_int, _f32p]
        L.or_free.argtypes = [C.c_void_p]
        L.free_ = L.or_free

    # -- stages -----------------------------------------------------------
    def quick_smooth(self, img):
        a = _as_vol(img).copy()
        nz, ny, nx = a.shape
        self.lib.or_quick_smooth(a, nx, ny, nz)
        return a

    def bwlabel(self, img, conn=18, only_largest=False, fill_bubbles=False):
        a = _as_vol(img).copy()
        nz, ny, nx = a.shape
        d = (C.c_size_t * 3)(nx, ny, nz)
        n = self.lib.or_bwlabel(a, conn, d, only_largest, fill_bubbles)
        return a, n

    def prepare_volume(self, img, iso, pre_smooth=True, only_largest=False, fill_bubbles=False):
        """Returns (volume entering marching cubes, iso, lo, hi, mn) or None."""
        a = _as_vol(img).copy()
        isoc = C.c_float(iso)
        lo, hi, mn = (C.c_int * 3)(), (C.c_int * 3)(), C.c_float()
        if self.lib.or_prepare_volume(a, _dims(a), C.byref(isoc), pre_smooth, only_largest, fill_bubbles, lo, hi, C.byref(mn)):
            return None
        return a, isoc.value, tuple(lo), tuple(hi), mn.value

    def marching_cubes(self, img, lo, hi, variant, iso):
        a = _as_vol(img)
        tp, pp, nv, nt = C.c_void_p(), C.c_void_p(), C.c_int(), C.c_int()
        r = self.lib.or_marching_cubes(a, _dims(a), (C.c_int * 3)(*lo), (C.c_int * 3)(*hi), variant, iso,
                                       C.byref(pp), C.byref(tp), C.byref(nv), C.byref(nt))
        if r:
            return None
        return _take_mesh(self.lib, tp, pp, nt.value, nv.value)

    def marching_cubes_sources(self, img, lo, hi, iso, original_mc=0):
        """(tris, pts, src): src[i] = (kind, grid index, axis) for raw vertex i"""
        a = _as_vol(img)
        tp, pp, nv, nt, sp = C.c_void_p(), C.c_void_p(), C.c_int(), C.c_int(), C.c_void_p()
        r = self.lib.or_marching_cubes_sources(a, _dims(a), (C.c_int * 3)(*lo), (C.c_int * 3)(*hi), original_mc, iso,
                                               C.byref(pp), C.byref(tp), C.byref(nv), C.byref(nt), C.byref(sp))
        if r:
            return None
        src = np.ctypeslib.as_array(C.cast(sp, C.POINTER(C.c_int)), shape=(nv.value, 3)).copy()
        self.lib.or_free(sp)
        t, p = _take_mesh(self.lib, tp, pp, nt.value, nv.value)
        return t, p, src

    def mc_raw(self, data, original_mc=0):
        a = _as_vol(data)
        nz, ny, nx = a.shape
        vp, tp, nv, nt = C.c_void_p(), C.c_void_p(), C.c_int(), C.c_int()
        self.lib.or_mc_raw(a, nx, ny, nz, original_mc, C.byref(vp), C.byref(tp), C.byref(nv), C.byref(nt))
        v = np.ctypeslib.as_array(C.cast(vp, C.POINTER(C.c_float)), shape=(nv.value, 3)).copy() if nv.value else np.zeros((0, 3), np.float32)
        t = np.ctypeslib.as_array(C.cast(tp, C.POINTER(C.c_int)), shape=(nt.value, 3)).copy() if nt.value else np.zeros((0, 3), np.int32)
        self.lib.or_free(vp)
        self.lib.or_free(tp)
        return t, v

    def meshify(self, img, iso, variant=MC33, pre_smooth=True, only_largest=True, fill_bubbles=False):
        a = _as_vol(img).copy()
        tp, pp, nt, np_ = C.c_void_p(), C.c_void_p(), C.c_int(), C.c_int()
        r = self.lib.or_meshify(a, _dims(a), variant, iso, C.byref(tp), C.byref(pp), C.byref(nt), C.byref(np_),
                                pre_smooth, only_largest, fill_bubbles)
        if r:
            return None
        return _take_mesh(self.lib, tp, pp, nt.value, np_.value)

    def laplacian_smoothHC(self, pts, tris, alpha=0.1, beta=0.5, iters=1, lock_edges=True):
        p = np.ascontiguousarray(pts, dtype=np.float64).copy()
        t = np.ascontiguousarray(tris, dtype=np.int32)
        self.lib.or_laplacian_smoothHC(p.ctypes.data, t.ctypes.data, len(p), len(t), alpha, beta, iters, lock_edges)
        return p

    def border_vertices(self, tris, nvert):
        t = np.ascontiguousarray(tris, dtype=np.int32)
        b = np.zeros(nvert + 1, np.uint8)
        self.lib.or_border_vertices(t.ctypes.data, nvert, len(t), b.ctypes.data)
        return b[:nvert].astype(bool)

    def apply_sform(self, pts, tris, srow_x, srow_y, srow_z):
        p = np.ascontiguousarray(pts, dtype=np.float64).copy()
        t = np.ascontiguousarray(tris, dtype=np.int32).copy()
        f = lambda r: (C.c_float * 4)(*r)
        self.lib.or_apply_sform(t.ctypes.data, p.ctypes.data, len(t), len(p), f(srow_x), f(srow_y), f(srow_z))
        return t, p

    def set_threshold(self, img, mode=2):
        a = np.ascontiguousarray(img, dtype=np.float32).ravel()
        return float(self.lib.or_set_threshold(a, a.size, mode))

    def binarize_label(self, img, label):
        a = np.ascontiguousarray(img, dtype=np.float32)
        out = np.empty_like(a)
        n = self.lib.or_binarize_label(a.ravel(), a.size, label, out.ravel())
        return out, n

    def selftest_field(self, obj):
        out = np.empty((60, 60, 60), np.float32)
        if self.lib.or_selftest_field(obj, out.ravel()):
            raise ValueError(obj)
        return out


class Reference:
    """The reference nii2mesh built from its own sources (oracle/_ref)."""

    def __init__(self, classic=False):
        name = "libn2m_ref_classic.so" if classic else "libn2m_ref_lewiner.so"
        path = REF_DIR / name
        if not path.exists():
            raise FileNotFoundError(path)
        L = C.CDLL(str(path))
        self.lib, self.classic = L, classic
        self.libc = C.CDLL(None)
        self.libc.free.argtypes = [C.c_void_p]
        L.meshify.argtypes = [_f32p, C.POINTER(C.c_short), C.c_int, C.c_float, C.POINTER(C.c_void_p),
                              C.POINTER(C.c_void_p), C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_bool, C.c_bool, C.c_bool, C.c_bool]
        L.laplacian_smoothHC.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_bool]
        L.setThreshold.argtypes = [_f32p, C.c_int, C.c_int]
        L.setThreshold.restype = C.c_float
        L.bwlabel.argtypes = [_f32p, C.c_int, C.POINTER(C.c_size_t), C.c_bool, C.c_bool]
        L.marchingCubes.argtypes = [_f32p, C.POINTER(C.c_short), C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int, C.c_float,
                                    C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.apply_sform.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                  C.POINTER(C.c_float)]
        L.free_ = self.libc.free

    def meshify(self, img, iso, variant=MC33, pre_smooth=True, only_largest=True, fill_bubbles=False, verbose=False):
        if (variant == OLDCUBES) != self.classic:
            raise ValueError("variant does not match this reference build")
        a = _as_vol(img).copy()
        tp, pp, nt, np_ = C.c_void_p(), C.c_void_p(), C.c_int(), C.c_int()
        r = self.lib.meshify(a, _dims(a), 1 if variant == MC_CLASSIC_TABLE else 0, iso, C.byref(tp), C.byref(pp),
                             C.byref(nt), C.byref(np_), pre_smooth, only_largest, fill_bubbles, verbose)
        if r:
            return None
        return _take_mesh(self.lib, tp, pp, nt.value, np_.value)

    def marching_cubes(self, img, lo, hi, variant, iso):
        a = _as_vol(img).copy()
        tp, pp, nv, nt = C.c_void_p(), C.c_void_p(), C.c_int(), C.c_int()
        r = self.lib.marchingCubes(a, _dims(a), (C.c_int * 3)(*lo), (C.c_int * 3)(*hi), 1 if variant == MC_CLASSIC_TABLE else 0,
                                   iso, C.byref(pp), C.byref(tp), C.byref(nv), C.byref(nt))
        if r:
            return None
        return _take_mesh(self.lib, tp, pp, nt.value, nv.value)

    def bwlabel(self, img, conn=18, only_largest=False, fill_bubbles=False):
        a = _as_vol(img).copy()
        nz, ny, nx = a.shape
        n = self.lib.bwlabel(a, conn, (C.c_size_t * 3)(nx, ny, nz), only_largest, fill_bubbles)
        return a, n

    def laplacian_smoothHC(self, pts, tris, alpha=0.1, beta=0.5, iters=1, lock_edges=True):
        p = np.ascontiguousarray(pts, dtype=np.float64).copy()
        t = np.ascontiguousarray(tris, dtype=np.int32)
        self.lib.laplacian_smoothHC(p.ctypes.data, t.ctypes.data, len(p), len(t), alpha, beta, iters, lock_edges)
        return p

    def apply_sform(self, pts, tris, srow_x, srow_y, srow_z):
        p = np.ascontiguousarray(pts, dtype=np.float64).copy()
        t = np.ascontiguousarray(tris, dtype=np.int32).copy()
        f = lambda r: (C.c_float * 4)(*r)
        self.lib.apply_sform(t.ctypes.data, p.ctypes.data, len(t), len(p), f(srow_x), f(srow_y), f(srow_z))
        return t, p

    def set_threshold(self, img, mode=2):
        a = np.ascontiguousarray(img, dtype=np.float32).ravel()
        return float(self.lib.setThreshold(a, a.size, mode))


# NIfTI datatypes load_nii reads (src/nii2mesh.c:114-117)
NIFTI_DT = {np.dtype(np.uint8): 2, np.dtype(np.int16): 4, np.dtype(np.float32): 16, np.dtype(np.uint16): 512}


def cast_voxels(raw, scl_slope, scl_inter):
    """load_nii's voxel cast (src/nii2mesh.c:122, :160-175) in float32 numpy
    arithmetic: (voxel * scl_slope) + scl_inter, multiply and add each rounded;
    a zero slope means 1."""
    slope = np.float32(scl_slope) if scl_slope != 0 else np.float32(1.0)
    return (np.asarray(raw).astype(np.float32) * slope) + np.float32(scl_inter)


def reference_available(classic=False):
    return (REF_DIR / ("libn2m_ref_classic.so" if classic else "libn2m_ref_lewiner.so")).exists()


# -- canonical mesh comparison ------------------------------------------------
def canonical(tris, pts):
    """Canonical form of a mesh: vertices sorted lexicographically by (x,y,z),
    triangle indices remapped, each triangle rotated so its smallest index
    comes first (winding kept), triangles sorted.  Unreferenced vertices are
    kept, so vertex counts compare as-is."""
    pts = np.asarray(pts, np.float64)
    tris = np.asarray(tris, np.int64)
    order = np.lexsort((pts[:, 2], pts[:, 1], pts[:, 0]))
    inv = np.empty_like(order)
    inv[order] = np.arange(len(order))
    cp = pts[order]
    ct = inv[tris] if len(tris) else tris.reshape(0, 3)
    if len(ct):
        r = np.argmin(ct, axis=1)
        idx = (np.arange(3)[None, :] + r[:, None]) % 3
        ct = np.take_along_axis(ct, idx, axis=1)
        ct = ct[np.lexsort((ct[:, 2], ct[:, 1], ct[:, 0]))]
    return ct.astype(np.int64), cp


def mesh_equal(a, b, pos_tol=0.0):
    """(equal, max |dpos|, message).  Connectivity must match exactly after
    canonical sorting; positions within pos_tol."""
    ta, pa = canonical(*a)
    tb, pb = canonical(*b)
    if pa.shape != pb.shape:
        return False, np.inf, f"vertex count {len(pa)} != {len(pb)}"
    if ta.shape != tb.shape:
        return False, np.inf, f"triangle count {len(ta)} != {len(tb)}"
    d = float(np.max(np.abs(pa - pb))) if len(pa) else 0.0
    if d > pos_tol:
        return False, d, f"max position difference {d:g} > {pos_tol:g}"
    if not np.array_equal(ta, tb):
        n = int(np.sum(np.any(ta != tb, axis=1)))
        return False, d, f"{n} triangles differ after canonical sort"
    return True, d, "ok"


def smoothed_equal(a_raw, a_smooth, b_raw, b_smooth, tol):
    """Compare two post-smoothed meshes whose un-smoothed meshes must match
    exactly: the vertex correspondence comes from the raw positions (a
    canonical sort of smoothed positions is unstable under tiny differences),
    then smoothed positions must agree within tol.  a_raw/b_raw = (tris, pts)."""
    ok, d, msg = mesh_equal(a_raw, b_raw, 0.0)
    if not ok:
        return False, d, "raw meshes differ: " + msg
    pa, pb = np.asarray(a_raw[1]), np.asarray(b_raw[1])
    oa = np.lexsort((pa[:, 2], pa[:, 1], pa[:, 0]))
    ob = np.lexsort((pb[:, 2], pb[:, 1], pb[:, 0]))
    d = float(np.abs(np.asarray(a_smooth)[oa] - np.asarray(b_smooth)[ob]).max()) if len(oa) else 0.0
    if d > tol:
        return False, d, f"max smoothed position difference {d:g} > {tol:g}"
    return True, d, "ok"
