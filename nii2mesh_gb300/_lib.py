"""ctypes binding of libn2m_gpu.so (C ABI declared in include/n2m_gpu.h).

The library is the product: every call below runs on the GPU.  Loading fails
loudly (RuntimeError) when the library has not been built — there is no CPU
fallback.
"""
import ctypes as C
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libn2m_gpu.so"

N2M_OK = 0
STATUS = ["ok", "no CUDA device", "CUDA error", "out of memory", "bad arguments", "no variability", "empty mesh",
          "non-finite voxels", "too large", "device wait timed out", "internal error"]

# exported symbols (the C-ABI contract; tests check that every one is present)
SYMBOLS = ["n2m_context_create", "n2m_context_destroy", "n2m_context_stream", "n2m_last_error",
           "n2m_status_string", "n2m_device_count", "meshify", "laplacian_smoothHC", "marchingCubes", "bwlabel",
           "apply_sform", "n2m_set_oldcubes", "n2m_meshify", "n2m_meshify_device", "n2m_smooth_hc_device",
           "n2m_kernel_launches", "n2m_meshify_backward", "n2m_smooth_hc_noalloc", "n2m_atlas", "n2m_atlas_device",
           "setThreshold", "n2m_set_threshold", "n2m_set_threshold_device", "n2m_cast_voxels_device",
           "n2m_meshify_typed", "save_mesh", "n2m_mesh_format_of", "n2m_encode_mesh", "n2m_encode_mesh_device",
           "n2m_encode_mesh_to_device", "n2m_meshify_into", "n2m_debug_fail_allocations",           "n2m_save_mesh", "n2m_save_mesh_device", "n2m_deflate_device"]


class vec3d(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


class vec3i(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("z", C.c_int)]


class Options(C.Structure):
    _fields_ = [("cubes", C.c_int), ("isolevel", C.c_float), ("pre_smooth", C.c_bool), ("only_largest", C.c_bool),
                ("fill_bubbles", C.c_bool), ("post_smooth", C.c_int), ("verbose", C.c_bool)]


class AtlasMesh(C.Structure):
    _fields_ = [("label", C.c_int), ("status", C.c_int), ("nvert", C.c_int), ("ntri", C.c_int),
                ("vert_offset", C.c_int64), ("tri_offset", C.c_int64)]


class Report(C.Structure):
    _fields_ = [("isolevel_used", C.c_float), ("vmin", C.c_float), ("vmax", C.c_float), ("lo", C.c_int * 3),
                ("hi", C.c_int * 3), ("nvert_raw", C.c_int64), ("ntri_raw", C.c_int64), ("nvert", C.c_int64),
                ("ntri", C.c_int64), ("welded", C.c_int), ("degenerate", C.c_int), ("ms_total", C.c_float),
                ("ms_stage", C.c_float * 8), ("kernel_launches", C.c_int64), ("ms_smooth_pass_a", C.c_float)]
    STAGES = ("smooth", "cluster", "count", "emit", "weld", "degenerate", "hc", "unused")

    def as_dict(self):
        return {f: (list(getattr(self, f)) if f in ("lo", "hi", "ms_stage") else getattr(self, f))
                for f, _ in self._fields_}


_lib = None


def load(path=None):
    """Load (once) and return the library with argtypes declared."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build the CUDA extension first (__graft_entry__.build() or "
                           f"python -m nii2mesh_gb300.build); there is no CPU fallback")
    L = C.CDLL(str(p))
    vp, ip = C.c_void_p, C.POINTER(C.c_int)
    L.n2m_context_create.argtypes = [C.POINTER(vp), C.c_int]
    L.n2m_context_destroy.argtypes = [vp]
    L.n2m_context_destroy.restype = None
    L.n2m_context_stream.argtypes = [vp]
    L.n2m_context_stream.restype = vp
    L.n2m_last_error.restype = C.c_char_p
    L.n2m_status_string.restype = C.c_char_p
    L.meshify.argtypes = [vp, C.POINTER(C.c_short), C.c_int, C.c_float, C.POINTER(vp), C.POINTER(vp), ip, ip,
                          C.c_bool, C.c_bool, C.c_bool, C.c_bool]
    L.laplacian_smoothHC.argtypes = [vp, vp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_bool]
    L.laplacian_smoothHC.restype = None
    L.marchingCubes.argtypes = [vp, C.POINTER(C.c_short), ip, ip, C.c_int, C.c_float, C.POINTER(vp), C.POINTER(vp),
                                ip, ip]
    L.bwlabel.argtypes = [vp, C.c_int, C.POINTER(C.c_size_t), C.c_bool, C.c_bool]
    L.apply_sform.argtypes = [vp, vp, C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float),
                              C.POINTER(C.c_float)]
    L.apply_sform.restype = None
    L.setThreshold.argtypes = [vp, C.c_int, C.c_int]
    L.setThreshold.restype = C.c_float
    L.n2m_set_threshold.argtypes = [vp, vp, C.c_int64, C.c_int, C.POINTER(C.c_float)]
    L.n2m_set_threshold_device.argtypes = [vp, vp, C.c_int64, C.c_int, C.POINTER(C.c_float)]
    L.n2m_cast_voxels_device.argtypes = [vp, vp, C.c_int, C.c_float, C.c_float, C.c_int64, vp]
    L.n2m_meshify_typed.argtypes = [vp, vp, C.c_int, C.c_float, C.c_float, ip, C.POINTER(Options), C.POINTER(vp),
                                    C.POINTER(vp), ip, ip, C.POINTER(Report)]
    L.n2m_set_oldcubes.argtypes = [C.c_int]
    L.n2m_meshify.argtypes = [vp, vp, ip, C.POINTER(Options), C.POINTER(vp), C.POINTER(vp), ip, ip, C.POINTER(Report)]
    L.n2m_debug_fail_allocations.argtypes = [C.c_int]
    L.n2m_meshify_into.argtypes = [vp, vp, ip, C.POINTER(Options), vp, C.c_int64, vp, C.c_int64, ip, ip,
                                   C.POINTER(Report)]
    L.n2m_meshify_device.argtypes = [vp, vp, ip, C.POINTER(Options), C.POINTER(vp), C.POINTER(vp), ip, ip,
                                     C.POINTER(Report)]
    L.n2m_kernel_launches.restype = C.c_longlong
    L.n2m_meshify_backward.argtypes = [vp, vp, vp]
    i64p = C.POINTER(C.c_int64)
    L.n2m_atlas.argtypes = [vp, vp, ip, C.POINTER(Options), C.c_int, ip, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp),
                            i64p, i64p]
    L.n2m_atlas_device.argtypes = [vp, vp, ip, C.POINTER(Options), C.c_int, ip, C.POINTER(C.POINTER(AtlasMesh)),
                                   C.POINTER(vp), C.POINTER(vp), i64p, i64p, C.POINTER(Report)]
    L.n2m_smooth_hc_device.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_bool]
    szp = C.POINTER(C.c_size_t)
    L.save_mesh.argtypes = [C.c_char_p, vp, vp, C.c_int, C.c_int, C.c_bool]
    L.n2m_mesh_format_of.argtypes = [C.c_char_p]
    L.n2m_encode_mesh.argtypes = [vp, C.c_int, vp, vp, C.c_int, C.c_int, C.c_int, C.POINTER(vp), szp]
    L.n2m_encode_mesh_device.argtypes = [vp, C.c_int, vp, vp, C.c_int, C.c_int, C.c_int, C.POINTER(vp), szp]
    L.n2m_encode_mesh_to_device.argtypes = [vp, C.c_int, vp, vp, C.c_int, C.c_int, C.c_int, C.POINTER(vp), szp]
    L.n2m_save_mesh.argtypes = [vp, C.c_char_p, vp, vp, C.c_int, C.c_int, C.c_int]
    L.n2m_save_mesh_device.argtypes = [vp, C.c_char_p, vp, vp, C.c_int, C.c_int, C.c_int]
    L.n2m_deflate_device.argtypes = [vp, vp, C.c_size_t, C.c_int, C.POINTER(vp), szp]
    libc = C.CDLL(None)
    libc.free.argtypes = [vp]
    L.libc_free = libc.free
    _lib = L
    return L


def check(status, what="n2m call"):
    if status != N2M_OK:
        L = load()
        msg = L.n2m_last_error().decode(errors="replace")
        name = STATUS[status] if 0 <= status < len(STATUS) else str(status)
        raise N2MError(status, f"{what}: {name}: {msg}")


class N2MError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(msg)
        self.status = status
