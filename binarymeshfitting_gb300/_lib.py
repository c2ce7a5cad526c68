"""ctypes binding of libbmf_gb300.so (the C ABI declared in include/bmf.h).

The library is the product: there is no CPU fallback.  Loading fails loudly
when the library cannot be built/loaded or no CUDA device is present.
"""
import ctypes
import os

from . import build as _build

c_int32, c_int64, c_float, c_void_p = ctypes.c_int32, ctypes.c_int64, ctypes.c_float, ctypes.c_void_p

# bmf_fields.h
FIELD_GRID, FIELD_SPHERE_WAVE, FIELD_TERRAIN_FBM = 0, 1, 2
FIELD_TORUS_Z, FIELD_SPHERE, FIELD_CUBOID, FIELD_PLANE_Y = 3, 4, 5, 6
FIELD_TERRAIN_2D = 7
MODE_R, MODE_Q = 0, 1
PLACE_CENTER, PLACE_MASSPOINT, PLACE_QEF = 0, 1, 2
FIT_ADJOINT_F64 = 1
FIT_ADJOINT_DF = 2

STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "output capacity exceeded", 4: "device wait timed out",
          5: "out of device memory", 6: "not supported"}
OK, ERR_INVALID_ARGUMENT, ERR_CUDA, ERR_CAPACITY, ERR_TIMEOUT, ERR_OUT_OF_MEMORY, ERR_NOT_SUPPORTED = range(7)


class BmfError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s (status %d): %s" % (STATUS.get(status, "?"), status, message))
        self.status = status


class Field(ctypes.Structure):
    _fields_ = [("kind", c_int32), ("params", c_float * 8)]

    @classmethod
    def make(cls, kind, params=()):
        f = cls()
        f.kind = kind
        for i, p in enumerate(params):
            f.params[i] = float(p)
        return f


class ChunkDesc(ctypes.Structure):
    _fields_ = [("origin", c_float * 3), ("scale", c_float), ("dim", c_int32), ("level", c_int32)]

    @classmethod
    def make(cls, origin, scale, dim, level=0):
        d = cls()
        for i in range(3):
            d.origin[i] = float(origin[i])
        d.scale = float(scale)
        d.dim = int(dim)
        d.level = int(level)
        return d


class ExtractOpts(ctypes.Structure):
    _fields_ = [("mode", c_int32), ("placement", c_int32), ("iters", c_int32), ("process_boundary", c_int32),
                ("smooth_normals", c_int32), ("reserved", c_int32)]


class Mesh(ctypes.Structure):
    _fields_ = [("d_pos", c_void_p), ("d_nrm", c_void_p), ("d_boundary", c_void_p), ("d_valence", c_void_p),
                ("d_idx", c_void_p), ("vcap", c_int64), ("icap", c_int64), ("n_verts", c_int64),
                ("n_idx", c_int64), ("contains_mesh", c_int32), ("prim_size", c_int32)]


class BatchOut(ctypes.Structure):
    _fields_ = [("d_pos", c_void_p), ("d_nrm", c_void_p), ("d_boundary", c_void_p), ("d_idx", c_void_p),
                ("vcap", c_int64), ("icap", c_int64), ("d_chunk_info", c_void_p), ("n_verts", c_int64),
                ("n_idx", c_int64)]


class LodParams(ctypes.Structure):
    _fields_ = [("root_pos", c_float * 3), ("root_size", c_float), ("focus", c_float * 3),
                ("split_multiplier", c_float), ("size_modifier", c_float), ("min_level", c_int32),
                ("max_level", c_int32), ("dim", c_int32), ("base_overlap", c_float),
                ("boundary_processing", c_int32), ("iters", c_int32)]


class BatchTuning(ctypes.Structure):
    _fields_ = [("fill_mode", c_int32), ("fill_run", c_int32), ("sweep_block", c_int32), ("fill_band", c_int32),
                ("reserved", c_int32 * 4)]


class Config(ctypes.Structure):
    _fields_ = [("device", c_int32), ("flags", c_int32), ("scratch_bytes", ctypes.c_size_t)]


# Every symbol declared in include/bmf.h, with its ctypes signature.
SIGNATURES = {
    "bmf_create": (c_int32, [ctypes.POINTER(Config), ctypes.POINTER(c_void_p)]),
    "bmf_destroy": (c_int32, [c_void_p]),
    "bmf_status_string": (ctypes.c_char_p, [c_int32]),
    "bmf_last_error": (ctypes.c_char_p, [c_void_p]),
    "bmf_launch_count": (c_int64, [c_void_p]),
    "bmf_sample_block": (c_int32, [c_void_p, ctypes.POINTER(ChunkDesc), ctypes.POINTER(Field), c_void_p, c_void_p]),
    "bmf_label_grid": (c_int32, [c_void_p, c_int32, c_void_p, c_void_p, ctypes.POINTER(c_int32), c_void_p]),
    "bmf_sample_label": (c_int32, [c_void_p, ctypes.POINTER(ChunkDesc), ctypes.POINTER(Field), c_void_p, c_void_p,
                                   ctypes.POINTER(c_int32), c_void_p]),
    "bmf_cell_masks": (c_int32, [c_void_p, c_int32, c_void_p, c_void_p, c_void_p]),
    "bmf_polygonize": (c_int32, [c_void_p, c_int32, c_void_p, c_void_p, c_int32, c_int32, ctypes.POINTER(Mesh),
                                 c_void_p]),
    "bmf_polygonize_noalloc": (c_int32, [c_int32, c_void_p, c_void_p, c_int32, c_int32, ctypes.POINTER(Mesh),
                                         c_void_p]),
    "bmf_process": (c_int32, [c_void_p, ctypes.POINTER(Mesh), c_int32, c_int32, c_int32, c_void_p]),
    "bmf_extract_chunk": (c_int32, [c_void_p, ctypes.POINTER(ChunkDesc), ctypes.POINTER(Field),
                                    ctypes.POINTER(ExtractOpts), ctypes.POINTER(Mesh), c_void_p]),
    "bmf_batch_create": (c_int32, [c_void_p, ctypes.POINTER(ChunkDesc), c_int32, ctypes.POINTER(Field),
                                   ctypes.POINTER(ExtractOpts), ctypes.POINTER(c_void_p)]),
    "bmf_batch_run": (c_int32, [c_void_p, ctypes.POINTER(BatchOut), c_int32, c_int32, c_void_p]),
    "bmf_batch_destroy": (c_int32, [c_void_p]),
    "bmf_batch_set_descs": (c_int32, [c_void_p, ctypes.POINTER(ChunkDesc), c_int32, c_void_p]),
    "bmf_batch_wait": (c_int32, [c_void_p, ctypes.POINTER(BatchOut), c_int32]),
    "bmf_batch_wait_extraction": (c_int32, [c_void_p, c_void_p]),
    "bmf_batch_profile": (c_int32, [c_void_p, ctypes.POINTER(BatchOut), ctypes.POINTER(c_float), c_void_p]),
    "bmf_lod_generate": (c_int32, [c_void_p, ctypes.POINTER(LodParams), c_void_p, c_int32, c_void_p, c_void_p]),
    "bmf_format": (c_int32, [c_void_p, ctypes.POINTER(Mesh), c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_int64,
                             ctypes.POINTER(c_int64), c_void_p]),
    "bmf_batch_format": (c_int32, [c_void_p, ctypes.POINTER(BatchOut), c_int32, c_int32, c_void_p, c_void_p, c_void_p,
                                   c_int64, c_void_p]),
    "bmf_batch_get_tuning": (c_int32, [c_void_p, ctypes.POINTER(BatchTuning)]),
    "bmf_batch_set_tuning": (c_int32, [c_void_p, ctypes.POINTER(BatchTuning)]),
    "bmf_batch_autotune": (c_int32, [c_void_p, ctypes.POINTER(BatchOut), c_int32, c_void_p, ctypes.POINTER(BatchTuning),
                                     ctypes.POINTER(c_float), c_int32, ctypes.POINTER(c_int32)]),
    "bmf_fit_create": (c_int32, [c_void_p, c_int32, c_int32, c_int32, c_int32, c_int64, c_int64, c_int32,
                                 ctypes.POINTER(c_void_p)]),
    "bmf_fit_forward": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, ctypes.POINTER(c_int64),
                                  c_void_p]),
    "bmf_fit_backward": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p]),
    "bmf_fit_loss_spheres": (c_int32, [c_void_p, c_void_p, c_void_p, c_int32, c_void_p, c_void_p, c_void_p]),
    "bmf_fit_adam": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_float, c_float,
                               c_float, c_float, c_void_p]),
    "bmf_fit_destroy": (c_int32, [c_void_p]),
}

_lib = None


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Loads libbmf_gb300.so (building it first if needed) and binds the ABI."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libbmf_gb300.so is missing (%s); run binarymeshfitting_gb300/build.py" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status, ctx=None, lib=None):
    if status != OK:
        lib = lib or _lib
        msg = lib.bmf_last_error(ctx).decode() if (lib is not None and ctx) else ""
        raise BmfError(status, msg)
