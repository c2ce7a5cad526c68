"""ctypes wrapper of the reference's own compiled code (oracle/_ref/libbmf_ref.so).

Test infrastructure only, and only usable where the reference sources are
present (the library is compiled from them by ``make -C oracle ref``).  It is
the pin for the C restatement and the generator of tests/golden/.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_ref", "libbmf_ref.so")
# The reference sources: $BMF_REFERENCE_SRC, else a checkout named
# reference/BinaryMeshFitting beside this repository's directory.
REF_SRC = os.environ.get("BMF_REFERENCE_SRC") or os.path.normpath(
    os.path.join(_HERE, "..", "..", "reference", "BinaryMeshFitting"))
_lib = None


def available():
    return os.path.isdir(REF_SRC)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            subprocess.check_call(["make", "-s", "-C", _HERE, "ref", "REF_SRC=" + REF_SRC],
                                  stdout=subprocess.DEVNULL)
        L = ctypes.CDLL(_LIB_PATH)
        vp = ctypes.c_void_p
        L.bmfref_run.restype = vp
        L.bmfref_run.argtypes = [ctypes.c_int, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.bmfref_count.restype = ctypes.c_longlong
        L.bmfref_count.argtypes = [vp, ctypes.c_int]
        L.bmfref_copy.argtypes = [vp, ctypes.c_int, vp]
        L.bmfref_free.argtypes = [vp]
        L.bmfref_process.argtypes = [ctypes.c_int, ctypes.c_longlong, vp, vp, vp, vp, vp, ctypes.c_longlong, vp,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.bmfref_implicit.argtypes = [ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, vp]
        L.bmfref_qef_3d.restype = ctypes.c_float
        L.bmfref_qef_3d.argtypes = [vp, vp, ctypes.c_int, vp]
        _lib = L
    return _lib


def run(dim, density, iters=0, boundary_processing=False, smooth_normals=False):
    """label_grid -> label_edges -> polygonize [-> MeshProcessor<3>] on a density block."""
    L = lib()
    d = np.ascontiguousarray(density, np.float32).reshape(-1)
    assert d.size == dim ** 3
    h = L.bmfref_run(dim, d.ctypes.data, iters, int(boundary_processing), int(smooth_normals))
    try:
        n = {k: L.bmfref_count(h, i) for i, k in enumerate(["words", "masks", "cells", "verts", "idx", "cm", "inds"])}

        def get(what, count, dtype, width=1):
            a = np.zeros(count * width, dtype)
            if count:
                L.bmfref_copy(h, what, a.ctypes.data)
            return a

        out = dict(contains_mesh=int(n["cm"]),
                   words=get(0, n["words"], np.uint32),
                   masks=get(1, n["masks"], np.uint64),
                   cell_mask=get(2, n["cells"], np.uint16),
                   cell_lin=get(3, n["cells"], np.uint32),
                   cell_vidx=get(4, n["cells"], np.uint32, 3).reshape(-1, 3),
                   pos=get(5, n["verts"], np.float32, 3).reshape(-1, 3),
                   nrm=get(6, n["verts"], np.float32, 3).reshape(-1, 3),
                   color=get(7, n["verts"], np.float32, 3).reshape(-1, 3),
                   boundary=get(8, n["verts"], np.uint8),
                   valence=get(9, n["verts"], np.uint8),
                   idx=get(10, n["idx"], np.uint32),
                   inds=get(11, n["inds"], np.uint32))
    finally:
        L.bmfref_free(h)
    return out


def process(N, pos, boundary, valence, idx, iters, boundary_processing=False, smooth_normals=False, nrm=None):
    L = lib()
    p = np.ascontiguousarray(pos, np.float32).reshape(-1).copy()
    n = np.zeros_like(p) if nrm is None else np.ascontiguousarray(nrm, np.float32).reshape(-1).copy()
    c = np.ones_like(p)
    b = np.ascontiguousarray(boundary, np.uint8)
    v = np.ascontiguousarray(valence, np.uint8)
    ix = np.ascontiguousarray(idx, np.uint32).copy()
    L.bmfref_process(N, len(b), p.ctypes.data, n.ctypes.data, c.ctypes.data, b.ctypes.data, v.ctypes.data, len(ix),
                     ix.ctypes.data, iters, int(boundary_processing), int(smooth_normals))
    return p.reshape(-1, 3), n.reshape(-1, 3), c.reshape(-1, 3)


def implicit(kind, resolution, origin, size, scale):
    L = lib()
    out = np.empty(size[0] * size[1] * size[2], np.float32)
    L.bmfref_implicit(kind, resolution, origin[0], origin[1], origin[2], size[0], size[1], size[2], scale,
                      out.ctypes.data)
    return out


def qef_3d(pos, nrm):
    L = lib()
    pos = np.ascontiguousarray(pos, np.float32)
    nrm = np.ascontiguousarray(nrm, np.float32)
    out = np.zeros(3, np.float32)
    e = L.bmfref_qef_3d(pos.ctypes.data, nrm.ctypes.data, len(pos), out.ctypes.data)
    return out, e
