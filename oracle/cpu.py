"""ctypes wrapper of the C restatement (oracle/bmf_oracle.c) -- test infrastructure only."""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libbmf_oracle.so")
_lib = None

_f32p = ctypes.POINTER(ctypes.c_float)


def build():
    """Compiles the restatement with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.check_call(["make", "-s", "-C", _HERE], stdout=subprocess.DEVNULL)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        vp, i64, c_int, c_float = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_float
        L.bmfo_sin.restype = c_float
        L.bmfo_sin.argtypes = [c_float]
        L.bmfo_fill_field.argtypes = [c_int, vp, c_int, vp, c_float, vp]
        L.bmfo_perm_init.argtypes = [ctypes.c_uint64, vp]
        for fn in (L.bmfo_perlin, L.bmfo_perlin_textbook):
            fn.restype = c_float
            fn.argtypes = [vp, c_float, c_float, c_float]
        L.bmfo_label_grid.restype = c_int
        L.bmfo_label_grid.argtypes = [c_int, vp, vp]
        L.bmfo_cell_masks.argtypes = [c_int, vp, vp]
        L.bmfo_extract_r.restype = c_int
        L.bmfo_extract_r.argtypes = [c_int, vp, vp, i64, i64, i64, vp, vp, vp, vp, vp, vp, vp]
        L.bmfo_extract_q.restype = c_int
        L.bmfo_extract_q.argtypes = [c_int, vp, vp, c_int, i64, i64, vp, vp, vp, vp, vp]
        L.bmfo_process.argtypes = [c_int, i64, vp, vp, vp, vp, i64, vp, c_int, c_int, c_int]
        L.bmfo_qef_f32.restype = c_float
        L.bmfo_qef_f32.argtypes = [vp, vp, c_int, vp]
        L.bmfo_qef_f64.restype = ctypes.c_double
        L.bmfo_qef_f64.argtypes = [vp, vp, c_int, vp]
        L.bmfo_fit_loss_f64.restype = ctypes.c_double
        L.bmfo_fit_loss_f64.argtypes = [c_int, vp, c_int, vp, vp, vp, vp, vp]
        L.bmfo_fit_loss_spheres_f64.restype = ctypes.c_double
        L.bmfo_fit_loss_spheres_f64.argtypes = [c_int, vp, c_int, vp, c_int, vp, vp, vp, vp]
        L.bmfo_lod_generate.restype = i64
        L.bmfo_lod_generate.argtypes = [vp, c_int, c_int, c_int, c_int, c_int, vp, i64]
        L.bmfo_format.restype = i64
        L.bmfo_format.argtypes = [i64, vp, vp, i64, vp, c_int, c_int, vp, vp, vp]
        L.bmfo_extract_batch.restype = i64
        L.bmfo_extract_batch.argtypes = [c_int, vp, c_int, vp, c_int, c_int, c_int, c_int, vp, c_int]
        L.bmfo_extract_batch_digest.restype = i64
        L.bmfo_extract_batch_digest.argtypes = [c_int, vp, c_int, vp, c_int, c_int, c_int, c_int, c_int, vp, vp,
                                                c_int]
        L.bmfo_terrain2d_height.restype = c_float
        L.bmfo_terrain2d_height.argtypes = [vp, vp, c_float, c_float]
        for fn in (L.bmfo_noise2_grad,):
            fn.restype = c_float
            fn.argtypes = [vp, c_int, c_float, c_float]
        L.bmfo_noise2_value.restype = c_float
        L.bmfo_noise2_value.argtypes = [vp, c_float, c_float]
        L.bmfo_digest64.restype = ctypes.c_uint64
        L.bmfo_digest64.argtypes = [vp, i64, c_int]
        _lib = L
    return _lib


class Counts(ctypes.Structure):
    _fields_ = [("n_cells", ctypes.c_int64), ("n_verts", ctypes.c_int64), ("n_idx", ctypes.c_int64)]


def _p(a):
    return None if a is None else a.ctypes.data


def perm(seed):
    """The noise permutation of a seed (256 bytes)."""
    out = np.empty(256, np.uint8)
    lib().bmfo_perm_init(seed, _p(out))
    return out


def perlin(p, x, y, z, textbook=False):
    """One noise value: the line-separable form, or the textbook order."""
    fn = lib().bmfo_perlin_textbook if textbook else lib().bmfo_perlin
    return fn(_p(p), x, y, z)


def noise2(p, x, z, kind="grad", c=0):
    """One 2D gradient (component c) or value noise value of BMF_FIELD_TERRAIN_2D."""
    if kind == "grad":
        return lib().bmfo_noise2_grad(_p(p), c, x, z)
    return lib().bmfo_noise2_value(_p(p), x, z)


def terrain2d_height(params, px, pz):
    prm = np.zeros(8, np.float32)
    prm[: len(params)] = params
    return lib().bmfo_terrain2d_height(_p(perm(int(params[6]))), _p(prm), px, pz)


def fill_field(kind, params, dim, origin=(0.0, 0.0, 0.0), scale=1.0):
    out = np.empty(dim ** 3, np.float32)
    prm = np.zeros(8, np.float32)
    prm[: len(params)] = params
    org = np.asarray(origin, np.float32)
    lib().bmfo_fill_field(kind, _p(prm), dim, _p(org), scale, _p(out))
    return out


def label_grid(dim, density):
    zc = (dim + 31) // 32
    words = np.empty(dim * dim * zc, np.uint32)
    cm = lib().bmfo_label_grid(dim, _p(np.ascontiguousarray(density, np.float32)), _p(words))
    return words, int(cm)


def cell_masks(dim, words):
    zc = (dim + 31) // 32
    masks = np.zeros(dim * dim * 4 * zc, np.uint64)
    lib().bmfo_cell_masks(dim, _p(np.ascontiguousarray(words, np.uint32)), _p(masks))
    return masks


def extract_r(dim, density, masks, with_cells=False):
    """Mode R: returns dict(pos, boundary, valence, idx[, cell_lin, cell_mask])."""
    d = np.ascontiguousarray(density, np.float32)
    c = Counts()
    lib().bmfo_extract_r(dim, _p(d), _p(masks), 0, 0, 0, None, None, None, None, None, None, ctypes.byref(c))
    nv, ni, nc = c.n_verts, c.n_idx, c.n_cells
    pos = np.empty(nv * 3, np.float32)
    bnd = np.empty(nv, np.uint8)
    val = np.empty(nv, np.uint8)
    idx = np.empty(ni, np.uint32)
    cl = np.empty(nc, np.uint32) if with_cells else None
    cm = np.empty(nc, np.uint16) if with_cells else None
    rc = lib().bmfo_extract_r(dim, _p(d), _p(masks), nv, ni, nc if with_cells else 0, _p(pos), _p(bnd), _p(val),
                              _p(idx), _p(cl), _p(cm), ctypes.byref(c))
    assert rc == 0
    out = dict(pos=pos.reshape(-1, 3), boundary=bnd, valence=val, idx=idx, n_cells=nc)
    if with_cells:
        out.update(cell_lin=cl, cell_mask=cm)
    return out


def extract_q(dim, density, words, placement=0):
    d = np.ascontiguousarray(density, np.float32)
    w = np.ascontiguousarray(words, np.uint32)
    c = Counts()
    lib().bmfo_extract_q(dim, _p(d), _p(w), placement, 0, 0, None, None, None, None, ctypes.byref(c))
    nv, ni = c.n_verts, c.n_idx
    pos = np.empty(nv * 3, np.float32)
    bnd = np.empty(nv, np.uint8)
    val = np.empty(nv, np.uint8)
    idx = np.empty(ni, np.uint32)
    rc = lib().bmfo_extract_q(dim, _p(d), _p(w), placement, nv, ni, _p(pos), _p(bnd), _p(val), _p(idx),
                              ctypes.byref(c))
    assert rc == 0
    return dict(pos=pos.reshape(-1, 3), boundary=bnd, valence=val, idx=idx, n_cells=c.n_cells)


def process(N, pos, boundary, valence, idx, iters, process_boundary=False, smooth_normals=False, nrm=None):
    p = np.ascontiguousarray(pos, np.float32).reshape(-1).copy()
    n = np.zeros_like(p) if nrm is None else np.ascontiguousarray(nrm, np.float32).reshape(-1).copy()
    b = np.ascontiguousarray(boundary, np.uint8)
    v = np.ascontiguousarray(valence, np.uint8)
    ix = np.ascontiguousarray(idx, np.uint32)
    lib().bmfo_process(N, len(b), _p(p), _p(n), _p(b), _p(v), len(ix), _p(ix), iters, int(process_boundary),
                       int(smooth_normals))
    return p.reshape(-1, 3), n.reshape(-1, 3)


def lod_generate(root_pos, root_size, focus, split_multiplier, size_modifier, min_level, max_level, dim,
                 base_overlap=0.035, boundary_processing=False, iters=0, cap=1 << 16):
    """WorldOctree::split_leaves restated: (n, 6) float32 rows (origin xyz,
    scale, dim, level) in the reference's leaf order."""
    prm = np.array(list(root_pos) + [root_size] + list(focus) + [split_multiplier, size_modifier, base_overlap],
                   np.float32)
    out = np.zeros((cap, 6), np.float32)
    n = lib().bmfo_lod_generate(_p(prm), min_level, max_level, dim, int(boundary_processing), iters, _p(out), cap)
    assert 0 <= n <= cap
    return out[:n]


def format_data(pos, nrm, idx, unwind, smooth_normals):
    """GLChunk::format_data restated: returns (p, n, c) as (count, 3) float32."""
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    nrm = None if nrm is None else np.ascontiguousarray(nrm, np.float32).reshape(-1, 3)
    idx = np.ascontiguousarray(idx, np.uint32)
    cnt = len(idx) // 4 * 4 if unwind else len(pos)
    p, n, c = (np.zeros((max(cnt, 1), 3), np.float32) for _ in range(3))
    got = lib().bmfo_format(len(pos), _p(pos), _p(nrm), len(idx), _p(idx), int(unwind), int(smooth_normals),
                            _p(p), _p(n), _p(c))
    assert got == cnt
    return p[:cnt], n[:cnt], c[:cnt]


def qef_f32(pos, nrm):
    pos = np.ascontiguousarray(pos, np.float32)
    nrm = np.ascontiguousarray(nrm, np.float32)
    out = np.zeros(3, np.float32)
    e = lib().bmfo_qef_f32(_p(pos), _p(nrm), len(pos), _p(out))
    return out, e


def qef_f64(pos, nrm):
    pos = np.ascontiguousarray(pos, np.float64)
    nrm = np.ascontiguousarray(nrm, np.float64)
    out = np.zeros(3, np.float64)
    e = lib().bmfo_qef_f64(_p(pos), _p(nrm), len(pos), _p(out))
    return out, e


def extract_batch(desc, field, params, mode=0, placement=0, iters=0, smooth_normals=False, n_threads=0):
    """Whole CPU path over a batch of chunks (OpenMP over chunks).  desc: (n, 5)
    float32 rows {origin xyz, scale, dim}.  Returns (total vertices, counts (n, 3))."""
    desc = np.ascontiguousarray(desc, np.float32)
    prm = np.zeros(8, np.float32)
    prm[: len(params)] = params
    counts = np.zeros((len(desc), 3), np.int64)
    tot = lib().bmfo_extract_batch(len(desc), _p(desc), field, _p(prm), mode, placement, iters,
                                   int(smooth_normals), _p(counts), n_threads)
    return int(tot), counts


def extract_batch_digest(desc, field, params, mode=0, placement=0, iters=0, process_boundary=False,
                         smooth_normals=False, n_threads=0):
    """The CPU path over a batch with per-chunk digests.  Returns (counts (n, 3)
    = {contains_mesh, vertices, indices}, digests (n, 4) uint64 = digest64 of
    {indices, positions, boundary flags, normals})."""
    desc = np.ascontiguousarray(desc, np.float32)
    prm = np.zeros(8, np.float32)
    prm[: len(params)] = params
    counts = np.zeros((len(desc), 3), np.int64)
    dig = np.zeros((len(desc), 4), np.uint64)
    lib().bmfo_extract_batch_digest(len(desc), _p(desc), field, _p(prm), mode, placement, iters,
                                    int(process_boundary), int(smooth_normals), _p(counts), _p(dig), n_threads)
    return counts, dig


def digest64(a, f32=None):
    """The oracle's FNV-1a digest of an array's bytes (floats NaN-canonicalised)."""
    a = np.ascontiguousarray(a)
    if f32 is None:
        f32 = a.dtype == np.float32
    return int(lib().bmfo_digest64(_p(a) if a.size else None, a.nbytes, int(f32)))


def chunk_digests(pos, idx, boundary, nrm):
    """digest64 of one chunk's {indices, positions, boundary flags, normals} as
    host arrays, in the order extract_batch_digest reports them."""
    pos = np.ascontiguousarray(pos, np.float32)
    nv = pos.size // 3
    nrm = np.zeros((nv, 3), np.float32) if nrm is None else np.ascontiguousarray(nrm, np.float32)
    bnd = np.zeros(nv, np.uint8) if boundary is None else np.ascontiguousarray(boundary, np.uint8)
    return (digest64(np.ascontiguousarray(idx).view(np.uint32)), digest64(pos), digest64(bnd), digest64(nrm))


def fit_loss_f64(dim, density, iters, box, want_grad=False, near_branch=None):
    """FP64 differentiable path: returns (loss, grad or None, counts, state_hash).
    near_branch (uint8 array of dim^3, optional) receives the mask of samples
    read by vertices whose placement branch a float32 forward may take
    differently."""
    d = np.ascontiguousarray(density, np.float64)
    b = np.ascontiguousarray(box, np.float64)
    g = np.zeros(dim ** 3, np.float64) if want_grad else None
    counts = np.zeros(3, np.int64)
    h = ctypes.c_uint64(0)
    loss = lib().bmfo_fit_loss_f64(dim, _p(d), iters, _p(b), _p(g), _p(counts), ctypes.byref(h), _p(near_branch))
    return loss, g, counts, int(h.value)


def fit_loss_spheres_f64(dim, density, iters, spheres, want_grad=False, near_branch=None):
    """FP64 differentiable path with a sphere-union target (spheres: (k, 4) rows
    of centre xyz, radius): returns (loss, grad or None, counts, state_hash)."""
    d = np.ascontiguousarray(density, np.float64)
    sp = np.ascontiguousarray(spheres, np.float64).reshape(-1, 4)
    g = np.zeros(dim ** 3, np.float64) if want_grad else None
    counts = np.zeros(3, np.int64)
    h = ctypes.c_uint64(0)
    loss = lib().bmfo_fit_loss_spheres_f64(dim, _p(d), iters, _p(sp), len(sp), _p(g), _p(counts), ctypes.byref(h),
                                           _p(near_branch))
    return loss, g, counts, int(h.value)
