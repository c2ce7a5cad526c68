"""Python host layer over the C ABI: device buffers are torch tensors, every
compute call goes through libbmf_gb300.so (no CPU path)."""
import ctypes

import numpy as np
from dataclasses import dataclass
from typing import Optional

import torch

from . import _lib as L


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def zpad(dim):
    return 32 * ((dim + 31) // 32)


def n_words(dim):
    return dim * dim * ((dim + 31) // 32)


@dataclass
class ChunkMesh:
    """One chunk's mesh (a VerticesIndicesBlock as device tensors)."""
    pos: torch.Tensor            # (V, 3) float32, sample-index coordinates
    nrm: Optional[torch.Tensor]  # (V, 3) float32
    boundary: torch.Tensor       # (V,) uint8
    valence: torch.Tensor        # (V,) uint8 (init_valence)
    idx: torch.Tensor            # (P * prim_size,) int32 view of uint32 indices
    contains_mesh: bool
    prim_size: int

    @property
    def n_verts(self):
        return self.pos.shape[0]

    @property
    def n_idx(self):
        return self.idx.shape[0]


class Context:
    """A bmf_ctx bound to one CUDA device (not thread-safe, like the C ABI)."""

    def __init__(self, device=0):
        if not torch.cuda.is_available():
            raise RuntimeError("binarymeshfitting_gb300 needs a CUDA device (no CPU fallback)")
        self.lib = L.load()
        self.device = torch.device("cuda", device)
        cfg = L.Config(device, 0, 0)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            L.check(self.lib.bmf_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.bmf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, status):
        L.check(status, self.h, self.lib)

    @property
    def launches(self):
        return int(self.lib.bmf_launch_count(self.h))

    # -- stages -------------------------------------------------------------
    def sample_block(self, desc: L.ChunkDesc, field: L.Field, out=None, stream=None):
        d = desc.dim
        out = out if out is not None else torch.empty(d ** 3, dtype=torch.float32, device=self.device)
        self._check(self.lib.bmf_sample_block(self.h, ctypes.byref(desc), ctypes.byref(field), _ptr(out),
                                              _stream(stream)))
        return out

    def sample_label(self, desc: L.ChunkDesc, field: L.Field, want_density=True, stream=None):
        d = desc.dim
        dens = torch.empty(d ** 3, dtype=torch.float32, device=self.device) if want_density else None
        words = torch.empty(n_words(d), dtype=torch.int32, device=self.device)
        cm = ctypes.c_int32(0)
        self._check(self.lib.bmf_sample_label(self.h, ctypes.byref(desc), ctypes.byref(field), _ptr(dens),
                                              _ptr(words), ctypes.byref(cm), _stream(stream)))
        return dens, words, bool(cm.value)

    def label_grid(self, dim, density, stream=None):
        words = torch.empty(n_words(dim), dtype=torch.int32, device=self.device)
        cm = ctypes.c_int32(0)
        density = density.contiguous()
        self._check(self.lib.bmf_label_grid(self.h, dim, _ptr(density), _ptr(words), ctypes.byref(cm),
                                            _stream(stream)))
        return words, bool(cm.value)

    def cell_masks(self, dim, words, stream=None):
        masks = torch.empty(dim * dim * zpad(dim), dtype=torch.uint8, device=self.device)
        self._check(self.lib.bmf_cell_masks(self.h, dim, _ptr(words), _ptr(masks), _stream(stream)))
        return masks

    def _alloc_mesh(self, vcap, icap, normals):
        pos = torch.empty((max(vcap, 1), 3), dtype=torch.float32, device=self.device)
        nrm = torch.zeros((max(vcap, 1), 3), dtype=torch.float32, device=self.device) if normals else None
        bnd = torch.empty(max(vcap, 1), dtype=torch.uint8, device=self.device)
        val = torch.empty(max(vcap, 1), dtype=torch.uint8, device=self.device)
        idx = torch.empty(max(icap, 1), dtype=torch.int32, device=self.device)
        m = L.Mesh(pos.data_ptr(), nrm.data_ptr() if nrm is not None else None, bnd.data_ptr(), val.data_ptr(),
                   idx.data_ptr(), vcap, icap, 0, 0, 0, 0)
        return m, (pos, nrm, bnd, val, idx)

    @staticmethod
    def _trim(m, bufs):
        pos, nrm, bnd, val, idx = bufs
        nv, ni = m.n_verts, m.n_idx
        return ChunkMesh(pos[:nv], nrm[:nv] if nrm is not None else None, bnd[:nv], val[:nv], idx[:ni],
                         bool(m.contains_mesh), m.prim_size)

    def _with_capacity(self, dim, call, normals):
        vcap, icap = max(1024, dim ** 3 // 16), max(4096, dim ** 3 // 3)
        for _ in range(2):
            m, bufs = self._alloc_mesh(vcap, icap, normals)
            st = call(m)
            if st == L.ERR_CAPACITY:
                vcap, icap = int(m.n_verts), int(m.n_idx)
                continue
            self._check(st)
            return m, bufs
        self._check(st)

    def polygonize(self, dim, density, words, mode=L.MODE_R, placement=L.PLACE_CENTER, normals=False, stream=None):
        dens = density.contiguous() if density is not None else None

        def call(m):
            return self.lib.bmf_polygonize(self.h, dim, _ptr(dens), _ptr(words), mode, placement, ctypes.byref(m),
                                           _stream(stream))

        m, bufs = self._with_capacity(dim, call, normals)
        return self._trim(m, bufs)

    def process(self, mesh: ChunkMesh, iters, process_boundary=False, smooth_normals=False, stream=None):
        """MeshProcessor<N> in place on mesh.pos (and mesh.nrm when present)."""
        m = L.Mesh(mesh.pos.data_ptr(), mesh.nrm.data_ptr() if mesh.nrm is not None else None,
                   mesh.boundary.data_ptr(), mesh.valence.data_ptr(), mesh.idx.data_ptr(), mesh.n_verts,
                   mesh.n_idx, mesh.n_verts, mesh.n_idx, int(mesh.contains_mesh), mesh.prim_size)
        self._check(self.lib.bmf_process(self.h, ctypes.byref(m), iters, int(process_boundary),
                                         int(smooth_normals), _stream(stream)))
        return mesh

    def lod_generate(self, root_pos, root_size, focus, split_multiplier=1.0, size_modifier=0.0, min_level=1,
                     max_level=7, dim=33, base_overlap=0.035, boundary_processing=False, iters=0, cap=16384,
                     stream=None):
        """WorldOctree split policy on the device: (n, 6) int32 tensor of
        bmf_chunk_desc rows (origin xyz and scale as float32 bits, dim, level)
        in the reference's leaf order."""
        p = L.LodParams()
        for i in range(3):
            p.root_pos[i] = float(root_pos[i])
            p.focus[i] = float(focus[i])
        p.root_size, p.split_multiplier, p.size_modifier = float(root_size), float(split_multiplier), float(size_modifier)
        p.min_level, p.max_level, p.dim = int(min_level), int(max_level), int(dim)
        p.base_overlap, p.boundary_processing, p.iters = float(base_overlap), int(boundary_processing), int(iters)
        rows = torch.empty((cap, 6), dtype=torch.int32, device=self.device)
        cnt = torch.zeros(1, dtype=torch.int32, device=self.device)
        self._check(self.lib.bmf_lod_generate(self.h, ctypes.byref(p), _ptr(rows), cap, _ptr(cnt), _stream(stream)))
        n = int(cnt.item())
        if n < 0:
            raise L.BmfError(L.ERR_CAPACITY, "more leaves than cap=%d" % cap)
        return rows[:n]

    @staticmethod
    def descs_from_rows(rows):
        """Host bmf_chunk_desc list from lod_generate rows."""
        r = rows.cpu().numpy()
        f = r[:, :4].copy().view(np.float32)
        return [L.ChunkDesc.make(f[i, :3], f[i, 3], int(r[i, 4]), int(r[i, 5])) for i in range(len(r))]

    def format(self, mesh: ChunkMesh, unwind=False, smooth_normals=False, stream=None):
        """GLChunk::format_data: (p, n, c) device tensors of shape (count, 3)."""
        m = L.Mesh(mesh.pos.data_ptr(), mesh.nrm.data_ptr() if mesh.nrm is not None else None,
                   mesh.boundary.data_ptr(), mesh.valence.data_ptr(), mesh.idx.data_ptr(), mesh.n_verts,
                   mesh.n_idx, mesh.n_verts, mesh.n_idx, int(mesh.contains_mesh), mesh.prim_size)
        cnt = mesh.n_idx // 4 * 4 if unwind else mesh.n_verts
        p, n, c = (torch.empty((max(cnt, 1), 3), dtype=torch.float32, device=self.device) for _ in range(3))
        got = ctypes.c_int64(0)
        self._check(self.lib.bmf_format(self.h, ctypes.byref(m), int(unwind), int(smooth_normals), _ptr(p), _ptr(n),
                                        _ptr(c), cnt, ctypes.byref(got), _stream(stream)))
        return p[:got.value], n[:got.value], c[:got.value]

    def extract_chunk(self, desc: L.ChunkDesc, field: L.Field, mode=L.MODE_R, placement=L.PLACE_CENTER, iters=0,
                      process_boundary=False, smooth_normals=False, stream=None):
        opts = L.ExtractOpts(mode, placement, iters, int(process_boundary), int(smooth_normals), 0)
        normals = smooth_normals

        def call(m):
            return self.lib.bmf_extract_chunk(self.h, ctypes.byref(desc), ctypes.byref(field), ctypes.byref(opts),
                                              ctypes.byref(m), _stream(stream))

        m, bufs = self._with_capacity(desc.dim, call, normals)
        return self._trim(m, bufs)


class Batch:
    """A batched update plan (bmf_batch): one CUDA graph per output arena."""

    def __init__(self, ctx: Context, descs, field: L.Field, mode=L.MODE_R, placement=L.PLACE_CENTER, iters=0,
                 process_boundary=False, smooth_normals=False):
        self.ctx = ctx
        self.n = len(descs)
        arr = (L.ChunkDesc * self.n)(*descs)
        self.descs = arr
        self.opts = L.ExtractOpts(mode, placement, iters, int(process_boundary), int(smooth_normals), 0)
        self.field = field
        self.mode = mode
        h = ctypes.c_void_p()
        ctx._check(ctx.lib.bmf_batch_create(ctx.h, arr, self.n, ctypes.byref(field), ctypes.byref(self.opts),
                                            ctypes.byref(h)))
        self.h = h
        self.out = None
        self.bufs = None

    def allocate(self, vcap, icap, normals=False, boundary=True):
        dev = self.ctx.device
        pos = torch.empty((max(vcap, 1), 3), dtype=torch.float32, device=dev)
        nrm = torch.zeros((max(vcap, 1), 3), dtype=torch.float32, device=dev) if normals else None
        bnd = torch.empty(max(vcap, 1), dtype=torch.uint8, device=dev) if boundary else None
        idx = torch.empty(max(icap, 1), dtype=torch.int32, device=dev)
        info = torch.zeros((self.n, 6), dtype=torch.int64, device=dev)
        self.bufs = dict(pos=pos, nrm=nrm, boundary=bnd, idx=idx, info=info)
        self.out = L.BatchOut(pos.data_ptr(), nrm.data_ptr() if nrm is not None else None,
                              bnd.data_ptr() if bnd is not None else None, idx.data_ptr(), vcap, icap,
                              info.data_ptr(), 0, 0)
        return self.bufs

    def run(self, use_graph=True, sync=True, stream=None):
        self.ctx._check(self.ctx.lib.bmf_batch_run(self.h, ctypes.byref(self.out), int(use_graph), int(sync),
                                                   _stream(stream)))
        return int(self.out.n_verts), int(self.out.n_idx)

    def wait(self, timeout_ms):
        """bmf_batch_wait: waits at most timeout_ms for the last run; returns
        (vertices, indices).  Raises BmfError(ERR_TIMEOUT) when the update is
        still running (nothing is cancelled; wait again)."""
        self.ctx._check(self.ctx.lib.bmf_batch_wait(self.h, ctypes.byref(self.out), int(timeout_ms)))
        return int(self.out.n_verts), int(self.out.n_idx)

    def wait_extraction(self, stream=None):
        """bmf_batch_wait_extraction: `stream` (default: the current one) waits on
        the device until the last run's extraction is done -- indices and chunk
        table final -- while its smoothing may still run."""
        self.ctx._check(self.ctx.lib.bmf_batch_wait_extraction(self.h, _stream(stream)))

    def set_descs(self, descs, stream=None):
        arr = (L.ChunkDesc * self.n)(*descs)
        self.ctx._check(self.ctx.lib.bmf_batch_set_descs(self.h, arr, self.n, _stream(stream)))

    def profile(self, stream=None):
        """Stage times (ms) of one update: fill+label, count, scan, offsets, emit, processing."""
        ms = (ctypes.c_float * 6)()
        self.ctx._check(self.ctx.lib.bmf_batch_profile(self.h, ctypes.byref(self.out), ms, _stream(stream)))
        return list(ms)

    def format(self, unwind=False, smooth_normals=False, stream=None):
        """GLChunk::format_data over the whole arena of the last run: (p, n, c)."""
        cnt = self.out.n_idx // 4 * 4 if unwind else self.out.n_verts
        p, n, c = (torch.empty((max(cnt, 1), 3), dtype=torch.float32, device=self.ctx.device) for _ in range(3))
        self.ctx._check(self.ctx.lib.bmf_batch_format(self.h, ctypes.byref(self.out), int(unwind), int(smooth_normals),
                                                      _ptr(p), _ptr(n), _ptr(c), cnt, _stream(stream)))
        return p[:cnt], n[:cnt], c[:cnt]

    def tuning(self):
        """The plan's launch tuning as a dict (bmf_batch_tuning)."""
        t = L.BatchTuning()
        self.ctx._check(self.ctx.lib.bmf_batch_get_tuning(self.h, ctypes.byref(t)))
        return dict(fill_mode=t.fill_mode, fill_run=t.fill_run, sweep_block=t.sweep_block, fill_band=t.fill_band)

    def set_tuning(self, fill_mode=None, fill_run=None, sweep_block=None, fill_band=None):
        t = L.BatchTuning()
        self.ctx._check(self.ctx.lib.bmf_batch_get_tuning(self.h, ctypes.byref(t)))
        if fill_mode is not None:
            t.fill_mode = fill_mode
        if fill_run is not None:
            t.fill_run = fill_run
        if sweep_block is not None:
            t.sweep_block = sweep_block
        if fill_band is not None:
            t.fill_band = fill_band
        self.ctx._check(self.ctx.lib.bmf_batch_set_tuning(self.h, ctypes.byref(t)))

    def autotune(self, reps=3, stream=None):
        """Runs the plan's autotuner on the allocated arena; returns (chosen
        tuning dict, median ms per candidate)."""
        t = L.BatchTuning()
        ms = (ctypes.c_float * 16)()
        n = ctypes.c_int32(0)
        self.ctx._check(self.ctx.lib.bmf_batch_autotune(self.h, ctypes.byref(self.out), reps, _stream(stream),
                                                        ctypes.byref(t), ms, 16, ctypes.byref(n)))
        return (dict(fill_mode=t.fill_mode, fill_run=t.fill_run, sweep_block=t.sweep_block, fill_band=t.fill_band),
                [float(ms[i]) for i in range(min(n.value, 16))])

    def chunk_mesh(self, i):
        """Views of chunk i's vertices and (chunk-local) indices in the arena."""
        info = self.bufs["info"][i].tolist()
        vo, vc, io, ic = info[0], info[1], info[2], info[3]
        b = self.bufs
        return dict(pos=b["pos"][vo:vo + vc], nrm=b["nrm"][vo:vo + vc] if b["nrm"] is not None else None,
                    boundary=b["boundary"][vo:vo + vc] if b["boundary"] is not None else None,
                    idx=b["idx"][io:io + ic], contains_mesh=bool(info[4]), status=int(info[5]))

    def close(self):
        if self.h:
            self.ctx.lib.bmf_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
