"""Failure handling through the C ABI, with every failure made on the host:
corrupt chunk descriptors and field parameters, an output arena of capacity 1,
and a bounded host-side wait that runs out.  None of these faults, traps or
hangs the GPU: descriptors are rejected before any launch, overflowing chunks
are skipped by the emit kernels (their status says so), and the wait only
polls an event."""
import ctypes
import math

import numpy as np
import pytest
import torch

from binarymeshfitting_gb300 import _lib as L
from binarymeshfitting_gb300 import workloads
from binarymeshfitting_gb300.engine import Batch

pytestmark = pytest.mark.gpu

BAD_DESCS = [((math.nan, 0.0, 0.0), 1.0, 33), ((0.0, math.inf, 0.0), 1.0, 33), ((0.0, 0.0, -math.inf), 1.0, 33),
             ((0.0, 0.0, 0.0), 0.0, 33), ((0.0, 0.0, 0.0), -1.0, 33), ((0.0, 0.0, 0.0), math.nan, 33),
             ((0.0, 0.0, 0.0), math.inf, 33), ((0.0, 0.0, 0.0), 1.0, 1), ((0.0, 0.0, 0.0), 1.0, -5),
             ((0.0, 0.0, 0.0), 1.0, 5000)]


@pytest.mark.parametrize("origin,scale,dim", BAD_DESCS)
def test_corrupt_descriptor_is_rejected_everywhere(ctx, origin, scale, dim):
    """Called straight through the C ABI with small buffers: the library
    rejects the descriptor before it sizes or touches anything."""
    desc = L.ChunkDesc.make(origin, scale, dim)
    field = workloads.terrain_field()
    good = L.ChunkDesc.make((0.0, 48.0, 0.0), 1.0, 33)  # holds the terrain surface
    lib, h = ctx.lib, ctx.h
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    buf = torch.empty(33 ** 3, device="cuda")
    words = torch.empty(33 * 33 * 2, dtype=torch.int32, device="cuda")
    cm = ctypes.c_int32(0)
    m, _ = ctx._alloc_mesh(4096, 16384, True)
    opts = L.ExtractOpts(L.MODE_R, 0, 2, 0, 1, 0)
    for status in (lib.bmf_sample_block(h, ctypes.byref(desc), ctypes.byref(field), ctypes.c_void_p(buf.data_ptr()),
                                        st),
                   lib.bmf_sample_label(h, ctypes.byref(desc), ctypes.byref(field), ctypes.c_void_p(buf.data_ptr()),
                                        ctypes.c_void_p(words.data_ptr()), ctypes.byref(cm), st),
                   lib.bmf_extract_chunk(h, ctypes.byref(desc), ctypes.byref(field), ctypes.byref(opts),
                                         ctypes.byref(m), st)):
        assert status == L.ERR_INVALID_ARGUMENT
    # one bad descriptor among good ones fails the whole plan, naming the chunk
    with pytest.raises(L.BmfError) as e:
        Batch(ctx, [good, good, desc, good], field)
    assert e.value.status == L.ERR_INVALID_ARGUMENT and "chunk 2" in str(e.value)
    # the context is still usable
    m = ctx.extract_chunk(good, field)
    assert m.n_verts > 0


def test_set_descs_rejects_a_corrupt_frame_and_keeps_the_plan(ctx):
    descs, _ = workloads.lod_update(n=8, seed=4)
    for d in descs:
        d.dim = 17
    b = Batch(ctx, descs, workloads.terrain_field(), mode=L.MODE_R, iters=2, smooth_normals=True)
    b.allocate(200000, 1200000, normals=True)
    before = b.run(use_graph=True)
    bad = [L.ChunkDesc.make(d.origin, d.scale, d.dim) for d in descs]
    bad[5].origin[1] = math.nan
    with pytest.raises(L.BmfError) as e:
        b.set_descs(bad)
    assert e.value.status == L.ERR_INVALID_ARGUMENT
    assert b.run(use_graph=True) == before  # the old descriptors are still in place
    b.close()


def test_non_finite_field_parameter_is_rejected(ctx):
    params = list(workloads.TERRAIN_PARAMS)
    params[2] = math.nan  # frequency
    with pytest.raises(L.BmfError) as e:
        ctx.sample_block(L.ChunkDesc.make((0, 0, 0), 1.0, 17), L.Field.make(L.FIELD_TERRAIN_FBM, params))
    assert e.value.status == L.ERR_INVALID_ARGUMENT


def test_batch_with_capacity_one_writes_nothing_out_of_bounds(ctx):
    """An arena of one vertex and one index: BMF_ERR_CAPACITY with the needed
    totals; every chunk with a mesh reports status 3 in the chunk table; the
    guard regions after the capacities stay untouched; the plan then runs
    correctly once the arena is large enough."""
    descs, _ = workloads.lod_update(n=64, seed=6)
    for d in descs:
        d.dim = min(d.dim, 33)
    b = Batch(ctx, descs, workloads.terrain_field(), mode=L.MODE_R, iters=2, smooth_normals=True)
    guard = 1 << 16
    dev = torch.device("cuda", 0)
    pos = torch.full((1 + guard, 3), -7.0, device=dev)
    nrm = torch.full((1 + guard, 3), -7.0, device=dev)
    bnd = torch.full((1 + guard,), 9, dtype=torch.uint8, device=dev)
    idx = torch.full((1 + guard,), -1, dtype=torch.int32, device=dev)
    info = torch.zeros((len(descs), 6), dtype=torch.int64, device=dev)
    b.bufs = dict(pos=pos, nrm=nrm, boundary=bnd, idx=idx, info=info)
    b.out = L.BatchOut(pos.data_ptr(), nrm.data_ptr(), bnd.data_ptr(), idx.data_ptr(), 1, 1, info.data_ptr(), 0, 0)
    for use_graph in (False, True):
        with pytest.raises(L.BmfError) as e:
            b.run(use_graph=use_graph)
        assert e.value.status == L.ERR_CAPACITY
        need_v, need_i = int(b.out.n_verts), int(b.out.n_idx)
        assert need_v > 1 and need_i > 1
        torch.cuda.synchronize()
        assert (pos[1:] == -7.0).all() and (nrm[1:] == -7.0).all()
        assert (bnd[1:] == 9).all() and (idx[1:] == -1).all()
        tab = info.cpu().numpy()
        assert (tab[tab[:, 1] > 0, 5] == 3).all()
        assert int(tab[:, 1].sum()) == need_v and int(tab[:, 3].sum()) == need_i
    b.allocate(need_v, need_i, normals=True)
    assert b.run(use_graph=True) == (need_v, need_i)
    assert (b.bufs["info"][:, 5] == 0).all()
    b.close()


def test_bounded_wait_times_out_then_completes(ctx):
    """bmf_batch_wait with a 0 ms budget right after enqueueing several updates
    returns BMF_ERR_TIMEOUT (the GPU is still working; nothing is cancelled);
    a longer wait then returns the same totals as a synchronous run."""
    descs, _ = workloads.lod_update(n=2048, seed=8)
    b = Batch(ctx, descs, workloads.terrain_field(), mode=L.MODE_R, iters=4, smooth_normals=True)
    vcap, icap = 20_000_000, 120_000_000
    b.allocate(vcap, icap, normals=True)
    want = b.run(use_graph=True, sync=True)
    for _ in range(4):  # tens of milliseconds of queued GPU work
        b.run(use_graph=True, sync=False)
    with pytest.raises(L.BmfError) as e:
        b.wait(0)
    assert e.value.status == L.ERR_TIMEOUT
    assert b.wait(60_000) == want
    assert b.wait(0) == want  # already done: a zero budget succeeds
    b.close()
    idle = Batch(ctx, descs[:4], workloads.terrain_field())
    idle.allocate(1 << 20, 1 << 22)
    with pytest.raises(L.BmfError) as e:
        idle.wait(0)  # never ran
    assert e.value.status == L.ERR_INVALID_ARGUMENT
    idle.close()
