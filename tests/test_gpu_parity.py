"""GPU path (libbmf_gb300.so through the C ABI) against the CPU oracle and the
golden fixtures generated from the reference's own code.

Bar: bit-exact for occupancy words, masks, counts, index buffers, boundary
flags and valences; vertex positions and normals bit-exact too (the kernels
keep the reference's single-precision operation order, --fmad=false), with
the path's stated tolerance of 1e-5 cell size reported alongside.
"""
import hashlib
import json
import os

import numpy as np
import pytest
import torch

from binarymeshfitting_gb300 import _lib as L
from binarymeshfitting_gb300 import workloads
from oracle import cpu
from tests.golden.cases import CASES, PROCESS_CASES, make_density

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "golden.json")))
GOLD_CASES = {c["name"]: c for c in GOLD["cases"]}
POS_TOL = 1e-5  # cell sizes (positions are in sample-index units)


def sha(a):
    """SHA-256 of the raw bytes; float NaNs are first canonicalised (x86, Arm and
    the GPU encode a NaN's sign and payload differently)."""
    a = np.ascontiguousarray(a)
    if a.dtype == np.float32:
        a = a.copy()
        a[np.isnan(a)] = np.float32("nan")
        a = np.where(np.isnan(a), np.uint32(0x7FC00000).view(np.float32), a)
    return hashlib.sha256(a.tobytes()).hexdigest()


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def assert_float_exact(gpu, ref, what):
    gpu = np.asarray(gpu, np.float32)
    ref = np.asarray(ref, np.float32)
    assert gpu.shape == ref.shape, what
    both_nan = np.isnan(gpu) & np.isnan(ref)
    diff = np.where(both_nan, 0.0, np.abs(gpu.astype(np.float64) - ref.astype(np.float64)))
    assert np.nanmax(diff, initial=0.0) <= POS_TOL, "%s: max |diff| %g > %g" % (what, np.nanmax(diff), POS_TOL)
    same = (bits(gpu) == bits(ref)) | both_nan
    assert same.all(), "%s: %d of %d values not bit-identical" % (what, (~same).sum(), same.size)


def dev(a, dtype=None):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def np_u32(t):
    return t.cpu().numpy().view(np.uint32)


EXTRA = [dict(name="uniform_%d" % d, dim=d, kind="uniform", seed=100 + d, lo=-1.0, hi=1.0)
         for d in (2, 3, 5, 17, 33, 65, 129)]
EXTRA += [dict(name="sphere_wave_%d" % d, dim=d, kind="field", field=1,
               params=[d / 2.0, d / 2.0, d / 2.0, d * 0.3, 1.5, 0.3], origin=[0, 0, 0], scale=1.0)
          for d in (33, 65, 129)]
EXTRA += [dict(name="all_inside_65", dim=65, kind="constant", value=-1.0),
          dict(name="all_outside_33", dim=33, kind="constant", value=0.0)]
ALL = CASES + EXTRA


@pytest.mark.parametrize("kind,params", [
    (L.FIELD_SPHERE_WAVE, workloads.SPHERE_WAVE_PARAMS), (L.FIELD_TERRAIN_FBM, workloads.TERRAIN_PARAMS),
    (L.FIELD_TORUS_Z, [64.0]), (L.FIELD_SPHERE, [64.0]), (L.FIELD_CUBOID, [64.0]), (L.FIELD_PLANE_Y, [64.0]),
    (L.FIELD_TERRAIN_2D, workloads.TERRAIN_2D_PARAMS)])
@pytest.mark.parametrize("dim,origin,scale", [(33, (-16.5, 3.25, -8.0), 1.0), (65, (0.0, 0.0, 0.0), 1.0),
                                              (65, (1024.0, 0.0, 512.0), 4.0)])
def test_field_fill_bit_exact(ctx, kind, params, dim, origin, scale):
    desc = L.ChunkDesc.make(origin, scale, dim)
    field = L.Field.make(kind, params)
    g = ctx.sample_block(desc, field).cpu().numpy()
    o = cpu.fill_field(kind, list(params), dim, origin, scale)
    assert_float_exact(g, o, "density")


@pytest.mark.parametrize("dim", [2, 3, 17, 30, 32, 47, 129])
@pytest.mark.parametrize("octaves", [0, 1, 5, 7, 9])
def test_terrain_fill_line_kernel_sizes(ctx, dim, octaves):
    """The line-mapped terrain kernel: ragged runs (partial last runs of 1 to
    15 samples), word ends, octave counts with and without the cell-state cache
    (more than 8 octaves rebuild it every run)."""
    params = list(workloads.TERRAIN_PARAMS)
    params[5] = octaves
    desc = L.ChunkDesc.make((37.0, -20.0, 1000.25), 2.0, dim)
    field = L.Field.make(L.FIELD_TERRAIN_FBM, params)
    g = ctx.sample_block(desc, field).cpu().numpy()
    o = cpu.fill_field(L.FIELD_TERRAIN_FBM, params, dim, (37.0, -20.0, 1000.25), 2.0)
    assert_float_exact(g, o, "density")
    ow, ocm = cpu.label_grid(dim, o)
    for want_density in (True, False):
        dens, words, cm = ctx.sample_label(desc, field, want_density=want_density)
        if want_density:
            assert_float_exact(dens.cpu().numpy(), o, "density")
        assert np.array_equal(np_u32(words), ow) and cm == bool(ocm)


@pytest.mark.parametrize("case", ALL, ids=[c["name"] for c in ALL])
def test_label_masks_mode_r(ctx, case):
    dim = case["dim"]
    d = make_density(case)
    words_t, cm = ctx.label_grid(dim, dev(d))
    words = np_u32(words_t)
    ow, ocm = cpu.label_grid(dim, d)
    np.testing.assert_array_equal(words, ow)
    assert cm == bool(ocm)
    masks = ctx.cell_masks(dim, words_t).cpu().numpy()
    om = cpu.cell_masks(dim, ow)
    np.testing.assert_array_equal(masks, om.view(np.uint8))
    g = GOLD_CASES.get(case["name"])
    if g is not None and g["dim"] == dim:
        assert sha(words) == g["words_sha"]
        if g["contains_mesh"]:
            assert sha(masks.view(np.uint64)) == g["masks_sha"]
    if not ocm:
        return
    m = ctx.polygonize(dim, dev(d), words_t, mode=L.MODE_R)
    O = cpu.extract_r(dim, d, om)
    assert m.n_verts == len(O["pos"]) and m.n_idx == len(O["idx"])
    assert_float_exact(m.pos.cpu().numpy(), O["pos"], "positions")
    np.testing.assert_array_equal(m.boundary.cpu().numpy(), O["boundary"])
    np.testing.assert_array_equal(m.valence.cpu().numpy(), O["valence"])
    np.testing.assert_array_equal(np_u32(m.idx), O["idx"])
    if g is not None and g["dim"] == dim:
        assert sha(m.pos.cpu().numpy()) == g["pos_sha"]
        assert sha(np_u32(m.idx)) == g["idx_sha"]
        assert sha(m.valence.cpu().numpy()) == g["valence_sha"]
        assert sha(m.boundary.cpu().numpy()) == g["boundary_sha"]


@pytest.mark.parametrize("placement", [L.PLACE_CENTER, L.PLACE_MASSPOINT, L.PLACE_QEF])
@pytest.mark.parametrize("name", ["sphere_wave_32", "terrain_fbm_64", "uniform_33", "uniform_3", "torus_64",
                                  "sphere_wave_129"])
def test_mode_q(ctx, name, placement):
    case = next(c for c in ALL if c["name"] == name)
    dim = case["dim"]
    d = make_density(case)
    words_t, cm = ctx.label_grid(dim, dev(d))
    m = ctx.polygonize(dim, dev(d), words_t, mode=L.MODE_Q, placement=placement)
    O = cpu.extract_q(dim, d, np_u32(words_t), placement)
    assert m.n_verts == len(O["pos"]) and m.n_idx == len(O["idx"])
    np.testing.assert_array_equal(np_u32(m.idx), O["idx"])
    np.testing.assert_array_equal(m.boundary.cpu().numpy(), O["boundary"])
    np.testing.assert_array_equal(m.valence.cpu().numpy(), O["valence"])
    assert_float_exact(m.pos.cpu().numpy(), O["pos"], "mode Q positions")


@pytest.mark.parametrize("rec", GOLD["process"], ids=lambda r: "%s-N%d-it%d-n%d-b%d" % (
    r["case"], r["N"], r["iters"], r["normals"], r["boundary"]))
def test_process_vs_reference(ctx, rec):
    base = next(c for c in CASES if c["name"] == rec["case"])
    dim = base["dim"]
    d = make_density(base)
    words_t, _ = ctx.label_grid(dim, dev(d))
    if rec["N"] == 3:
        m = ctx.polygonize(dim, dev(d), words_t, mode=L.MODE_R, normals=True)
    else:
        m = ctx.polygonize(dim, dev(d), words_t, mode=L.MODE_Q, placement=1, normals=True)
    ctx.process(m, rec["iters"], rec["boundary"], rec["normals"])
    pos, nrm = m.pos.cpu().numpy(), m.nrm.cpu().numpy()
    assert len(pos) == rec["n_verts"]
    # oracle chain for a readable diff first, then the reference digests
    if rec["N"] == 3:
        M = cpu.extract_r(dim, d, cpu.cell_masks(dim, cpu.label_grid(dim, d)[0]))
    else:
        M = cpu.extract_q(dim, d, cpu.label_grid(dim, d)[0], 1)
    op, on = cpu.process(rec["N"], M["pos"], M["boundary"], M["valence"], M["idx"], rec["iters"], rec["boundary"],
                         rec["normals"])
    assert_float_exact(pos, op, "smoothed positions")
    assert_float_exact(nrm, on, "normals")
    assert sha(pos) == rec["pos_sha"]
    assert sha(nrm) == rec["nrm_sha"]


@pytest.mark.parametrize("mode,placement,iters,normals", [(L.MODE_R, 0, 0, False), (L.MODE_R, 0, 4, True),
                                                          (L.MODE_Q, 0, 0, False), (L.MODE_Q, 1, 4, True),
                                                          (L.MODE_Q, 2, 4, True)])
def test_extract_chunk_sphere_wave_65(ctx, mode, placement, iters, normals):
    desc = L.ChunkDesc.make((0, 0, 0), 1.0, 65)
    m = ctx.extract_chunk(desc, workloads.sphere_wave_field(), mode=mode, placement=placement, iters=iters,
                          smooth_normals=normals)
    d = cpu.fill_field(1, list(workloads.SPHERE_WAVE_PARAMS), 65)
    w, cm = cpu.label_grid(65, d)
    assert m.contains_mesh == bool(cm)
    if mode == L.MODE_R:
        O = cpu.extract_r(65, d, cpu.cell_masks(65, w))
        N = 3
    else:
        O = cpu.extract_q(65, d, w, placement)
        N = 4
    op, on = O["pos"], np.zeros_like(O["pos"])
    if iters:
        op, on = cpu.process(N, O["pos"], O["boundary"], O["valence"], O["idx"], iters, False, normals)
    np.testing.assert_array_equal(np_u32(m.idx), O["idx"])
    assert_float_exact(m.pos.cpu().numpy(), op, "positions")
    if normals:
        assert_float_exact(m.nrm.cpu().numpy(), on, "normals")


def test_extract_chunk_terrain_129_with_smoothing(ctx):
    desc = L.ChunkDesc.make((0, 0, 0), 1.0, 129)
    m = ctx.extract_chunk(desc, workloads.terrain_field(), mode=L.MODE_Q, placement=L.PLACE_MASSPOINT, iters=4,
                          smooth_normals=True)
    d = cpu.fill_field(2, list(workloads.TERRAIN_PARAMS), 129)
    w, _ = cpu.label_grid(129, d)
    O = cpu.extract_q(129, d, w, 1)
    op, on = cpu.process(4, O["pos"], O["boundary"], O["valence"], O["idx"], 4, False, True)
    np.testing.assert_array_equal(np_u32(m.idx), O["idx"])
    assert_float_exact(m.pos.cpu().numpy(), op, "positions")
    assert_float_exact(m.nrm.cpu().numpy(), on, "normals")


def _small_batch(n=40, seed=5):
    descs, rows = workloads.lod_update(n=n, seed=seed)
    # keep the CPU-checked batch small: clamp 129-sample chunks to 65
    for dsc, r in zip(descs, rows):
        if dsc.dim > 65:
            dsc.dim = 65
            r[4] = 65
    return descs, rows


@pytest.mark.parametrize("mode,placement,iters", [(L.MODE_R, 0, 0), (L.MODE_R, 0, 4), (L.MODE_Q, 1, 4),
                                                  (L.MODE_Q, 2, 0)])
@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_matches_oracle_per_chunk(ctx, mode, placement, iters, use_graph):
    from binarymeshfitting_gb300.engine import Batch
    descs, rows = _small_batch()
    b = Batch(ctx, descs, workloads.terrain_field(), mode=mode, placement=placement, iters=iters,
              smooth_normals=iters > 0)
    b.allocate(400000, 2400000, normals=iters > 0)
    for rep in range(2):  # replay: same result
        nv, ni = b.run(use_graph=use_graph)
    tot_v = 0
    for i, r in enumerate(rows):
        dim = int(r[4])
        d = cpu.fill_field(2, list(workloads.TERRAIN_PARAMS), dim, r[:3], r[3])
        w, cm = cpu.label_grid(dim, d)
        got = b.chunk_mesh(i)
        assert got["contains_mesh"] == bool(cm) and got["status"] == 0
        if not cm:
            assert len(got["pos"]) == 0
            continue
        if mode == L.MODE_R:
            O = cpu.extract_r(dim, d, cpu.cell_masks(dim, w))
            N = 3
        else:
            O = cpu.extract_q(dim, d, w, placement)
            N = 4
        op = O["pos"]
        if iters:
            op, _ = cpu.process(N, O["pos"], O["boundary"], O["valence"], O["idx"], iters, False, True)
        np.testing.assert_array_equal(np_u32(got["idx"]), O["idx"])
        assert_float_exact(got["pos"].cpu().numpy(), op, "chunk %d positions" % i)
        np.testing.assert_array_equal(got["boundary"].cpu().numpy(), O["boundary"])
        tot_v += len(op)
    assert tot_v == nv
    b.close()


@pytest.mark.parametrize("mode", [L.MODE_R, L.MODE_Q])
def test_chunk_sweeps_match_whole_mesh_sweeps(ctx, mode):
    """A Mode R batch of 512 chunks or more (Mode Q: 2048) runs its sweeps
    chunk by chunk (one CTA per chunk); smaller batches run them as whole-mesh
    kernels.  Split into batches below the threshold, the same chunks give
    bit-identical positions, normals and indices; a sample of chunks also
    matches the oracle."""
    from binarymeshfitting_gb300.engine import Batch
    descs, rows = workloads.lod_update(n=2100, seed=9)
    for dsc, r in zip(descs, rows):  # small chunks keep the test quick
        dsc.dim = 17
        r[4] = 17
    kw = dict(mode=mode, placement=L.PLACE_MASSPOINT, iters=4, smooth_normals=True)
    big = Batch(ctx, descs, workloads.terrain_field(), **kw)
    big.allocate(3000000, 12000000, normals=True)
    nv, ni = big.run(use_graph=True)
    parts = [(k, k + 420) for k in range(0, 2100, 420)]  # below both thresholds
    got_v = 0
    checked = 0
    for lo, hi in parts:
        sub = Batch(ctx, descs[lo:hi], workloads.terrain_field(), **kw)
        sub.allocate(1500000, 6000000, normals=True)
        sv, si = sub.run(use_graph=True)
        got_v += sv
        for i in range(hi - lo):
            a, b_ = big.chunk_mesh(lo + i), sub.chunk_mesh(i)
            for k in ("pos", "nrm", "idx"):
                assert torch.equal(a[k].view(torch.int32) if a[k].is_floating_point() else a[k],
                                   b_[k].view(torch.int32) if b_[k].is_floating_point() else b_[k]), (lo + i, k)
            if a["contains_mesh"] and checked < 8 and len(a["pos"]) > 0:
                r = rows[lo + i]
                d = cpu.fill_field(2, list(workloads.TERRAIN_PARAMS), 17, r[:3], r[3])
                w, _ = cpu.label_grid(17, d)
                if mode == L.MODE_R:
                    O, N = cpu.extract_r(17, d, cpu.cell_masks(17, w)), 3
                else:
                    O, N = cpu.extract_q(17, d, w, L.PLACE_MASSPOINT), 4
                op, _ = cpu.process(N, O["pos"], O["boundary"], O["valence"], O["idx"], 4, False, True)
                assert_float_exact(a["pos"].cpu().numpy(), op, "chunk %d positions" % (lo + i))
                checked += 1
        sub.close()
    assert got_v == nv and checked == 8
    big.close()


def test_batch_tunings_give_identical_results(ctx):
    """Every launch tuning (fill kernel form, tile height, sweep block) changes
    speed only: the whole arena is bit-identical to the default's."""
    from binarymeshfitting_gb300.engine import Batch
    descs, rows = _small_batch()
    b = Batch(ctx, descs, workloads.terrain_field(), mode=L.MODE_R, iters=4, smooth_normals=True)
    bufs = b.allocate(400000, 2400000, normals=True)
    assert b.tuning() == dict(fill_mode=2, fill_run=16, sweep_block=256, fill_band=1)
    b.set_tuning(fill_band=0)  # the reference arena: every density exact
    nv, ni = b.run(use_graph=True)
    ref = [bufs[k][:n].clone() for k, n in (("pos", nv), ("nrm", nv), ("idx", ni))] + [bufs["info"].clone()]
    for fm, fr, sb, band in [(0, 8, 256, 0), (1, 4, 128, 1), (1, 16, 512, 0), (2, 4, 256, 1), (2, 16, 128, 1),
                             (1, 8, 512, 1), (2, 8, 256, 1), (2, 16, 256, 0)]:
        b.set_tuning(fill_mode=fm, fill_run=fr, sweep_block=sb, fill_band=band)
        for use_graph in (False, True):
            assert b.run(use_graph=use_graph) == (nv, ni)
            got = [bufs[k][:n] for k, n in (("pos", nv), ("nrm", nv), ("idx", ni))] + [bufs["info"]]
            for r, g_ in zip(ref, got):
                assert torch.equal(r.view(torch.int32) if r.is_floating_point() else r,
                                   g_.view(torch.int32) if g_.is_floating_point() else g_), (fm, fr, sb, band)
    chosen, ms = b.autotune(reps=2)
    assert len(ms) == 10 and all(m > 0 for m in ms)
    assert chosen["fill_mode"] in (0, 1, 2) and chosen["sweep_block"] in (128, 256, 512)
    assert b.tuning() == chosen
    got = [bufs[k][:n] for k, n in (("pos", nv), ("nrm", nv), ("idx", ni))] + [bufs["info"]]
    for r, g_ in zip(ref, got):
        assert torch.equal(r.view(torch.int32) if r.is_floating_point() else r,
                           g_.view(torch.int32) if g_.is_floating_point() else g_)
    with pytest.raises(L.BmfError):
        b.set_tuning(fill_run=5)
    b.close()


def test_capacity_overflow_reports_needed_counts(ctx):
    import ctypes
    dim = 33
    d = make_density(next(c for c in ALL if c["name"] == "uniform_33"))
    words_t, _ = ctx.label_grid(dim, dev(d))
    m, bufs = ctx._alloc_mesh(16, 16, False)
    st = ctx.lib.bmf_polygonize(ctx.h, dim, ctypes.c_void_p(dev(d).data_ptr()), ctypes.c_void_p(words_t.data_ptr()),
                                L.MODE_R, 0, ctypes.byref(m), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == L.ERR_CAPACITY
    O = cpu.extract_r(dim, d, cpu.cell_masks(dim, cpu.label_grid(dim, d)[0]))
    assert m.n_verts == len(O["pos"]) and m.n_idx == len(O["idx"])
    # the context stays usable
    mm = ctx.polygonize(dim, dev(d), words_t)
    assert mm.n_verts == len(O["pos"])


def test_invalid_arguments(ctx):
    with pytest.raises(L.BmfError) as e:
        ctx.sample_block(L.ChunkDesc.make((0, 0, 0), 1.0, 1), workloads.sphere_wave_field())
    assert e.value.status == L.ERR_INVALID_ARGUMENT
    with pytest.raises(L.BmfError):
        ctx.sample_block(L.ChunkDesc.make((0, 0, 0), 1.0, 4096), workloads.sphere_wave_field())
