"""Host-side logic: workloads, descriptor sharding, C-ABI struct layouts (CPU only)."""
import ctypes

import numpy as np

from binarymeshfitting_gb300 import _lib, workloads


def test_lod_update_matches_spec():
    descs, rows = workloads.lod_update()
    assert len(descs) == 4096
    dims, counts = np.unique(rows[:, 4], return_counts=True)
    assert dims.tolist() == [33, 65, 129] and counts.tolist() == [2048, 1434, 614]
    assert int((rows[:, 4] ** 3).sum()) == 1785478272
    assert set(np.unique(rows[:, 3]).tolist()) == {1.0, 2.0, 4.0, 8.0}
    ext = (rows[:, 4] - 1) * rows[:, 3]
    assert np.all(rows[:, :3] >= 0) and np.all(rows[:, :3] + ext[:, None] <= workloads.WORLD)
    assert np.all(np.mod(rows[:, :3], ext[:, None]) == 0), "origins snap to the chunk extent"
    _, rows2 = workloads.lod_update()
    np.testing.assert_array_equal(rows, rows2)


def test_shard_partitions_chunks():
    _, rows = workloads.lod_update(n=512)
    for ws in (1, 2, 3, 8):
        parts = [workloads.shard(rows, r, ws) for r in range(ws)]
        allidx = np.concatenate(parts)
        np.testing.assert_array_equal(np.sort(allidx), np.arange(len(rows)))
        w = [(rows[p, 4] ** 3).sum() for p in parts]
        assert max(w) <= (rows[:, 4] ** 3).sum() / ws + 129 ** 3


def test_struct_layouts_match_header():
    # include/bmf.h: bmf_chunk_desc is 24 bytes, bmf_field 36, bmf_mesh 80, bmf_batch_out 72
    assert ctypes.sizeof(_lib.ChunkDesc) == 24
    assert ctypes.sizeof(_lib.Field) == 36
    assert ctypes.sizeof(_lib.ExtractOpts) == 24
    assert ctypes.sizeof(_lib.Mesh) == 80
    assert ctypes.sizeof(_lib.BatchOut) == 72
    assert ctypes.sizeof(_lib.BatchTuning) == 32


def test_fill_fp32_op_count():
    """The bench's algorithmic FP32 instruction count of the line-separable
    FBM: per sample 5 per octave + 1, plus per-line and per-layer set-up terms;
    on the mixed-LOD update about 45 per sample, and a single 1-octave chunk
    inside one z-lattice cell matches the closed form exactly."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), ".."))
    import bench
    _, rows = workloads.lod_update()
    ops = bench.fill_fp32_ops(rows, workloads.TERRAIN_PARAMS)
    per_sample = ops / (rows[:, 4] ** 3).sum()
    assert 40.0 < per_sample < 50.0, per_sample
    # one 33^3 chunk, one octave at a frequency that keeps every line in one cell
    params = (64.0, 40.0, 1e-4, 2.0, 0.5, 1, 1337)
    one = np.array([[0.0, 0.0, 0.0, 1.0, 33, 0]])
    dim = 33
    want = (dim ** 3 * (bench.OPS_PER_SAMPLE_OCTAVE + bench.OPS_PER_SAMPLE)
            + dim ** 2 * (bench.OPS_PER_LINE_OCTAVE + bench.OPS_PER_LINE) + dim ** 2 * 2 * bench.OPS_PER_LAYER)
    assert bench.fill_fp32_ops(one, params) == want


def test_bench_tier_split_matches_generator():
    """The bench's config names the update's tiers as the generator draws them,
    for the default 4096 chunks and for other batch sizes."""
    import collections
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), ".."))
    import bench
    assert bench.tier_split(4096) == "2048x33^3 + 1434x65^3 + 614x129^3"
    for n in (4096, 2048, 777, 256):
        _, rows = workloads.lod_update(n=n)
        got = collections.Counter(rows[:, 4].astype(int))
        want = " + ".join("%dx%d^3" % (got[d], d) for d in (33, 65, 129))
        assert bench.tier_split(n) == want, (n, bench.tier_split(n), want)
