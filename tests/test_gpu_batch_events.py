"""bmf_batch_wait_extraction: a stream made to wait on a run's extraction
event reads the run's final indices and chunk table while the smoothing may
still be running -- in direct runs and in graph replays."""
import pytest
import torch

from binarymeshfitting_gb300 import _lib as L
from binarymeshfitting_gb300 import workloads
from binarymeshfitting_gb300.engine import Batch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("use_graph", [False, True])
def test_wait_extraction_gives_final_topology(ctx, use_graph):
    descs, rows = workloads.lod_update(n=600, seed=31)  # >= 512 chunks: the chunk-by-chunk sweeps
    for dsc in descs:
        dsc.dim = 17
    b = Batch(ctx, descs, workloads.terrain_field(), mode=L.MODE_R, iters=4, smooth_normals=True)
    bufs = b.allocate(2_000_000, 12_000_000, normals=True)
    nv, ni = b.run(use_graph=use_graph)
    ref_idx, ref_info = bufs["idx"][:ni].clone(), bufs["info"].clone()
    side = torch.cuda.Stream()
    for _ in range(3):
        bufs["idx"].fill_(-1)
        bufs["info"].fill_(-1)
        side.wait_stream(torch.cuda.current_stream())
        b.run(use_graph=use_graph, sync=False)
        b.wait_extraction(side)
        with torch.cuda.stream(side):
            got_idx, got_info = bufs["idx"][:ni].clone(), bufs["info"].clone()
        torch.cuda.synchronize()
        assert torch.equal(got_idx, ref_idx) and torch.equal(got_info, ref_info)
    b.close()
