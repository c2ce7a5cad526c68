"""The drop-in from C++: a compiled caller (binarymeshfitting_gb300/dropin/
bmf_dropin.cpp) that includes include/bmf.h and include/bmf_adapter.hpp the way a
BinaryMeshFitting maintainer would, runs the per-chunk replacement of
ChunkGenerator::extract_chunk (ChunkGenerator.cpp:98-124), the reference-named
DMCChunk / MeshProcessor<3> sequence and ChunkGenerator::process_queue twice
with one queue shape (plan reuse), and reports counts; they are checked here
against the oracle."""
import json
import os
import subprocess

import numpy as np
import pytest

from binarymeshfitting_gb300 import _lib as L
from binarymeshfitting_gb300 import build, workloads
from oracle import cpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def report():
    build.build()
    r = subprocess.run([build.DROPIN, "check"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return json.loads(r.stdout)


def test_per_chunk_counts_match_oracle(report):
    d = cpu.fill_field(L.FIELD_SPHERE_WAVE, list(workloads.SPHERE_WAVE_PARAMS), 65)
    w, cm = cpu.label_grid(65, d)
    O = cpu.extract_r(65, d, cpu.cell_masks(65, w))
    pc = report["per_chunk"]
    assert pc["contains_mesh"] == cm == 1
    assert pc["n_verts"] == len(O["pos"]) and pc["n_idx"] == len(O["idx"])
    assert report["per_chunk_smoothed"]["n_verts"] == len(O["pos"])


def test_reference_named_classes_match_extract_chunk(report):
    c = report["classes"]
    assert c["match_extract_chunk"] == 1 and c["has_adjacency"] == 1
    assert c["n_verts"] == report["per_chunk_smoothed"]["n_verts"]


def test_process_queue_reuses_its_plan_and_matches_oracle(report):
    q0, q1 = report["queues"]
    assert q0["plans_reused"] == 0 and q1["plans_reused"] == 1
    checked = 0
    for q in (q0, q1):
        total = 0
        for ch in q["chunks"]:
            org = np.array(ch["origin_bits"], np.uint32).view(np.float32)
            scale = float(np.array([ch["scale_bits"]], np.uint32).view(np.float32)[0])
            counts, _ = cpu.extract_batch_digest(np.array([[*org, scale, 33]], np.float32), L.FIELD_TERRAIN_FBM,
                                                 list(workloads.TERRAIN_PARAMS), 0, 0, 2, False, True)
            assert ch["contains_mesh"] == counts[0, 0]
            assert ch["n_verts"] == counts[0, 1] and ch["n_idx"] == counts[0, 2]
            total += ch["n_verts"]
            checked += int(ch["n_verts"] > 0)
        assert q["n_verts"] == total
    assert checked >= 4


def test_time_loop_runs(tmp_path):
    """The per-chunk timing mode (used by bench.py) on a few chunks."""
    build.build()
    descs, _ = workloads.lod_update(n=16, seed=3)
    path = os.path.join(tmp_path, "descs.bin")
    with open(path, "wb") as f:
        for dsc in descs:
            f.write(bytes(dsc))
    prm = [str(x) for x in list(workloads.TERRAIN_PARAMS) + [0.0]]
    r = subprocess.run([build.DROPIN, "time", path, str(L.FIELD_TERRAIN_FBM)] + prm + ["0", "0", "4", "1", "4"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = json.loads(r.stdout)
    assert out["chunks"] == 16 and out["chunks_per_s"] > 0 and out["launches"] > 0
