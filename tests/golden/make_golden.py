"""Generates the golden fixtures of this directory from the REFERENCE's own code.

Run where the reference sources are present (they are compiled into
oracle/_ref/libbmf_ref.so by oracle/Makefile):

    python tests/golden/make_golden.py

Every case's input density is reproducible without the reference: either one
of the bit-reproducible fields of oracle/bmf_oracle.c (bmf_fields.h ids) or a
seeded numpy PCG64 uniform array; its SHA-256 is stored so a consumer can check
it rebuilt the very same input.  Outputs of the reference's
DMCChunk::label_grid / label_edges / polygonize (and MeshProcessor<3>/<4>) are
stored as SHA-256 digests of the raw little-endian arrays plus counts; the
dim-32 sphere case also keeps full arrays in golden_small.npz.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from oracle import cpu, ref  # noqa: E402
from tests.golden.cases import CASES, PROCESS_CASES, make_density  # noqa: E402


def sha(a):
    """SHA-256 of the raw bytes; float NaNs are first canonicalised (x86, Arm and
    the GPU encode a NaN's sign and payload differently)."""
    a = np.ascontiguousarray(a)
    if a.dtype == np.float32:
        a = a.copy()
        a[np.isnan(a)] = np.float32("nan")
        a = np.where(np.isnan(a), np.uint32(0x7FC00000).view(np.float32), a)
    return hashlib.sha256(a.tobytes()).hexdigest()


def main():
    out = {"cases": [], "process": [], "implicit": [], "qef": None}
    small = {}
    for case in CASES:
        dim = case["dim"]
        d = make_density(case)
        R = ref.run(dim, d)
        rec = dict(case, density_sha=sha(d), contains_mesh=R["contains_mesh"], words_sha=sha(R["words"]),
                   n_cells=len(R["cell_lin"]), n_verts=len(R["pos"]), n_idx=len(R["idx"]))
        if R["contains_mesh"]:
            rec.update(masks_sha=sha(R["masks"]), cell_lin_sha=sha(R["cell_lin"]), cell_mask_sha=sha(R["cell_mask"]),
                       pos_sha=sha(R["pos"]), boundary_sha=sha(R["boundary"]), valence_sha=sha(R["valence"]),
                       idx_sha=sha(R["idx"]))
        out["cases"].append(rec)
        if case["name"] == "sphere_wave_32":
            for k in ("words", "masks", "pos", "boundary", "valence", "idx", "cell_lin", "cell_mask"):
                small[k] = R[k]
        print("case", case["name"], rec["n_verts"], rec["n_idx"])
    for pc in PROCESS_CASES:
        base = next(c for c in CASES if c["name"] == pc["case"])
        dim = base["dim"]
        d = make_density(base)
        if pc["N"] == 3:
            R = ref.run(dim, d, iters=pc["iters"], boundary_processing=pc["boundary"],
                        smooth_normals=pc["normals"])
            pos, nrm = R["pos"], R["nrm"]
        else:
            words, _ = cpu.label_grid(dim, d)
            Q = cpu.extract_q(dim, d, words, pc.get("placement", 1))
            pos, nrm, _ = ref.process(4, Q["pos"], Q["boundary"], Q["valence"], Q["idx"], pc["iters"],
                                      pc["boundary"], pc["normals"])
        rec = dict(pc, n_verts=len(pos), pos_sha=sha(pos), nrm_sha=sha(nrm))
        out["process"].append(rec)
        if pc["case"] == "sphere_wave_32" and pc["N"] == 3 and pc["iters"] == 4 and pc["normals"]:
            small["proc_pos"] = pos
            small["proc_nrm"] = nrm
        print("process", pc)
    # the reference's analytic fields through its own block filler
    for kind, name in ((3, "torus_z"), (4, "sphere"), (5, "cuboid"), (6, "plane_y")):
        res, org, size, scale = 32.0, (-15.5, -16.25, -15.75), 32, 1.0
        v = ref.implicit(kind - 3, res, org, (size, size, size), scale)
        out["implicit"].append(dict(kind=kind, name=name, resolution=res, origin=org, dim=size, scale=scale,
                                    sha=sha(v)))
    # QEF: seeded hermite sets through the reference's SSE solver
    rng = np.random.default_rng(7)
    P, N, C, X = [], [], [], []
    for _ in range(256):
        k = int(rng.integers(2, 13))
        p = rng.uniform(0, 1, (12, 3)).astype(np.float32)
        n = rng.normal(size=(12, 3)).astype(np.float32)
        n /= np.linalg.norm(n, axis=1, keepdims=True)
        x, _ = ref.qef_3d(p[:k], n[:k])
        P.append(p); N.append(n); C.append(k); X.append(x)
    small["qef_pos"] = np.stack(P)
    small["qef_nrm"] = np.stack(N)
    small["qef_count"] = np.array(C, np.int32)
    small["qef_ref"] = np.stack(X)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    np.savez_compressed(os.path.join(HERE, "golden_small.npz"), **small)
    print("wrote golden.json and golden_small.npz")


if __name__ == "__main__":
    main()
