"""The oracle's restatement of the WorldOctree split policy
(WorldOctree::split_leaves / node_needs_split, WorldOctree.cpp:129-161,
237-247): the leaves tile the root cube exactly, none of them needs a split,
every one of their parents does, and they come in depth-first stack order
(children pushed 0..7, popped 7..0).  The chunk frame is DMCChunk.cpp:94-97
with ChunkGenerator.cpp:98's overlap."""
import numpy as np
import pytest

from oracle import cpu

ROOT, SIZE = (-4096.0, -4096.0, -4096.0), 8192.0
MCD = [(0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1), (0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)]


def needs_split(pos, size, level, focus, sm, smod, lo, hi):
    f = np.float32
    if level >= hi:
        return False
    if level < lo:
        return True
    m = [f(f(p) + f(f(size) * f(0.5))) for p in pos]
    d = [f(f(focus[k]) - m[k]) for k in range(3)]
    dist = f(np.sqrt(f(f(f(d[0] * d[0]) + f(d[1] * d[1])) + f(d[2] * d[2]))))
    return bool(dist < f(f(f(f(size) * f(sm)) + f(smod)) + f(f(size) * f(0.5))))


def reference_leaves(focus, sm, smod, lo, hi):
    """Direct Python walk of split_leaves (pure-Python twin, small trees)."""
    f = np.float32
    stack = [((f(ROOT[0]), f(ROOT[1]), f(ROOT[2])), f(SIZE), 0)]
    out = []
    while stack:
        pos, size, level = stack.pop()
        if not needs_split(pos, size, level, focus, sm, smod, lo, hi):
            out.append((pos, size, level))
            continue
        cs = f(size * f(0.5))
        for dx, dy, dz in MCD:
            stack.append(((f(pos[0] + f(dx) * cs), f(pos[1] + f(dy) * cs), f(pos[2] + f(dz) * cs)),
                          f(size * f(0.5)), level + 1))
    return out


@pytest.mark.parametrize("focus,sm,smod,lo,hi", [((10.0, 64.0, 20.0), 1.0, 0.0, 1, 7),
                                                ((1000.0, -300.0, 5.0), 1.5, 16.0, 2, 8),
                                                ((0.0, 0.0, 0.0), 0.5, 0.0, 0, 5)])
def test_lod_restatement_matches_python_walk(focus, sm, smod, lo, hi):
    dim = 33
    rows = cpu.lod_generate(ROOT, SIZE, focus, sm, smod, lo, hi, dim)
    ref = reference_leaves(focus, sm, smod, lo, hi)
    assert len(rows) == len(ref) > 8
    f = np.float32
    vol = 0.0
    for r, (pos, size, level) in zip(rows, ref):
        ov = f(0.0) if level == hi else f(f(0.035) + f(0.005) * f(0.0))
        delta = f(f(size * f(f(1.0) + f(ov * f(2.0)))) / f(dim - 1))
        assert r[3] == delta and int(r[4]) == dim and int(r[5]) == level
        assert tuple(r[:3]) == tuple(f(p - f(size * ov)) for p in pos)
        assert not needs_split(pos, size, level, focus, sm, smod, lo, hi)
        vol += float(size) ** 3
    assert vol == SIZE ** 3  # the leaves tile the root


def test_lod_overlap_and_iters():
    rows0 = cpu.lod_generate(ROOT, SIZE, (10.0, 64.0, 20.0), 1.0, 0.0, 1, 6, 65, base_overlap=0.035,
                             boundary_processing=True, iters=4)
    lv = rows0[:, 5].astype(int)
    # with boundary processing and iterations every level overlaps (0.035 + 0.02)
    size = np.float32(SIZE) / np.float32(2.0) ** lv.astype(np.float32)
    assert np.allclose(rows0[:, 3], size * (1 + 2 * 0.055) / 64, rtol=1e-6)
