"""bmf_polygonize_noalloc: the extraction entry point for callers that cannot
allocate device memory (hosts that own every device allocation through their
own pool, or threads that may not block on the driver's allocator).

It is called straight through the C ABI with ctypes -- no bmf_ctx, no library
allocation -- and must give exactly what bmf_polygonize gives (the same
bit-exact bar the other parity tests use), on two calls in a row, since the
calls share one static scratch array that keeps the previous call's contents.
This file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest
import torch

from binarymeshfitting_gb300 import _lib as L
from tests.golden.cases import make_density

pytestmark = pytest.mark.gpu


def _mesh(vcap, icap):
    dev = torch.device("cuda", 0)
    bufs = dict(pos=torch.full((vcap, 3), -7.0, device=dev), bnd=torch.full((vcap,), 9, dtype=torch.uint8, device=dev),
                val=torch.full((vcap,), 9, dtype=torch.uint8, device=dev),
                idx=torch.full((icap,), -1, dtype=torch.int32, device=dev))
    m = L.Mesh(bufs["pos"].data_ptr(), None, bufs["bnd"].data_ptr(), bufs["val"].data_ptr(), bufs["idx"].data_ptr(),
               vcap, icap, 0, 0, 0, 0)
    return m, bufs


def _call(lib, dim, dens, words, mode, placement, m):
    return lib.bmf_polygonize_noalloc(dim, ctypes.c_void_p(dens.data_ptr()), ctypes.c_void_p(words.data_ptr()), mode,
                                      placement, ctypes.byref(m),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


def _noalloc(lib, dim, dens, words, mode, placement, vcap, icap):
    m, bufs = _mesh(vcap, icap)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    st = _call(lib, dim, dens, words, mode, placement, m)
    free_after = torch.cuda.mem_get_info()[0]
    assert st == L.OK, L.STATUS.get(st)
    # the output buffers exist before the call: the call itself takes no device memory
    assert free_after == free_before, "bmf_polygonize_noalloc changed free device memory by %d bytes" % (
        free_before - free_after)
    nv, ni = m.n_verts, m.n_idx
    return dict(pos=bufs["pos"][:nv].cpu().numpy(), boundary=bufs["bnd"][:nv].cpu().numpy(),
                valence=bufs["val"][:nv].cpu().numpy(), idx=bufs["idx"][:ni].cpu().numpy(),
                contains_mesh=m.contains_mesh, prim_size=m.prim_size)


CASES = [
    dict(name="sphere_wave_65", dim=65, kind="field", field=1, params=[32.0, 32.0, 32.0, 20.0, 1.5, 0.3],
         origin=[0, 0, 0], scale=1.0),
    dict(name="uniform_33", dim=33, kind="uniform", seed=133, lo=-1.0, hi=1.0),
    dict(name="terrain_129", dim=129, kind="field", field=2, params=[64.0, 40.0, 0.01, 2.0, 0.5, 5, 1337],
         origin=[0, 0, 0], scale=1.0),
]


@pytest.mark.parametrize("mode,placement", [(L.MODE_R, 0), (L.MODE_Q, 0), (L.MODE_Q, 1), (L.MODE_Q, 2)])
def test_noalloc_matches_polygonize_on_two_calls(mode, placement):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from binarymeshfitting_gb300.engine import Context
    lib = L.load()
    ctx = Context(0)
    try:
        # the first call on the device may load the module and place the static
        # array (lazy loading): make it once before any call is measured
        warm = torch.from_numpy(make_density(CASES[1])).cuda()
        ww, _ = ctx.label_grid(33, warm)
        m, _ = _mesh(1 << 17, 1 << 20)  # room for any 33^3 chunk (at most 15 indices per cell)
        assert _call(lib, 33, warm, ww, mode, placement, m) == L.OK
        for case in CASES:  # consecutive calls of different sizes reuse the shared scratch
            dim = case["dim"]
            dens = torch.from_numpy(make_density(case)).cuda()
            words, _ = ctx.label_grid(dim, dens)
            ref = ctx.polygonize(dim, dens, words, mode=mode, placement=placement)
            for _ in range(2):
                got = _noalloc(lib, dim, dens, words, mode, placement, ref.n_verts + 16, ref.n_idx + 16)
                assert got["contains_mesh"] == int(ref.contains_mesh)
                assert got["prim_size"] == ref.prim_size
                np.testing.assert_array_equal(got["idx"], ref.idx.cpu().numpy())
                np.testing.assert_array_equal(got["pos"].view(np.uint32), ref.pos.cpu().numpy().view(np.uint32))
                np.testing.assert_array_equal(got["boundary"], ref.boundary.cpu().numpy())
                np.testing.assert_array_equal(got["valence"], ref.valence.cpu().numpy())
    finally:
        ctx.close()


def test_noalloc_rejects_oversized_chunk():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = L.load()
    dim = 130  # one past BMF_NOALLOC_MAX_DIM
    dens = torch.zeros(8, device="cuda")
    words = torch.zeros(8, dtype=torch.int32, device="cuda")
    m, _ = _mesh(4, 4)
    st = lib.bmf_polygonize_noalloc(dim, ctypes.c_void_p(dens.data_ptr()), ctypes.c_void_p(words.data_ptr()),
                                    L.MODE_R, 0, ctypes.byref(m), None)
    assert st == L.ERR_NOT_SUPPORTED


@pytest.mark.parametrize("mode,placement", [(L.MODE_R, 0), (L.MODE_Q, 2)])
def test_noalloc_reports_capacity_and_writes_nothing_past_it(mode, placement):
    """Capacities one short of the needed counts: BMF_ERR_CAPACITY with the
    full needed counts, and the guard regions after vcap / icap untouched."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from binarymeshfitting_gb300.engine import Context
    lib = L.load()
    ctx = Context(0)
    try:
        case = CASES[0]
        dim = case["dim"]
        dens = torch.from_numpy(make_density(case)).cuda()
        words, _ = ctx.label_grid(dim, dens)
        ref = ctx.polygonize(dim, dens, words, mode=mode, placement=placement)
        guard = 4096
        vcap, icap = ref.n_verts - 1, ref.n_idx - 1
        m, bufs = _mesh(vcap + guard, icap + guard)
        m.vcap, m.icap = vcap, icap
        assert _call(lib, dim, dens, words, mode, placement, m) == L.ERR_CAPACITY
        assert m.n_verts == ref.n_verts and m.n_idx == ref.n_idx
        torch.cuda.synchronize()
        assert (bufs["pos"][vcap:] == -7.0).all()
        assert (bufs["bnd"][vcap:] == 9).all() and (bufs["val"][vcap:] == 9).all()
        assert (bufs["idx"][icap:] == -1).all()
        # the shared scratch is left in a state the next call handles
        got = _noalloc(lib, dim, dens, words, mode, placement, ref.n_verts, ref.n_idx)
        np.testing.assert_array_equal(got["idx"], ref.idx.cpu().numpy())
        np.testing.assert_array_equal(got["pos"].view(np.uint32), ref.pos.cpu().numpy().view(np.uint32))
    finally:
        ctx.close()
