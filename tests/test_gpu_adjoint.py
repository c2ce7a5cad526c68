"""The differentiable extraction on the GPU (bmf_fit_* through the C ABI and its
torch.autograd binding) against the oracles.

* forward: Mode Q topology, QEF placement and 8 boundary-frozen MeshProcessor<4>
  sweeps -- positions and quad indices bit-identical to the float oracle
  (bmf_oracle.c: extract_q + process);
* backward: dL/d(density) of L = mean_v sdf_box(p_v)^2 against the FP64 adjoint
  of oracle/bmf_oracle_fit.c (itself checked against central differences).
  The forward is float32 (the reference's QEF).  At a vertex where it takes a
  different branch than the FP64 forward (QEF vs mass point, an eigenvalue at
  the 1e-3 truncation threshold) the two functions are different pieces of a
  discontinuous map and their gradients differ by O(1): the oracle flags the
  samples such vertices read (near_branch) and the comparison runs on the
  rest.  Bars there: with the FP64 QEF adjoint (the default) 2e-4 relative L2
  (the float forward's positions feed dL/dp) and 99.9% of the support's
  entries within 1e-3 relative + 1e-4 max|g|; the FP32 adjoint, whose error is
  1/s^2 times the ~1e-6 FP32 error of small kept eigenvalues, 1e-2 relative L2.
  Loss within 1e-4 relative.
* batching: a chunk's gradient in a 3-chunk batch equals its single-chunk
  gradient up to float32 reordering of the atomics (1e-5 of max|g|);
* batched fitting (per-chunk sphere-union targets, loss = sum of per-chunk
  means): the loss and spot-checked chunks' gradients against the FP64 oracle
  with the same bars;
* fitting: 40 Adam steps on the density move the mesh towards the target.
"""
import numpy as np
import pytest
import torch

from binarymeshfitting_gb300 import _lib as L
from binarymeshfitting_gb300 import workloads
from binarymeshfitting_gb300.engine import Context
from binarymeshfitting_gb300.fitting import ExtractFit, FitPlan, rounded_box_sdf, sphere_union_loss
from oracle import cpu

pytestmark = pytest.mark.gpu

DIM = 65
ITERS = 8
BOX = [32.0, 32.0, 32.0, 18.0, 14.0, 10.0, 4.0]


def sphere_noise(seed=3, radius=20.0, sigma=0.1):
    g = np.arange(DIM, dtype=np.float64)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    rng = np.random.default_rng(seed)
    d = np.sqrt((X - 32) ** 2 + (Y - 32) ** 2 + (Z - 32) ** 2) - radius + rng.normal(0, sigma, X.shape)
    return d.reshape(-1).astype(np.float32)


def box_loss(pos, reduce="mean"):
    b = torch.tensor(BOX, dtype=torch.float32, device=pos.device)
    d = rounded_box_sdf(pos, b[:3], b[3:6], b[6])
    return (d * d).mean() if reduce == "mean" else (d * d).sum()


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


def test_fit_forward_bit_exact(ctx):
    d = sphere_noise()
    plan = FitPlan(ctx, 1, DIM, L.PLACE_QEF, ITERS)
    pos, idx, info = plan.forward(torch.from_numpy(d).cuda())
    words, _ = cpu.label_grid(DIM, d)
    ref = cpu.extract_q(DIM, d, words, placement=2)
    rpos, _ = cpu.process(4, ref["pos"], ref["boundary"], ref["valence"], ref["idx"], ITERS)
    assert pos.shape[0] == len(rpos) and idx.numel() == len(ref["idx"])
    assert np.array_equal(idx.cpu().numpy().view(np.uint32), ref["idx"])
    g = pos.cpu().numpy()
    assert np.array_equal(g.view(np.uint32), rpos.astype(np.float32).view(np.uint32)), \
        "max |diff| %g" % np.abs(g - rpos).max()
    inf = info.cpu().numpy()[0]
    assert inf[0] == 0 and inf[1] == len(rpos) and inf[2] == 0 and inf[3] == len(ref["idx"])
    plan.close()


def gpu_grad(ctx, d, reduce="mean", adjoint="df"):
    plan = FitPlan(ctx, 1, DIM, L.PLACE_QEF, ITERS, adjoint=adjoint)
    dens = torch.from_numpy(d).cuda().requires_grad_(True)
    pos = ExtractFit.apply(dens, plan)
    loss = box_loss(pos, reduce)
    loss.backward()
    out = float(loss.detach()), dens.grad.double().cpu().numpy()
    plan.close()
    return out


def compare_kept(g, g64, near_branch):
    keep = near_branch == 0
    gk = g64[keep]
    rel_l2 = np.linalg.norm(g[keep] - gk) / np.linalg.norm(gk)
    gmax = np.abs(gk).max()
    sup = keep & (np.abs(g64) > 1e-6 * gmax)
    ok = np.abs(g[sup] - g64[sup]) <= 1e-3 * np.abs(g64[sup]) + 1e-4 * gmax
    return rel_l2, ok.mean(), keep.mean(), sup.sum()


def test_fit_gradient_fp32_adjoint(ctx):
    d = sphere_noise()
    _, g = gpu_grad(ctx, d, adjoint="f32")
    nb = np.zeros(DIM ** 3, np.uint8)
    _, g64, _, _ = cpu.fit_loss_f64(DIM, d.astype(np.float64), ITERS, BOX, want_grad=True, near_branch=nb)
    rel_l2, ok, _, _ = compare_kept(g, g64, nb)
    print("FP32 adjoint: rel_l2 %.3g, entries within tol %.4f" % (rel_l2, ok))
    assert rel_l2 <= 1e-2


@pytest.mark.parametrize("adjoint", ["df", "f64"])
def test_fit_gradient_matches_fp64_adjoint(ctx, adjoint):
    """The double-float and the FP64 re-solve against the FP64 oracle gradient."""
    d = sphere_noise()
    loss, g = gpu_grad(ctx, d, adjoint=adjoint)
    nb = np.zeros(DIM ** 3, np.uint8)
    loss64, g64, counts, _ = cpu.fit_loss_f64(DIM, d.astype(np.float64), ITERS, BOX, want_grad=True,
                                              near_branch=nb)
    assert abs(loss - loss64) <= 1e-4 * abs(loss64), (loss, loss64)
    rel_l2, ok, kept, nsup = compare_kept(g, g64, nb)
    print("%s: loss %.9g vs %.9g  rel_l2 %.3g  entries within tol %.5f of %d (samples kept %.4f; vertices %d, "
          "QEF-placed %d)" % (adjoint, loss, loss64, rel_l2, ok, nsup, kept, counts[0], counts[2]))
    assert rel_l2 <= 2e-4
    assert ok >= 0.999
    assert kept >= 0.98


def test_df_adjoint_matches_f64_adjoint(ctx):
    """Double-float and FP64 re-solves give the same gradient to well below the
    oracle tolerance (both differentiate the exact-arithmetic placement)."""
    d = sphere_noise(seed=5)
    _, g_df = gpu_grad(ctx, d, adjoint="df")
    _, g_64 = gpu_grad(ctx, d, adjoint="f64")
    rel = np.linalg.norm(g_df - g_64) / np.linalg.norm(g_64)
    print("df vs f64 adjoint: rel_l2 %.3g" % rel)
    assert rel <= 2e-5


def test_fit_batched_equals_single(ctx):
    ds = [sphere_noise(seed=s, radius=r) for s, r in ((7, 18.0), (8, 21.0), (9, 24.0))]
    plan = FitPlan(ctx, 3, DIM, L.PLACE_QEF, ITERS)
    dens = torch.from_numpy(np.concatenate(ds)).cuda().requires_grad_(True)
    pos = ExtractFit.apply(dens, plan)
    loss = box_loss(pos, "sum")
    loss.backward()
    gb = dens.grad.double().cpu().numpy().reshape(3, -1)
    info = plan.info.cpu().numpy()
    plan.close()
    for k, d in enumerate(ds):
        l1, g1 = gpu_grad(ctx, d, "sum")
        assert np.abs(gb[k] - g1).max() <= 1e-5 * np.abs(g1).max(), k
        assert info[k, 1] > 0


def test_fit_adam_moves_mesh_to_target(ctx):
    d = sphere_noise(seed=12, sigma=0.0)
    plan = FitPlan(ctx, 1, DIM, L.PLACE_QEF, 4)
    dens = torch.from_numpy(d).cuda().requires_grad_(True)
    opt = torch.optim.Adam([dens], lr=0.05)
    losses = []
    # the surface has to travel up to 10 cells; Adam moves each sample by at
    # most ~lr per step, so 40 steps take the loss down by about a fifth
    for _ in range(40):
        opt.zero_grad()
        pos = ExtractFit.apply(dens, plan)
        loss = box_loss(pos)
        loss.backward()
        opt.step()
        losses.append(float(loss.detach()))
    print("loss %.4g -> %.4g" % (losses[0], losses[-1]))
    assert all(np.isfinite(losses))
    assert losses[-1] < 0.9 * losses[0]
    assert sum(b < a for a, b in zip(losses, losses[1:])) >= 0.6 * (len(losses) - 1)
    plan.close()


def test_batched_fit_spheres_fp64_spot_check(ctx):
    n = 8
    dens, sph = workloads.fit_batch(n, dim=DIM, seed=21)
    plan = FitPlan(ctx, n, DIM, L.PLACE_QEF, ITERS)
    d = dens.clone().requires_grad_(True)
    pos = ExtractFit.apply(d, plan)
    loss = sphere_union_loss(pos, plan.info, sph)
    loss.backward()
    g = d.grad.double().cpu().numpy().reshape(n, -1)
    hd = dens.cpu().numpy().astype(np.float64).reshape(n, -1)
    hs = sph.cpu().numpy()
    plan.close()
    loss64 = 0.0
    for k in range(n):
        want = k in (0, 3, 7)
        nb = np.zeros(DIM ** 3, np.uint8)
        lk, gk, _, _ = cpu.fit_loss_spheres_f64(DIM, hd[k], ITERS, hs[k], want_grad=want, near_branch=nb)
        loss64 += lk
        if want:
            rel_l2, ok, kept, _ = compare_kept(g[k], gk, nb)
            print("chunk %d: rel_l2 %.3g, entries within tol %.5f, samples kept %.4f" % (k, rel_l2, ok, kept))
            assert rel_l2 <= 2e-4 and ok >= 0.999, k
    assert abs(float(loss) - loss64) <= 1e-4 * abs(loss64), (float(loss), loss64)


def test_fit_create_rejects_two_wide_adjoints(ctx):
    """BMF_FIT_ADJOINT_F64 and BMF_FIT_ADJOINT_DF are exclusive."""
    import ctypes
    h = ctypes.c_void_p()
    st = ctx.lib.bmf_fit_create(ctx.h, 1, DIM, L.PLACE_QEF, ITERS, 100000, 400000,
                                L.FIT_ADJOINT_F64 | L.FIT_ADJOINT_DF, ctypes.byref(h))
    assert st == L.ERR_INVALID_ARGUMENT and not h.value


def test_chunk_sweep_fit_matches_whole_mesh_fit(ctx):
    """A fit plan of 2048 chunks or more runs its forward sweeps chunk by
    chunk, with the CSR offsets and adjacency built inside that kernel, and
    from 256 chunks its adjoint sweeps too.  The same chunks in a 100-chunk
    plan (whole-mesh forward and adjoint sweeps) and a 2000-chunk plan
    (whole-mesh forward, chunk-by-chunk adjoint) give bit-identical positions
    and indices, and the same density gradient up to float32 reordering of the
    QEF adjoint's atomics (1e-5 of max|g|)."""
    n, dim = 2100, 13
    g = np.arange(dim, dtype=np.float64)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    rng = np.random.default_rng(31)
    radii = rng.uniform(3.0, 5.5, n)
    base = np.sqrt((X - 6) ** 2 + (Y - 6) ** 2 + (Z - 6) ** 2).reshape(1, -1)
    dens = (base - radii[:, None] + rng.normal(0, 0.1, (n, dim ** 3))).astype(np.float32)
    dd = torch.from_numpy(dens.reshape(-1)).cuda()

    def run(lo, hi):
        plan = FitPlan(ctx, hi - lo, dim, L.PLACE_QEF, ITERS)
        pos, idx, info = plan.forward(dd[lo * dim ** 3: hi * dim ** 3].contiguous())
        pos, idx, info = pos.clone(), idx.clone(), info.clone()
        w = torch.sin(torch.arange(pos.numel(), device=pos.device, dtype=torch.float32) * 0.37).view(-1, 3)
        grad = plan.backward(w).clone()
        plan.close()
        return pos, idx, info, grad

    pos, idx, info, grad = run(0, n)
    parts = [run(0, 100), run(100, n)]
    assert info[:, 1].sum().item() == pos.shape[0] and (info[:, 4] > 0).sum().item() > n // 2
    assert torch.equal(pos.view(torch.int32), torch.cat([p[0] for p in parts]).view(torch.int32))
    # indices are chunk-local: the two plans' concatenation is the big plan's
    assert torch.equal(idx, torch.cat([p[1] for p in parts]))
    # the weights restart at vertex 0 in each part: compare each part's chunks
    # with a big-plan backward whose weights restart the same way
    nv0 = parts[0][0].shape[0]
    plan = FitPlan(ctx, n, dim, L.PLACE_QEF, ITERS)
    plan.forward(dd)
    w = torch.cat([torch.sin(torch.arange(p[0].numel(), device=dd.device, dtype=torch.float32) * 0.37).view(-1, 3)
                   for p in parts])
    gb = plan.backward(w).double().cpu().numpy()
    plan.close()
    gs = torch.cat([p[3] for p in parts]).double().cpu().numpy()
    assert nv0 > 0 and np.abs(gs).max() > 0
    assert np.abs(gb - gs).max() <= 1e-5 * np.abs(gs).max()


def test_device_sphere_loss_matches_torch_and_captures_in_a_graph():
    """bmf_fit_loss_spheres (loss and position gradient read off the device
    chunk table) against the torch sphere-union loss and its autograd
    gradient; then a whole fitting step (forward, loss, backward) captured as a
    CUDA graph gives the eager step's loss bit for bit and its density gradient
    up to the order of the chain rule's float atomics."""
    from binarymeshfitting_gb300.fitting import FitPlan, sphere_union_loss
    ctx = Context(0)
    n, dim = 6, 33
    dens, spheres = workloads.fit_batch(n, dim=dim, seed=12)
    plan = FitPlan(ctx, n, dim, L.PLACE_QEF, 4)
    pos, _, info = plan.forward(dens)
    leaf = pos.detach().clone().requires_grad_(True)
    want = sphere_union_loss(leaf, info, spheres)
    (gwant,) = torch.autograd.grad(want, leaf)
    loss, grad = plan.loss_spheres(spheres)
    nv = pos.shape[0]
    assert abs(float(loss) - float(want)) <= 1e-5 * abs(float(want))
    assert torch.allclose(grad[:nv], gwant, rtol=1e-5, atol=1e-7)
    assert (grad[nv:] == 0).all()
    # eager asynchronous step vs the same step replayed from a CUDA graph
    lb, gp = torch.zeros(1, device="cuda"), torch.empty((plan.vcap, 3), device="cuda")
    g_eager, g_graph = torch.empty_like(dens), torch.empty_like(dens)
    plan.step_grad(dens, spheres, lb, gp, g_eager)
    torch.cuda.synchronize()
    loss_eager = float(lb)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        plan.step_grad(dens, spheres, lb, gp, g_graph)
    torch.cuda.current_stream().wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        plan.step_grad(dens, spheres, lb, gp, g_graph)
    g_graph.zero_()
    graph.replay()
    torch.cuda.synchronize()
    assert float(lb) == loss_eager
    assert torch.allclose(g_graph, g_eager, rtol=1e-5, atol=1e-6 * float(g_eager.abs().max()))
    g_ref = plan.backward(gwant)  # the same adjoint applied to torch's position gradient
    assert float((g_eager - g_ref).norm()) <= 1e-4 * float(g_ref.norm())
    plan.close()
    ctx.close()


def test_device_adam_matches_torch_adam():
    """bmf_fit_adam against torch.optim.Adam (same hyper-parameters, no weight
    decay) over five steps, on a length that is not a multiple of four and on
    an unaligned view (the scalar path)."""
    from binarymeshfitting_gb300.fitting import FitPlan
    ctx = Context(0)
    plan = FitPlan(ctx, 1, 17, L.PLACE_MASSPOINT, 0)
    gen = torch.Generator(device="cuda").manual_seed(3)
    for n, off in ((100_003, 0), (4099, 1)):
        base = torch.randn(n + off, device="cuda", generator=gen)
        p_ours = base.clone()[off:]
        p_ref = torch.nn.Parameter(base.clone()[off:].clone())
        opt = torch.optim.Adam([p_ref], lr=3e-2, betas=(0.9, 0.999), eps=1e-8)
        state = {}
        for k in range(5):
            g = torch.randn(n, device="cuda", generator=gen)
            p_ref.grad = g.clone()
            opt.step()
            plan.adam(p_ours, g, state, lr=3e-2)
        torch.cuda.synchronize()
        assert int(state["step"]) == 5
        assert torch.allclose(p_ours, p_ref.detach(), rtol=1e-5, atol=1e-6)
    plan.close()
    ctx.close()


def test_fit_checkpoint_resume(tmp_path):
    """Checkpoint / resume of the batched fitting loop: three device steps,
    save_checkpoint, three more; against load_checkpoint into fresh tensors and
    the same three steps.  The Adam step count resumes at 3 and the grids
    agree up to the order of the backward pass's float atomics."""
    from binarymeshfitting_gb300.fitting import FitPlan, load_checkpoint, save_checkpoint
    ctx = Context(0)
    n, dim = 6, 33
    dens, spheres = workloads.fit_batch(n, dim=dim, seed=17)
    plan = FitPlan(ctx, n, dim, L.PLACE_QEF, 4)
    lb, gp = torch.zeros(1, device="cuda"), torch.empty((plan.vcap, 3), device="cuda")
    gd = torch.empty_like(dens)

    def steps(d, state, k):
        for _ in range(k):
            plan.step_grad(d, spheres, lb, gp, gd)
            plan.adam(d, gd, state, lr=5e-2)
        torch.cuda.synchronize()

    state = {}
    steps(dens, state, 3)
    path = str(tmp_path / "fit.pt")
    save_checkpoint(path, dens, state, step=3, lr=5e-2)
    steps(dens, state, 3)
    d2, s2, extra = load_checkpoint(path, "cuda")
    assert extra == {"step": 3, "lr": 5e-2} and int(s2["step"]) == 3
    steps(d2, s2, 3)
    assert int(s2["step"]) == int(state["step"]) == 6
    assert float((d2 - dens).norm()) <= 1e-4 * float(dens.norm())
    plan.close()
    ctx.close()
