"""torch.autograd binding of the differentiable extraction (bmf_fit_* in bmf.h).

Density grids in, mesh vertex positions out; gradients flow back into the
density through the library's adjoint kernels (QEF placement and position
sweeps).  Topology and index buffers never carry gradients.  This module is the
thin test/fitting binding; the compute is in libbmf_gb300.so.
"""
import ctypes

import torch

from . import _lib as L
from .engine import Context, _stream


class FitPlan:
    """n_chunks learnable grids of dim^3 samples (bmf_fit).  adjoint: "df" (the
    default) or "f64" take the QEF derivative from a re-solve of the hermite
    data and eigen pairs in double-float or FP64 arithmetic (the derivative of
    the exact-arithmetic placement; double-float gives FP64's accuracy here at
    a fraction of the cost); "f32" differentiates the forward's own FP32 eigen
    pairs.  adjoint_f64 (True / False) is the older spelling of "f64" / "f32"."""

    def __init__(self, ctx: Context, n_chunks, dim, placement=L.PLACE_QEF, iters=8, vcap=None, icap=None,
                 adjoint="df", adjoint_f64=None):
        self.ctx = ctx
        self.n, self.dim, self.iters = n_chunks, dim, iters
        self.vcap = vcap or n_chunks * dim * dim * 4
        self.icap = icap or 4 * self.vcap
        h = ctypes.c_void_p()
        if adjoint_f64 is not None:
            adjoint = "f64" if adjoint_f64 else "f32"
        flags = {"df": L.FIT_ADJOINT_DF, "f64": L.FIT_ADJOINT_F64, "f32": 0}[adjoint]
        ctx._check(ctx.lib.bmf_fit_create(ctx.h, n_chunks, dim, placement, iters, self.vcap, self.icap, flags,
                                          ctypes.byref(h)))
        self.h = h
        dev = ctx.device
        self.pos = torch.empty((self.vcap, 3), dtype=torch.float32, device=dev)
        self.idx = torch.empty(self.icap, dtype=torch.int32, device=dev)
        self.info = torch.zeros((n_chunks, 6), dtype=torch.int64, device=dev)
        self.n_verts = self.n_idx = 0

    def forward(self, density: torch.Tensor, sync=True):
        """Extracts all chunks.  sync=True reads the totals back and returns views
        of exactly the output; sync=False only enqueues (whole buffers returned)."""
        assert density.is_cuda and density.dtype == torch.float32 and density.is_contiguous()
        assert density.numel() == self.n * self.dim ** 3
        counts = (ctypes.c_int64 * 2)()
        self.ctx._check(self.ctx.lib.bmf_fit_forward(self.h, ctypes.c_void_p(density.data_ptr()),
                                                     ctypes.c_void_p(self.pos.data_ptr()),
                                                     ctypes.c_void_p(self.idx.data_ptr()),
                                                     ctypes.c_void_p(self.info.data_ptr()),
                                                     counts if sync else None, _stream()))
        if not sync:
            return self.pos, self.idx, self.info
        self.n_verts, self.n_idx = int(counts[0]), int(counts[1])
        return self.pos[: self.n_verts], self.idx[: self.n_idx], self.info

    def backward(self, grad_pos: torch.Tensor, out: torch.Tensor = None):
        g = grad_pos.contiguous()
        out = out if out is not None else torch.empty(self.n * self.dim ** 3, dtype=torch.float32,
                                                      device=self.ctx.device)
        self.ctx._check(self.ctx.lib.bmf_fit_backward(self.h, ctypes.c_void_p(g.data_ptr()), g.shape[0],
                                                      ctypes.c_void_p(out.data_ptr()), _stream()))
        return out

    def loss_spheres(self, spheres: torch.Tensor, loss: torch.Tensor = None, grad: torch.Tensor = None):
        """bmf_fit_loss_spheres on the last forward's positions: (loss (1,),
        dL/dpos (vcap, 3), zero past the vertex total); asynchronous."""
        sp = spheres.contiguous()
        assert sp.is_cuda and sp.dtype == torch.float32 and sp.shape[0] == self.n and sp.shape[-1] == 4
        loss = loss if loss is not None else torch.empty(1, dtype=torch.float32, device=self.ctx.device)
        grad = grad if grad is not None else torch.empty((self.vcap, 3), dtype=torch.float32, device=self.ctx.device)
        self.ctx._check(self.ctx.lib.bmf_fit_loss_spheres(self.h, ctypes.c_void_p(self.pos.data_ptr()),
                                                          ctypes.c_void_p(sp.data_ptr()), sp.shape[1],
                                                          ctypes.c_void_p(loss.data_ptr()),
                                                          ctypes.c_void_p(grad.data_ptr()), _stream()))
        return loss, grad

    def step_grad(self, density: torch.Tensor, spheres: torch.Tensor, loss: torch.Tensor, grad_pos: torch.Tensor,
                  grad_density: torch.Tensor):
        """One fitting step's device work without a host sync (capturable in a
        CUDA graph): forward, sphere-union loss and its position gradient,
        backward into grad_density."""
        self.forward(density, sync=False)
        self.loss_spheres(spheres, loss, grad_pos)
        self.ctx._check(self.ctx.lib.bmf_fit_backward(self.h, ctypes.c_void_p(grad_pos.data_ptr()), self.vcap,
                                                      ctypes.c_void_p(grad_density.data_ptr()), _stream()))

    def adam(self, param: torch.Tensor, grad: torch.Tensor, state: dict, lr=1e-2, betas=(0.9, 0.999), eps=1e-8):
        """bmf_fit_adam: one Adam step in place on param; state holds the
        moments and the device step count (created on the first call)."""
        if not state:
            state.update(m=torch.zeros_like(param), v=torch.zeros_like(param),
                         step=torch.zeros(1, dtype=torch.int32, device=param.device))
        self.ctx._check(self.ctx.lib.bmf_fit_adam(self.h, ctypes.c_void_p(param.data_ptr()),
                                                  ctypes.c_void_p(grad.data_ptr()),
                                                  ctypes.c_void_p(state["m"].data_ptr()),
                                                  ctypes.c_void_p(state["v"].data_ptr()), param.numel(),
                                                  ctypes.c_void_p(state["step"].data_ptr()), lr, betas[0], betas[1],
                                                  eps, _stream()))

    def close(self):
        if self.h:
            self.ctx.lib.bmf_fit_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def save_checkpoint(path, density: torch.Tensor, state: dict, **extra):
    """The fitting loop's checkpoint: the learnable grids and the Adam state of
    FitPlan.adam (both moments and the device step count), with torch.save;
    extra entries (step number, hyper-parameters) are stored beside them."""
    torch.save({"density": density.detach().cpu(), "m": state["m"].detach().cpu(),
                "v": state["v"].detach().cpu(), "step": state["step"].detach().cpu(), "extra": extra}, path)


def load_checkpoint(path, device):
    """(density, Adam state, extra) from save_checkpoint, on device; the loop
    continues with FitPlan.adam(density, grad, state) as if never stopped."""
    ck = torch.load(path, map_location="cpu", weights_only=True)
    state = {k: ck[k].to(device) for k in ("m", "v", "step")}
    return ck["density"].to(device).contiguous(), state, ck["extra"]


class ExtractFit(torch.autograd.Function):
    """positions = extract(density) with the topology held fixed."""

    @staticmethod
    def forward(ctx, density, plan: FitPlan):
        pos, _, _ = plan.forward(density.detach().contiguous())
        ctx.plan = plan
        ctx.shape = density.shape
        return pos.clone()

    @staticmethod
    def backward(ctx, grad_pos):
        g = ctx.plan.backward(grad_pos)
        return g.view(ctx.shape), None


def rounded_box_sdf(p, centre, half, radius):
    """Signed distance to a box with rounded edges (half extents, corner radius)."""
    q = (p - centre).abs() - half + radius
    outside = torch.clamp(q, min=0.0).norm(dim=-1)
    inside = torch.clamp(q.max(dim=-1).values, max=0.0)
    return outside + inside - radius


def sphere_union_sdf(p, centres, radii):
    """Signed distance to a union of spheres (centres (k, 3), radii (k,))."""
    d = (p[:, None, :] - centres[None]).norm(dim=-1) - radii[None]
    return d.min(dim=1).values


def vertex_chunk_ids(info, n_verts):
    """Chunk of each output vertex, from the per-chunk table (column 0: vertex
    offset, ascending; an empty chunk shares its offset with the next one)."""
    v = torch.arange(n_verts, device=info.device, dtype=info.dtype)
    return torch.searchsorted(info[:, 0].contiguous(), v, right=True) - 1


def sphere_union_loss(pos, info, spheres):
    """Sum over chunks of the mean squared sphere-union SDF of each chunk's
    vertices.  spheres: (n_chunks, k, 4) rows of centre xyz, radius (unused rows
    are placed far away)."""
    cid = vertex_chunk_ids(info, pos.shape[0])
    sp = spheres[cid]
    d = ((pos[:, None, :] - sp[..., :3]).norm(dim=-1) - sp[..., 3]).min(dim=1).values
    cnt = info[:, 1].clamp(min=1).to(pos.dtype)
    per_chunk = torch.zeros(info.shape[0], dtype=pos.dtype, device=pos.device).index_add_(0, cid, d * d)
    return (per_chunk / cnt).sum()
