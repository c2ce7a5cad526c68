"""Benchmark of the chunk-extraction hot path on one GB300 (or N, one process each).

One step = one batched WorldOctree-style update: 4096 chunks of the FBM terrain
field y - 64 - 40 FBM(p) at mixed LOD (2048 x 33^3, 1434 x 65^3, 614 x 129^3
samples, cell size 1/2/4/8), each chunk going through density filling ->
occupancy words -> cell masks -> compaction + emission (reference Marching-Cubes
topology by default) -> 4 MeshProcessor iterations with smoothed normals,
replayed as one captured CUDA graph.  Inputs are seeded synthetic chunk
descriptors; every step writes 7.1 GB of density, far more than the 129 MB L2.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the CPU implementation of the same path (the oracle
restatement of the reference's DMCChunk / MeshProcessor code, OpenMP over
chunks like ChunkGenerator::extract_chunk) on the host cores.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "chunks/s (mixed-LOD batch vs per-chunk, same GB300, exact topology)"
# FP32 instructions of the line-separable FBM, counted from the kernel source
# (a fused multiply-add is one instruction; the denominator is the FP32
# instruction rate)
OPS_PER_SAMPLE_OCTAVE = 5   # l0, l1 (one fma each), l1 - l0, fma(w, ., l0), fma(amp, n, sum)
OPS_PER_SAMPLE = 1          # fma(-a, sum, py - h)
OPS_PER_LINE_OCTAVE = 20    # xs, ys, 2 floor, xf, yf, 2 fade (5 each), x1, y1, fr, amp
OPS_PER_LINE = 1            # py - h
OPS_PER_LAYER = 20          # 4 corners (mul + fma), alpha and beta (3 lerps of 2 each)
# DRAM bytes (read + write) of one launch of each kernel on the 4096-chunk update
# (seed 2024, Mode R, 4 sweeps + normals), from one ncu capture of
# dram__bytes_read.sum + dram__bytes_write.sum (one pass; profiles/
# dram_bytes_lod_update_4096.txt).  Other workloads scale them: the fill and
# count by samples, the emit, scan and sweeps by output indices.
DRAM_UPDATE_SAMPLES = 1_785_478_272
DRAM_UPDATE_INDICES = 167_847_141
DRAM_BYTES = {"fill": 390.0e6 + 1311.7e6 + 19.9e6 + 10.4e6,   # k_fill_terrain<16, band> + k_fill_fixup
              "count": 331.0e6 + 1462.8e6, "scan": 590.5e6 + 530.9e6, "emit": 1865.2e6 + 2281.4e6,
              "sweeps": 11777.4e6 + 8051.2e6}


def fill_fp32_ops(rows, params):
    """Algorithmic FP32 operations of one terrain fill over the update: per
    sample and octave, per line and octave, and one layer set-up per z-lattice
    cell a line enters (two for its first cell or after a jump of more than
    one cell), with z-lattice cells taken from float coordinates as the
    kernels compute them."""
    freq, lac, octaves = np.float32(params[2]), np.float32(params[3]), int(params[5])
    total = 0
    for (oz, scale, dim), n in zip(*np.unique(rows[:, [2, 3, 4]], axis=0, return_counts=True)):
        dim = int(dim)
        pz = np.float32(oz) + np.arange(dim, dtype=np.float32) * np.float32(scale)
        layers = 0
        fr = freq
        for _ in range(octaves):
            cell = np.floor(pz * fr).astype(np.int64)
            step = np.diff(cell)
            layers += 2 + int((step == 1).sum()) + 2 * int((step > 1).sum())
            fr = np.float32(fr * lac)
        lines = dim * dim
        per_chunk = (lines * dim * (OPS_PER_SAMPLE_OCTAVE * octaves + OPS_PER_SAMPLE)
                     + lines * (OPS_PER_LINE_OCTAVE * octaves + OPS_PER_LINE) + lines * layers * OPS_PER_LAYER)
        total += int(n) * per_chunk
    return total


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--mode", default="R", choices=["R", "Q"])
    p.add_argument("--field", default="fbm", choices=["fbm", "2d"],
                   help="fbm: the configs' 3D terrain FBM; 2d: the reference's default perturbed heightmap sampler")
    p.add_argument("--placement", type=int, default=1)
    p.add_argument("--iters", type=int, default=4)
    p.add_argument("--no-normals", action="store_true")
    p.add_argument("--chunks", type=int, default=4096)
    p.add_argument("--cpu-sample", type=int, default=128, help="chunks per CPU sample")
    p.add_argument("--skip-per-chunk", action="store_true")
    p.add_argument("--skip-cpu", action="store_true")
    p.add_argument("--fit-chunks", type=int, default=512)
    p.add_argument("--fit-steps", type=int, default=200)
    p.add_argument("--skip-fit", action="store_true")
    p.add_argument("--no-autotune", action="store_true", help="keep the plan's default launch tuning")
    return p.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(5)
        self.t.join(2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return d.get("hbm_gbs", 6800.0), d.get("sm_max_mhz", 2070.0), "measured"
    return 6800.0, 2070.0, "fallback"


def cpu_sample_rows(rows, n, seed):
    """A bounded, tier-stratified random sample of an update's chunks."""
    rng = np.random.default_rng(seed)
    pick = []
    for dim in np.unique(rows[:, 4]):
        idx = np.flatnonzero(rows[:, 4] == dim)
        k = max(1, int(round(n * len(idx) / len(rows))))
        pick.append(rng.choice(idx, size=min(k, len(idx)), replace=False))
    return np.sort(np.concatenate(pick))


def update_rows(args, seed=2024):
    """The update's chunk descriptors and rows (origin xyz, scale, dim, level);
    for the 2D heightmap the origins move down by 128 into its band."""
    from binarymeshfitting_gb300 import workloads
    descs, rows = workloads.lod_update(n=args.chunks, seed=seed)
    if args.field == "2d":
        for d, r in zip(descs, rows):
            d.origin[1] = float(r[1]) - 128.0
            r[1] = d.origin[1]
    return descs, rows


def field_spec(args):
    """(kind, params) of the update's density field."""
    from binarymeshfitting_gb300 import _lib as L
    from binarymeshfitting_gb300 import workloads
    if args.field == "2d":
        return L.FIELD_TERRAIN_2D, list(workloads.TERRAIN_2D_PARAMS)
    return L.FIELD_TERRAIN_FBM, list(workloads.TERRAIN_PARAMS)


def cpu_run(rows, args, threads):
    from binarymeshfitting_gb300 import workloads
    from oracle import cpu
    mode = 0 if args.mode == "R" else 1
    t0 = time.perf_counter()
    kind, params = field_spec(args)
    tot, counts = cpu.extract_batch(rows[:, :5].astype(np.float32), kind, params, mode,
                                    args.placement, args.iters, not args.no_normals, n_threads=threads)
    return time.perf_counter() - t0, tot


def run_reference(args):
    """CPU implementation of the path (the oracle port), all host threads."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    from binarymeshfitting_gb300 import workloads
    from oracle import cpu
    cpu.build()
    threads = os.cpu_count() or 1
    _, rows = update_rows(args)
    for w in range(args.warmup):
        cpu_run(rows[cpu_sample_rows(rows, args.cpu_sample, 100 + w)], args, threads)
    times, chunks = [], 0
    for k in range(args.steps):
        sub = rows[cpu_sample_rows(rows, args.cpu_sample, 1000 + k)]
        t, _ = cpu_run(sub, args, threads)
        times.append(t)
        chunks += len(sub)
    total = sum(times)
    value = chunks / total
    sample = "%d steps x ~%d tier-stratified chunks of the %d-chunk update" % (args.steps, args.cpu_sample,
                                                                                 args.chunks)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "chunks/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config(args),
            "cpu_baseline": {"value": value, "unit": "chunks/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "chunks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def tier_split(n):
    """'2048x33^3 + 1434x65^3 + 614x129^3' for the n-chunk update's tiers (the
    split workloads.lod_update draws)."""
    tiers = ((32, 0.50), (64, 0.35), (128, 0.15))
    counts = [int(round(n * f)) for _, f in tiers]
    counts[0] += n - sum(counts)
    return " + ".join("%dx%d^3" % (c, r + 1) for (r, _), c in zip(tiers, counts))


def config(args):
    return {"workload": "lod_update_%d" % args.chunks,
            "chunks": args.chunks, "chunk_samples": tier_split(args.chunks),
            "field": ("terrain y-64-40*FBM(p), 5 octaves perlin, freq 0.01, lacunarity 2, gain 0.5, seed 1337"
                      if args.field == "fbm" else
                      "perturbed 2D heightmap -(0.25 y) - 75 n(x, z) (the reference's default world sampler shape): "
                      "13 gradient-noise perturb octaves amp 0.87 freq 0.585 gain 0.488, 3 value-noise octaves, "
                      "seed 1337; chunk origins lowered by 128 to its band"),
            "topology": "mode R (reference Marching-Cubes triangles)" if args.mode == "R" else
            "mode Q (DMC quads, placement %d)" % args.placement,
            "smoothing_iters": args.iters, "smoothed_normals": not args.no_normals,
            "l2": "working set larger than L2: a step moves about %.0f GB through DRAM (ncu on the 4096-chunk "
                  "update: 29 GB, scaled by chunks), no flush between steps" % (29.0 * args.chunks / 4096),
            "parallelism": "replicas" if
            args.gpus == 1 else "weak: one independent update per GPU"}


def arena_chunks(bufs, chunk_ids, normals):
    """Host copies of the given chunks' slices of a batch arena: per chunk
    (info row, positions, indices, boundary flags, normals or None)."""
    info = bufs["info"].cpu().numpy()
    out = []
    for i in chunk_ids:
        vo, vc, io, ic = (int(x) for x in info[i, :4])
        out.append((info[i].copy(), bufs["pos"][vo:vo + vc].cpu().numpy(),
                    bufs["idx"][io:io + ic].cpu().numpy().view(np.uint32),
                    bufs["boundary"][vo:vo + vc].cpu().numpy(),
                    bufs["nrm"][vo:vo + vc].cpu().numpy() if normals else None))
    return out


def time_per_chunk_c(descs, field, mode, args, normals):
    """The plain per-chunk drop-in timed by the compiled C++ caller
    (binarymeshfitting_gb300/dropin/bmf_dropin.cpp, `time` mode) over the same
    chunk descriptors."""
    import tempfile

    from binarymeshfitting_gb300 import build
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "descs.bin")
        with open(path, "wb") as f:
            for dsc in descs:
                f.write(bytes(dsc))
        cmd = [build.DROPIN, "time", path, str(field.kind)] + ["%r" % float(field.params[i]) for i in range(8)] + [
            str(mode), str(args.placement), str(args.iters), str(int(normals)), "16"]
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        raise RuntimeError("bmf_dropin time failed: %s" % r.stderr.strip())
    out = json.loads(r.stdout)
    return {"value": out["chunks_per_s"], "unit": "chunks/s", "kind": "c_loop",
            "launches": "one bmf_extract_chunk per chunk from C++, buffers allocated once (%d kernels)" %
                        out["launches"], "vertices": out["vertices"], "seconds": out["seconds"]}


def check_parity(sub, gpu_chunks, args):
    """The oracle's CPU path on the sampled chunks of the benchmarked update
    (the chunks the CPU baseline timed) against the same chunks of the GPU
    arena: counts and digests of indices, positions, boundary flags and
    normals, bit for bit."""
    from binarymeshfitting_gb300 import workloads
    from oracle import cpu
    mode = 0 if args.mode == "R" else 1
    kind, params = field_spec(args)
    counts, want = cpu.extract_batch_digest(sub[:, :5].astype(np.float32), kind, params, mode,
                                            args.placement, args.iters, False, not args.no_normals)
    bad, with_mesh, verts = [], 0, 0
    for k, (info, pos, idx, bnd, nrm) in enumerate(gpu_chunks):
        got = cpu.chunk_digests(pos, idx, bnd, nrm)
        ok = (int(info[4]) == counts[k, 0] and int(info[1]) == counts[k, 1] and int(info[3]) == counts[k, 2]
              and int(info[5]) == 0 and tuple(int(x) for x in want[k]) == got)
        if not ok:
            bad.append(k)
        with_mesh += int(counts[k, 1] > 0)
        verts += int(counts[k, 1])
    tiers = {int(d): int((sub[:, 4] == d).sum()) for d in np.unique(sub[:, 4])}
    return {"chunks_checked": len(gpu_chunks), "chunks_with_mesh": with_mesh, "vertices_checked": verts,
            "tiers": tiers, "bit_exact": not bad, "mismatched_chunks": bad[:16],
            "compared": "per chunk: contains_mesh, vertex and index counts, status, and digests of indices, "
                        "positions, boundary flags and normals (oracle CPU path vs the GPU arena)"}


def run_fit(ctx, args, stream):
    """Batched fitting: forward / backward kernel times (bwd/fwd) and an Adam
    loop on fit_chunks learnable 65^3 grids with sphere-union targets."""
    import torch

    from binarymeshfitting_gb300 import _lib as L
    from binarymeshfitting_gb300 import workloads
    from binarymeshfitting_gb300.fitting import FitPlan, sphere_union_loss

    n, dim, iters = args.fit_chunks, 65, 8
    dens0, spheres = workloads.fit_batch(n, dim=dim, seed=77)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    plan = FitPlan(ctx, n, dim, L.PLACE_QEF, iters)
    plan_bytes = free0 - torch.cuda.mem_get_info()[0]
    pos, _, info = plan.forward(dens0)
    leaf = pos.detach().clone().requires_grad_(True)
    (gpos,) = torch.autograd.grad(sphere_union_loss(leaf, info, spheres), leaf)
    gden = torch.empty_like(dens0)
    nv = plan.n_verts
    for _ in range(3):
        plan.forward(dens0, sync=False)
        plan.backward(gpos, out=gden)
    torch.cuda.synchronize()
    k = max(args.steps, 5)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    e[0].record(stream)
    for _ in range(k):
        plan.forward(dens0, sync=False)
    e[1].record(stream)
    torch.cuda.synchronize()
    e[2].record(stream)
    for _ in range(k):
        plan.backward(gpos, out=gden)
    e[3].record(stream)
    torch.cuda.synchronize()
    fwd_ms = e[0].elapsed_time(e[1]) / k
    bwd_ms = e[2].elapsed_time(e[3]) / k
    # the same backward with the FP64 and the FP32 QEF adjoints, for comparison
    other = {}
    for name in ("f64", "f32"):
        plan2 = FitPlan(ctx, n, dim, L.PLACE_QEF, iters, adjoint=name)
        plan2.forward(dens0)
        for _ in range(3):
            plan2.backward(gpos, out=gden)
        torch.cuda.synchronize()
        e[2].record(stream)
        for _ in range(k):
            plan2.backward(gpos, out=gden)
        e[3].record(stream)
        torch.cuda.synchronize()
        other[name] = e[2].elapsed_time(e[3]) / k
        plan2.close()
        del plan2
    # the fitting loop: topology recomputed every forward, smoothing adjoint
    # applied without stored iterates (the sweeps are linear in positions).
    # One step = forward + loss and its position gradient (bmf_fit_loss_spheres)
    # + backward + fused Adam, all on the device with no host sync; after 3
    # eager steps (Adam's state) the step is captured as one CUDA graph and
    # replayed.  Device time by CUDA events, host time by the host clock.
    def fit_loop(lr, steps):
        param = dens0.clone()
        gden = torch.zeros_like(dens0)
        adam = {}
        loss_buf = torch.zeros(1, dtype=torch.float32, device=dens0.device)
        gpos = torch.empty((plan.vcap, 3), dtype=torch.float32, device=dens0.device)

        def step():
            plan.step_grad(param, spheres, loss_buf, gpos, gden)
            plan.adam(param, gden, adam, lr=lr)

        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        first = None
        with torch.cuda.stream(side):
            for w in range(3):
                step()
                if w == 0:
                    first = float(loss_buf.item())
        torch.cuda.current_stream().wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            step()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        ev0.record()
        for _ in range(steps - 3):
            graph.replay()
        ev1.record()
        torch.cuda.synchronize()
        host_ms = (time.perf_counter() - t0) * 1000.0 / max(steps - 3, 1)
        dev_ms = ev0.elapsed_time(ev1) / max(steps - 3, 1)
        plan.forward(param, sync=False)
        last, _ = plan.loss_spheres(spheres)
        res = (first, float(last.item()), dev_ms, host_ms)
        del graph, adam, param
        return res

    torch.cuda.reset_peak_memory_stats()
    loss_first, loss_last, step_ms, step_host_ms = fit_loop(1e-2, args.fit_steps)
    peak = torch.cuda.max_memory_allocated() + plan_bytes
    _, loss_last_lr01, _, _ = fit_loop(1e-1, args.fit_steps)
    out = {"workload": "fit_%dx65^3" % n, "fwd_ms": fwd_ms, "bwd_ms": bwd_ms, "ratio": bwd_ms / fwd_ms,
           "adjoint": "QEF adjoint from a double-float re-solve (default)", "bwd_ms_fp64_adjoint": other["f64"],
           "bwd_ms_fp32_adjoint": other["f32"],
           "vertices": nv, "fit_steps": args.fit_steps, "step_ms": step_ms, "step_ms_host": step_host_ms,
           "step_kernels": "bmf_fit_forward + bmf_fit_loss_spheres + bmf_fit_backward + bmf_fit_adam, one CUDA graph "
                           "per step",
           "peak_mem_bytes": int(peak), "loss_first": loss_first, "loss_last": loss_last,
           "loss_last_lr_0.1": loss_last_lr01,
           "note": "fwd = bmf_fit_forward (label, count, scan, offsets, emit with QEF, 8 sweeps); bwd = "
                   "bmf_fit_backward (sweep adjoint + QEF/hermite adjoint); step_ms = CUDA-event time of a "
                   "replayed step, step_ms_host = host clock over the same replays; loss_last_lr_0.1 = the same "
                   "200 steps at lr 0.1"}
    plan.close()
    return out


def run_gb300(args):
    import torch
    import torch.distributed as dist

    from binarymeshfitting_gb300 import _lib as L
    from binarymeshfitting_gb300 import workloads
    from binarymeshfitting_gb300.engine import Batch, Context

    world, rank, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ctx = Context(local)
    mode = L.MODE_R if args.mode == "R" else L.MODE_Q
    normals = not args.no_normals
    descs, rows = update_rows(args, seed=2024 + rank)
    field = workloads.terrain_field() if args.field == "fbm" else workloads.terrain2d_field()
    b = Batch(ctx, descs, field, mode=mode, placement=args.placement, iters=args.iters, smooth_normals=normals)
    # size the output arena from one sizing pass (counts are exact), then keep it
    vcap, icap = 40_000_000, 240_000_000
    for _ in range(3):
        b.allocate(vcap, icap, normals=normals)
        try:
            nv, ni = b.run(use_graph=False, sync=True)
            break
        except L.BmfError as e:
            if e.status != L.ERR_CAPACITY:
                raise
            vcap, icap = int(b.out.n_verts * 1.05) + 1024, int(b.out.n_idx * 1.05) + 1024
    bufs = b.allocate(nv + 1024, ni + 1024, normals=normals)
    stream = torch.cuda.current_stream()
    # the plan's autotuner picks the fill form / tile height and the sweep block
    # size on this very update (outside the timed region)
    if args.no_autotune:
        tuned, tune_ms = b.tuning(), []
    else:
        tuned, tune_ms = b.autotune(reps=3)
    for _ in range(max(args.warmup, 1)):
        nv, ni = b.run(use_graph=True, sync=True)
    # ---- timed region: K graph replays ----
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    l0 = ctx.launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        b.run(use_graph=True, sync=False)
    e1.record(stream)
    torch.cuda.synchronize()
    launches = ctx.launches - l0
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    if world > 1:
        dist.barrier()
    ms_t = torch.tensor([ms], device=dev)
    if world > 1:
        dist.all_reduce(ms_t, op=dist.ReduceOp.MAX)
    ms = float(ms_t.item())
    value = args.chunks * world / (ms / 1000.0)
    nv, ni = b.run(use_graph=True, sync=True)
    # the GPU meshes of the chunks the CPU leg re-computes (parity, below)
    parity_idx = cpu_sample_rows(rows, args.cpu_sample, 7)
    gpu_chunks = arena_chunks(bufs, parity_idx, normals)

    # ---- per-stage profile (outside the timed region) ----
    stages = [b.profile() for _ in range(3)]
    st_ms = [statistics.median(s[k] for s in stages) for k in range(6)]
    samples = int((rows[:, 4] ** 3).sum())
    words = int((rows[:, 4] ** 2 * np.ceil(rows[:, 4] / 32)).sum())
    hbm_peak, sm_max, peak_kind = measured_peaks()
    clock_mhz = clk["sm_mhz"] or sm_max
    fp32_peak = 152 * 128 * sm_max * 1e6 / 1e12  # nominal FP32 instruction rate at max clock, Tops/s
    fill_ops = fill_fp32_ops(rows, workloads.TERRAIN_PARAMS) if args.field == "fbm" else 0
    s_scale, i_scale = samples / DRAM_UPDATE_SAMPLES, ni / DRAM_UPDATE_INDICES
    dram = {k: v * (s_scale if k in ("fill", "count") else i_scale) for k, v in DRAM_BYTES.items()}
    # algorithmic HBM bytes of the extraction kernels (count + scan + offsets + emit)
    per_vertex = 12 + 1 + 1 + 8 + (12 if normals else 0)
    ext_bytes = words * (4 + 8 + 8 + 4) + nv * per_vertex + ni * 4
    ext_ms = st_ms[1] + st_ms[2] + st_ms[3] + st_ms[4]
    ext_gbs = ext_bytes / (ext_ms / 1000.0) / 1e9
    ext_dram = dram["count"] + dram["scan"] + dram["emit"]
    # logical bytes of the mesh processing (CSR scan + adjacency + iters x (dual, primal)),
    # each array counted once per pass: dual reads indices + positions (+ normals) and writes
    # dual points + normals; primal reads offsets, adjacency, dual points + normals, flags and
    # writes positions + normals
    n_per = 3 if args.mode == "R" else 4
    n_prims = ni // n_per
    nb = 12 if normals else 0
    # adjacency entries count 4 B each, as the algorithmic per-unit figure
    # defines them; the chunk-by-chunk sweeps store 16-bit lists for chunks of
    # at most 65535 primitives, so the bytes that kernel's own layout touches
    # (own_bytes) are fewer
    chunk_path = args.chunks >= (512 if args.mode == "R" else 2048)
    ic = bufs["info"][:, 3].cpu().numpy()
    adj16_entries = int(ic[ic // n_per <= 65535].sum()) if chunk_path else 0
    dual_b = 4 * ni + 12 * nv + nb * nv + (12 + nb) * n_prims
    primal_b = 4 * nv + 4 * ni + (12 + nb) * n_prims + 2 * nv + (12 + nb) * nv
    proc_bytes = args.iters * (dual_b + primal_b) + (1 + 4) * nv + (4 + 4) * nv + 4 * ni
    own_bytes = proc_bytes - (args.iters + 1) * 2 * adj16_entries
    proc_gbs = proc_bytes / (st_ms[5] / 1000.0) / 1e9 if st_ms[5] > 0 else 0.0
    sweep_name = ("k_sweep_chunks (CSR scan, adjacency, %d x (dual, primal), chunk by chunk)" if chunk_path
                  else "scan + adj_build + %d x (dual, primal)") % args.iters
    # the dominant kernel: the mesh-processing sweeps (HBM-bound gathers)
    roofline = {"kernel": sweep_name, "bound": "hbm", "achieved": proc_gbs, "peak": hbm_peak, "unit": "GB/s",
                "frac": proc_gbs / hbm_peak, "peak_kind": peak_kind,
                "achieved_bytes": "logical: every array of every pass counted once (%.2f GB per launch)"
                                  % (proc_bytes / 1e9),
                "own_bytes": own_bytes, "own_frac": own_bytes / (st_ms[5] / 1000.0) / 1e9 / hbm_peak
                if st_ms[5] > 0 else 0.0,
                "own_bytes_note": "the logical bytes with the kernel's 16-bit adjacency lists (%d entries) "
                                  "counted at 2 B" % adj16_entries,
                "traffic": dram["sweeps"], "traffic_unit": "DRAM bytes per launch (ncu, scaled to this update)",
                "dram_achieved": dram["sweeps"] / (st_ms[5] / 1000.0) / 1e9,
                "dram_frac": dram["sweeps"] / (st_ms[5] / 1000.0) / 1e9 / hbm_peak,
                "ms_per_launch": st_ms[5],
                "fill": {"kernels": ("k_columns2d (one thread per (x, z) column height) + k_sample_label "
                                     "(occupancy words from the heights) + k_fill_fixup (densities at the ends of "
                                     "crossings only)" if args.field == "2d" and args.mode == "R" else
                                     "k_sample_label (x-plane CTAs; one height evaluation per (x, z) column)"
                                     if args.field == "2d" else
                                     "k_fill_terrain<16, band> + k_fill_fixup (terrain FBM, occupancy words, exact "
                                     "densities at the ends of crossings)" if args.mode == "R" else
                                     "k_fill_terrain<16> (every density exact)"),
                         "ms": st_ms[0], "samples_per_s": samples / (st_ms[0] / 1000.0),
                         "dram_bytes": dram["fill"] if (args.mode == "R" and args.field == "fbm") else None,
                         "density_write_gbs": (4 * samples + 4 * words) / (st_ms[0] / 1000.0) / 1e9
                         if args.field == "2d" and args.mode != "R" else None,
                         "full_fill_fp32_ops": fill_ops, "full_fill_fp32_ops_per_sample": fill_ops / samples,
                         "full_fill_equivalent_tops": fill_ops / (st_ms[0] / 1000.0) / 1e12,
                         "full_fill_equivalent_frac": fill_ops / (st_ms[0] / 1000.0) / 1e12 / fp32_peak,
                         "fp32_peak": fp32_peak,
                         "peak_kind": "nominal 152 SM x 128 FP32 lanes x %.0f MHz (no measured FP32 peak exists)"
                                      % sm_max,
                         "note": "the band fill stops a run's octaves once their bound fixes every sign, so its "
                                 "own FP32 work is data-dependent; full_fill_* is the work of evaluating every "
                                 "octave of every sample, divided by the band fill's time"},
                "extraction_hbm": {"kernels": "count+scan+offsets+emit", "achieved": ext_gbs, "peak": hbm_peak,
                                   "unit": "GB/s", "frac": ext_gbs / hbm_peak, "bytes": ext_bytes,
                                   "dram_bytes": ext_dram, "dram_frac": ext_dram / (ext_ms / 1000.0) / 1e9 / hbm_peak,
                                   "ms": ext_ms, "peak_kind": peak_kind,
                                   "note": "issue-bound bit arithmetic: too few bytes per unit of work for HBM to "
                                           "bind"},
                "stage_ms": {"fill_label": st_ms[0], "count": st_ms[1], "scan": st_ms[2], "offsets": st_ms[3],
                             "emit": st_ms[4], "process": st_ms[5]}}

    # ---- end to end through the public API with host buffers ----
    # Every step uploads its descriptors from pinned host memory, runs the
    # update and reads everything it produced back to pinned host memory:
    # positions, indices, the chunk table, normals and boundary flags.  Two plans (double-buffered output arenas) let the read-back
    # of step i run on a copy stream while step i + 1 computes.
    h_desc_list = descs
    vbytes = nv * 12
    ibytes = ni * 4
    b2 = Batch(ctx, descs, field, mode=mode, placement=args.placement, iters=args.iters, smooth_normals=normals)
    bufs2 = b2.allocate(nv + 1024, ni + 1024, normals=normals)
    t_chosen = b.tuning()
    b2.set_tuning(**t_chosen)
    plans = [(b, bufs), (b2, bufs2)]
    hosts = [(torch.empty((nv, 3), dtype=torch.float32, pin_memory=True),
              torch.empty(ni, dtype=torch.int32, pin_memory=True),
              torch.empty((args.chunks, 6), dtype=torch.int64, pin_memory=True),
              torch.empty((nv, 3), dtype=torch.float32, pin_memory=True) if normals else None,
              torch.empty(nv, dtype=torch.uint8, pin_memory=True)) for _ in range(2)]
    copy_stream = torch.cuda.Stream()
    done = [torch.cuda.Event() for _ in range(2)]
    copied = [torch.cuda.Event() for _ in range(2)]
    h2d = args.chunks * 56
    d2h = vbytes + ibytes + args.chunks * 48 + (vbytes if normals else 0) + nv

    def e2e_step(k):
        pb, pbufs = plans[k & 1]
        hp, hi, hn, hnr, hb = hosts[k & 1]
        stream.wait_event(copied[k & 1])  # this arena's previous read-back is done
        pb.set_descs(h_desc_list, stream=stream)
        pb.run(use_graph=True, sync=False, stream=stream)
        done[k & 1].record(stream)
        with torch.cuda.stream(copy_stream):
            # indices and chunk table are final once the extraction is: their
            # read-back runs while the smoothing sweeps still compute
            pb.wait_extraction(copy_stream)
            hi.copy_(pbufs["idx"][:ni], non_blocking=True)
            hn.copy_(pbufs["info"], non_blocking=True)
            copy_stream.wait_event(done[k & 1])
            hp.copy_(pbufs["pos"][:nv], non_blocking=True)
            if hnr is not None:
                hnr.copy_(pbufs["nrm"][:nv], non_blocking=True)
            hb.copy_(pbufs["boundary"][:nv], non_blocking=True)
            copied[k & 1].record(copy_stream)

    for k in range(4):
        e2e_step(k)
    torch.cuda.synchronize()
    assert torch.equal(hosts[0][1][:ni], hosts[1][1][:ni]), "both plans produce the same update"
    e0.record(stream)
    t0 = time.perf_counter()
    for k in range(args.steps):
        e2e_step(k)
    stream.wait_event(copied[0])
    stream.wait_event(copied[1])
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = max(e0.elapsed_time(e1), (time.perf_counter() - t0) * 1000.0) / args.steps
    e2e = {"value": args.chunks * world / (e2e_ms / 1000.0), "unit": "chunks/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
           "read_back": "positions, indices, chunk table" + (", normals" if normals else "") + ", boundary flags",
           "pipeline": "two plans; step i's read-back on a copy stream overlaps step i + 1, its indices and "
                       "chunk table from the end of its extraction (bmf_batch_wait_extraction)"}
    b2.close()
    del plans, hosts, bufs2

    # ---- the plain per-chunk path (the drop-in), same chunks ----
    # Timed as a C++ caller makes it (bmf_dropin time: one bmf_extract_chunk
    # per chunk on device buffers allocated once, one context, one stream), and
    # through the Python binding for comparison.
    per_chunk = None
    if not args.skip_per_chunk and rank == 0:
        per_chunk = time_per_chunk_c(descs, field, mode, args, normals)
        per_chunk["vertices_match_batch"] = per_chunk["vertices"] == nv
        per_chunk["batch_speedup"] = value / world / per_chunk["value"]
        for dsc in descs[:16]:
            ctx.extract_chunk(dsc, field, mode=mode, placement=args.placement, iters=args.iters,
                              smooth_normals=normals)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pv = 0
        for dsc in descs:
            m = ctx.extract_chunk(dsc, field, mode=mode, placement=args.placement, iters=args.iters,
                                  smooth_normals=normals)
            pv += m.n_verts
        torch.cuda.synchronize()
        pc_s = time.perf_counter() - t0
        per_chunk["python_binding"] = {"value": args.chunks / pc_s, "unit": "chunks/s",
                                       "kind": "python ctypes, torch buffers allocated per call",
                                       "vertices_match_batch": pv == nv}

    # ---- batched fitting: backward vs forward ----
    bwd_fwd = None
    if not args.skip_fit and rank == 0:
        b.close()
        b = None
        del bufs
        torch.cuda.empty_cache()
        bwd_fwd = run_fit(ctx, args, stream)

    # ---- CPU baseline (rank 0): bounded sample of the same update, all host threads ----
    cpu_baseline = None
    parity = None
    if not args.skip_cpu and rank == 0:
        from oracle import cpu
        cpu.build()
        threads = os.cpu_count() or 1
        sub = rows[cpu_sample_rows(rows, args.cpu_sample, 7)]
        cpu_run(sub[:8], args, threads)
        t, _ = cpu_run(sub, args, threads)
        cpu_baseline = {"value": len(sub) / t, "unit": "chunks/s", "cores": threads, "kind": "port",
                        "sample": "%d tier-stratified chunks of the %d-chunk update, OpenMP over chunks" %
                                  (len(sub), args.chunks)}
        parity = check_parity(sub, gpu_chunks, args)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "chunks/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config(args),
                "samples_per_s": samples * world / (ms / 1000.0),
                "vertices_per_s": nv * world / (ms / 1000.0), "vertices_per_step": nv, "indices_per_step": ni,
                "roofline": roofline, "cpu_baseline": cpu_baseline, "parity": parity, "e2e": e2e,
                "per_chunk": per_chunk,
                "gpu_launches": launches, "clocks": clk, "bwd_fwd": bwd_fwd,
                "tuning": {"chosen": tuned, "candidates_ms": tune_ms,
                           "candidates": "fill (mode, run): (0,8) (1,4) (1,8) (1,16) (2,4) (2,8) (2,16); "
                                         "sweep block: 128 256 512"}}
        print(json.dumps(line), flush=True)
    if b is not None:
        b.close()
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
