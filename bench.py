#!/usr/bin/env python
"""Benchmark of the NeuS / Neuralangelo training step on GB300.

Workload ("full"): the Neuralangelo sparse training step -- 16-level 2^22 hash
grid (base 32, finest 2048, all 16 levels active: global step 6000 of the
band schedule, FD eps 1/2048), 128^3 occupancy grid, marching step
sqrt(3)*2*0.5/512, rays resized toward 2^18 samples (at most 8192), eikonal
0.1 + curvature 5e-4 + rgb MSE, AdamW -- on 1600x1200 synthetic views of an
analytic torus/box/sphere union (seeded; Gaussian noise 0.01).  A step is one
full training iteration: update_step (occupancy refresh every 16 steps),
forward, losses, backward, optimizer step.

value : rays/s with the target views resident in HBM (rays sampled on device)
e2e   : rays/s through NeuSModel / NeuSTrainer with each step's rays and
        colours sampled on the host and copied from pinned memory, the loss
        read back.
Both forms of the path are run: "plain" (the reference's structure with the
library's encode / march / composite kernels) and, when built, "fused"; and
"fused_bg", the fused step with the sparse configs' learned NeRF++ background
added (a wider workload than the headline, reported under "forms").

--impl reference times the oracle's vectorised CPU restatement of the same
step (oracle/cpu_step.py) on the host cores, in 1024-ray sub-batches (the
reference itself is Python over tcnn/nerfacc CUDA kernels, none of which
exists here or has a CPU implementation).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "instant-angelo_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402
import torch  # noqa: E402

GLOBAL_STEP = 6000
INV_S_VARIANCE = 0.7          # inv_s = exp(7) ~ 1097, a mid-training sharpness
N_VIEWS, W, H, FOV, CAM_R = 8, 1600, 1200, 40.0, 1.5


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--forms", default="auto",
                    help="comma list of plain,fused,fused_bg (auto: all built)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-mesh", action="store_true")
    ap.add_argument("--max-rays", type=int, default=8192,
                    help="ray budget per step (profiling case: fewer rays, same model and views)")
    ap.add_argument("--sdf-case", type=int, default=0, metavar="N",
                    help="profiling case: 3 fused VolumeSDF training passes (16 levels x 2^22, "
                         "FD + curvature) on N points of the full model, then exit")
    ap.add_argument("--sdf-timing", action="store_true",
                    help="time the fused VolumeSDF forward and backward calls (CUDA events, "
                         "median of --steps passes) on the samples of one training step's march "
                         "(8192 rays through the analytic occupancy grid), then exit")
    return ap.parse_args()


# ------------------------------------------------------------------ plumbing


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi sampling of SM clock and throttle reasons.  The sampler starts
    before the warm-up steps (its own start-up then falls outside the timed
    region) and the summary keeps the samples stamped inside the window that
    `mark()` opened and closed; with fewer than three there, every sample of
    the sampler's run (warm-up and timed steps, all under load)."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    PERIOD_MS = 100

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.window = [None, None]

    def __enter__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", str(self.PERIOD_MS)], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        # wait (up to 5 s) for the first sample: the sampler is then running
        # when the warm-up steps start
        t_end = time.time() + 5.0
        while self.proc is not None and self.proc.poll() is None and time.time() < t_end:
            if os.path.getsize(self.f.name) > 0:
                break
            time.sleep(0.02)
        return self

    def mark(self, i):
        """i = 0: the timed region starts now; i = 1: it ended."""
        self.window[i] = time.time()

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait(timeout=10)

    @staticmethod
    def _stamp(s):
        import datetime
        try:
            return datetime.datetime.strptime(s.strip(), "%Y/%m/%d %H:%M:%S.%f").timestamp()
        except ValueError:
            return None

    def summary(self):
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        parsed = []
        for r in rows:
            try:
                parsed.append((self._stamp(r[0]), float(r[2]), float(r[3]),
                               {nm for nm, v in zip(names, r[6:10]) if v.strip().lower() == "active"}))
            except (ValueError, IndexError):
                continue
        t0, t1 = self.window
        inside = [p for p in parsed if p[0] is not None and t0 is not None and t1 is not None
                  and t0 - 0.05 <= p[0] <= t1 + 0.05]
        use, where = (inside, "timed steps") if len(inside) >= 3 else (parsed, "warm-up and timed steps")
        sm = [p[1] for p in use]
        reasons = set().union(*[p[3] for p in use]) if use else set()
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": use[-1][2] if use else None, "samples": len(sm),
                "period_ms": self.PERIOD_MS, "window": where, "reasons": sorted(reasons)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs"), d.get("bf16_tflops"), "measured"
    return 6800.0, 1900.0, "fallback"


# --------------------------------------------------------------- the workload


def make_views(dev):
    from angelo_gb import scenes
    return scenes.TargetViews(scenes.UnionScene(), N_VIEWS, W, H, FOV, CAM_R, seed=0, device=dev)


MAX_RAYS = 8192   # the full workload's ray budget (--max-rays shrinks it for kernel captures)
VALUE_PASSES = 3  # timed passes per form for `value` (the median is reported)
E2E_PASSES = 3    # timed passes per form for `e2e` (the median is reported)


def make_trainer(form, dev, seed=0):
    from angelo_gb import models, scenes, workloads
    from angelo_gb.system import NeuSTrainer
    torch.manual_seed(seed)
    extra = workloads.background() if form == "fused_bg" else {}
    if form == "fused_fp16_table":
        # the encode gathers from an fp16 copy of the fp32 table (made once
        # per pass); gradients and AdamW stay fp32
        extra["fused_table_dtype"] = "fp16"
    cfg = workloads.model_config("full", fused=form != "plain", **extra)
    model = models.make("neus", cfg).to(dev)
    model.train()
    with torch.no_grad():
        model.variance.variance.fill_(INV_S_VARIANCE)
        occ = scenes.analytic_occupancy(scenes.UnionScene(), 128, device=dev)
        g = model.occupancy_grid
        g.occs.copy_(occ.float())
        bits = torch.zeros(g.bits.numel() * 32, dtype=torch.int64, device=dev)
        bits[: occ.numel()] = occ.long()
        w = (bits.view(-1, 32) << torch.arange(32, device=dev)).sum(-1)
        g.bits.copy_(w.to(torch.int64).bitwise_and(0xFFFFFFFF).to(torch.int32))
        if form == "fused_bg":
            # the background grid starts with every cell occupied
            model.occupancy_grid_bg.occs.fill_(1.0)
            model.occupancy_grid_bg.bits.fill_(-1)
    # the dynamic ray count aims at 2^18 samples per step; with the learned
    # background the reference's target counts its samples too
    # (train_num_rays * (num_samples_per_ray + num_samples_per_ray_bg),
    # systems/neus.py:28), and so does the count it is compared with
    target = 1 << 18
    if form == "fused_bg":
        target = target * (cfg["num_samples_per_ray"] + cfg["num_samples_per_ray_bg"]) // cfg["num_samples_per_ray"]
    tr = NeuSTrainer(model, workloads.SYSTEM, train_num_rays=MAX_RAYS, max_train_num_rays=MAX_RAYS,
                     train_num_samples=target)
    tr.global_step = GLOBAL_STEP
    return model, tr


def step_device(tr, views, gen):
    rays, rgb = views.sample_rays(tr.train_num_rays, generator=gen)
    bg = torch.rand(3, device=rays.device, generator=gen)
    n_rays = rays.shape[0]
    loss, n_samples = tr.step(rays, rgb, bg)
    return n_rays, n_samples


class HostFeed:
    """Host-side copy of the views; rays are built on the CPU per step and copied
    from pinned memory (the reference samples on the CPU: systems/neus.py:35-118)."""

    def __init__(self, views, seed=1):
        self.images = views.images.cpu()
        self.c2w = views.c2w.cpu()
        self.dirs = views.dirs.cpu()
        self.rng = np.random.default_rng(seed)
        self.W, self.H = views.W, views.H
        self.ready = None
        self.pending = None
        self.losses = []

    def batch(self, n):
        from angelo_gb.scenes import rays_from
        idx = torch.from_numpy(self.rng.integers(0, self.images.shape[0], n))
        pix = torch.from_numpy(self.rng.integers(0, self.W * self.H, n))
        rays = rays_from(self.dirs[pix], self.c2w[idx]).contiguous().pin_memory()
        rgb = self.images[idx, pix].contiguous().pin_memory()
        bg = torch.from_numpy(self.rng.random(3).astype(np.float32)).pin_memory()
        return rays, rgb, bg

    def prepare(self, n):
        """Build the next batch (host work, fresh pinned buffers) while the
        GPU runs the current step, as a data loader's worker would."""
        self.ready = self.batch(n)

    def next(self, n):
        b = self.ready if self.ready is not None and self.ready[0].shape[0] == n else self.batch(n)
        self.ready = None
        return b

    def read_result(self):
        """Host read of the previous step's loss (waits for its copy only)."""
        if self.pending is not None:
            loss_h, done = self.pending
            done.synchronize()
            self.losses.append(float(loss_h))
            self.pending = None


def step_host(tr, feed, dev):
    rays_h, rgb_h, bg_h = feed.next(tr.train_num_rays)
    rays = rays_h.to(dev, non_blocking=True)
    rgb = rgb_h.to(dev, non_blocking=True)
    bg = bg_h.to(dev, non_blocking=True)
    loss, n_samples = tr.step(rays, rgb, bg)
    feed.prepare(tr.train_num_rays)            # next batch, overlapping this step on the GPU
    # the step's result: copied to pinned host memory on the stream, read on
    # the host once the copy completed (during the next step; the last one
    # when the timed region ends), as a training loop that logs its loss does
    loss_h = torch.empty((), dtype=loss.dtype).pin_memory()
    loss_h.copy_(loss.detach(), non_blocking=True)
    done = torch.cuda.Event()
    done.record()
    feed.read_result()
    feed.pending = (loss_h, done)
    h2d = rays_h.numel() * 4 + rgb_h.numel() * 4 + bg_h.numel() * 4
    return rays.shape[0], n_samples, h2d, loss_h.numel() * loss_h.element_size()


def max_over_ranks(x, dev, world):
    """The largest value of x over the ranks (the job's time is its slowest
    rank's); x itself with one rank."""
    if world <= 1:
        return float(x)
    t = torch.tensor([float(x)], device=dev, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(values, dev, world):
    """Element-wise sums of a list of counts over the ranks (whole-job work)."""
    if world <= 1:
        return [int(v) for v in values]
    t = torch.tensor([float(v) for v in values], device=dev, dtype=torch.float64)
    torch.distributed.all_reduce(t)
    return [int(v) for v in t.tolist()]


def timed(fn, steps, dev, world, clk=None):
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if clk is not None:
        clk.mark(0)
    e0.record()
    acc = [fn() for _ in range(steps)]
    e1.record()
    torch.cuda.synchronize(dev)
    if clk is not None:
        clk.mark(1)
    if world > 1:
        torch.distributed.barrier()
    ms = max_over_ranks(e0.elapsed_time(e1), dev, world)
    return ms, acc


# ------------------------------------------------------------------ roofline


def algorithmic_bytes(name, u):
    """Algorithmic bytes of one call (each input read once, each output
    written once, table atomics counted as read + write)."""
    if u is None:
        return None
    if name == "angelo_hashgrid_fwd":
        return u["n"] * (12 + u["active"] * 8 * 2 * u["tbytes"] + (u["L"] * 2 + 3 * u["xyz"]) * 4)
    if name == "angelo_hashgrid_bwd":
        b = 12 + (u["L"] * 2 + 3) * 4
        if u["dtable"]:
            b += u["active"] * 8 * 2 * 4 * 2
        if u["dx"]:
            b += u["active"] * 8 * 2 * u["tbytes"] + 12
        return u["n"] * b
    if name == "angelo_sdf_stencil_fwd":
        # per sample: position + curvature direction, outputs (sdf, grad,
        # feature [od + 3], laplace), and per evaluation one encoded point
        # (x 12 B, 8 corner gathers and the F features of every active level);
        # the stencil taps share corner gathers, so the kernel moves less
        per_eval = 12 + u["active"] * 2 * u["tbytes"] * (8 + 1)
        return u["n"] * (24 + 4 + 12 + (u["od"] + 3) * 4 + 4 + u["evals"] * per_eval)
    if name == "angelo_sdf_stencil_bwd":
        # per sample: position, direction, incoming gradients, and per
        # evaluation the fp32 table-gradient atomics of one encoded point
        # (8 corners x F features per active level, read + write)
        per_eval = u["active"] * 8 * 2 * 4 * 2
        return u["n"] * (24 + 4 + 12 + u["od"] * 4 + 4 + u["evals"] * per_eval)
    return None


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per processed
# sample of a call, from one ncu capture of its kernels on a step of this
# workload (the three kernels of one angelo_sdf_stencil_bwd call: 2.293 GB
# for 283,862 samples); `traffic` scales it to the launch's samples.
TRAFFIC_BYTES_PER_SAMPLE = {"angelo_sdf_stencil_bwd": 2.2934e9 / 283862}


def mlp_flops(name, u):
    """Algorithmic tensor-core FLOPs of the geometry MLP inside one fused
    VolumeSDF call (the per-unit figures of the hot-path measurement plan:
    the point 2(35*64 + 64*64 + 64*65), a stencil tap 2(35*64 + 64*64 + 64)
    for the 16-level model); the backward recomputes the forward and runs the
    two backward products (dX and dW): 3x the forward."""
    if u is None or name not in ("angelo_sdf_stencil_fwd", "angelo_sdf_stencil_bwd"):
        return None
    if u.get("levels") != 16:
        return None
    point, tap = 2 * (35 * 64 + 64 * 64 + 64 * 65), 2 * (35 * 64 + 64 * 64 + 64)
    fwd = point + (u["evals"] - 1) * tap
    return u["n"] * fwd * (3 if name == "angelo_sdf_stencil_bwd" else 1)


# tensor-pipe activity of the backward MLP kernels, from the ncu capture of
# the 65,536-point case (sm__pipe_tensor_cycles_active, both tap groups)
TENSOR_PIPE_ACTIVE = {"angelo_sdf_stencil_bwd": 0.11}


def roofline(summary, hbm_peak, peak_kind, tensor_peak=None):
    best = None
    for name, (calls, ms, units) in summary.items():
        if best is None or ms > best[2]:
            best = (name, calls, ms, units)
    if best is None:
        return None, None
    name, calls, ms, units = best
    total_bytes = 0
    for u in units:
        b = algorithmic_bytes(name, u)
        if b is None:
            total_bytes = None
            break
        total_bytes += b
    shares = {k: round(v[1], 3) for k, v in sorted(summary.items(), key=lambda kv: -kv[1][1])}
    if total_bytes is None:
        return {"kernel": name, "bound": "hbm", "achieved": None, "peak": hbm_peak,
                "unit": "GB/s", "frac": None, "traffic": None,
                "peak_source": peak_kind}, shares
    gbs = total_bytes / (ms * 1e-3) / 1e9
    traffic = None
    if name in TRAFFIC_BYTES_PER_SAMPLE:
        traffic = int(TRAFFIC_BYTES_PER_SAMPLE[name] * sum(u["n"] for u in units) / calls)
    out = {"kernel": name, "bound": "hbm", "achieved": round(gbs, 1), "peak": hbm_peak,
           "unit": "GB/s", "frac": round(gbs / hbm_peak, 4), "traffic": traffic,
           "traffic_source": "ncu DRAM bytes per sample of this call on the full step, "
           "times the launch's samples" if traffic else None,
           "bytes_per_launch": int(total_bytes / calls), "launches": calls,
           "ms_per_launch": round(ms / calls, 4), "peak_source": peak_kind}
    if name == "angelo_sdf_stencil_bwd":
        # the measured limiters of the call's kernels: the table scatter's L2
        # atomics and the tcgen05 MLP backward's epilogue issue (not HBM
        # bandwidth: its DRAM traffic is a third of the algorithmic bytes)
        out["limiter"] = ("L2 atomics (table scatter) and instruction issue of the tensor-core "
                          "MLP epilogue; DRAM traffic ~1/3 of the algorithmic bytes")
        fl = [mlp_flops(name, u) for u in units]
        if tensor_peak and all(f is not None for f in fl):
            tf = sum(fl) / (ms * 1e-3) / 1e12
            out["tensor"] = {"achieved": round(tf, 2), "peak": tensor_peak, "unit": "TFLOP/s",
                             "frac": round(tf / tensor_peak, 4),
                             "flops_per_launch": int(sum(fl) / calls),
                             "pipe_active_ncu": TENSOR_PIPE_ACTIVE.get(name),
                             "note": "useful MLP FLOPs (one bf16 product each) over the whole "
                                     "call's time; the bf16x3 form issues ~3x as many"}
    return out, shares


# -------------------------------------------------------------- CPU baseline


class CpuStep:
    """The same training step on the host cores: oracle/cpu_step.py (the
    reference's step restated in vectorised float32 torch: C restatement of
    nerfacc's march, reference initialisation, AdamW), on rays drawn like the
    GPU workload's (8 poses on the radius-1.5 sphere, 1600x1200 pixels),
    targets rendered from the analytic scene outside the timed part.  Touches
    neither CUDA nor libangelo_gb.so."""

    def __init__(self, seed=0):
        from angelo_gb import scenes, workloads
        from oracle import cpu_step
        torch.set_num_threads(os.cpu_count() or 1)
        self.scene = scenes.UnionScene()
        occ = scenes.analytic_occupancy(self.scene, 128, device="cpu").reshape(-1)
        self.step_fn = cpu_step.TrainStep(workloads.model_config("full"), workloads.SYSTEM,
                                          GLOBAL_STEP, INV_S_VARIANCE, occ, seed=seed)
        self.poses = scenes.sphere_poses(N_VIEWS, CAM_R, 0).float()
        self.dirs = scenes.pixel_directions(W, H, FOV).reshape(-1, 3)
        self.rng = np.random.default_rng(seed + 7)

    def batch(self, n):
        from angelo_gb import scenes
        pix = torch.from_numpy(self.rng.integers(0, W * H, n))
        cam = torch.from_numpy(self.rng.integers(0, N_VIEWS, n))
        rays = scenes.rays_from(self.dirs[pix], self.poses[cam]).float().contiguous()
        rgb = scenes.render_analytic(self.scene, rays).float()
        return rays, rgb

    def step(self, n):
        rays, rgb = self.batch(n)
        return self.step_fn.step(rays, rgb)


CPU_SUB_BATCH = 1024   # rays per CPU step: the 1024-ray sub-batches of the full step


def cpu_sub_batch(cs, budget_s):
    """The sub-batch size: 1024 rays, or fewer when one step of 1024 would
    exceed budget_s (estimated from a 128-ray step)."""
    dt, _ = cs.step(128)
    est = dt * CPU_SUB_BATCH / 128
    if est <= budget_s:
        return CPU_SUB_BATCH
    return int(max(64, CPU_SUB_BATCH * budget_s / est))


def cpu_baseline(steps=3, budget_s=8.0):
    cs = CpuStep(seed=11)
    n = cpu_sub_batch(cs, budget_s)
    tot_t, tot_r, tot_s = 0.0, 0, 0
    for k in range(steps):
        dt, s = cs.step(n)
        tot_t += dt
        tot_r += n
        tot_s += s
    return {"value": round(tot_r / tot_t, 2), "unit": "rays/s", "cores": torch.get_num_threads(),
            "kind": "port",
            "sample": f"{steps} step(s) of {n} rays ({tot_s} samples) of the same workload "
                      "(forward, backward, AdamW), in the oracle's vectorised float32 CPU "
                      "restatement (oracle/cpu_step.py), after one 128-ray warm-up step"}


# ---------------------------------------------------------------------- arms


def available_forms():
    forms = ["plain"]
    try:
        from angelo_gb import fused  # noqa: F401
        if fused.available():
            forms += ["fused", "fused_fp16_table", "fused_bg"]
    except ImportError:
        pass
    return forms


def run_ours(args):
    rank, world, local = dist_env()
    if world > 1:
        torch.distributed.init_process_group("nccl")
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    from angelo_gb import build, _lib
    build.build()
    views = make_views(dev)
    forms = available_forms() if args.forms == "auto" else args.forms.split(",")
    results = {}
    hbm_peak, tensor_peak, peak_kind = measured_peaks()
    for form in forms:
        model, tr = make_trainer(form, dev)
        # every measured pass starts from the same state: the model's
        # parameters and buffers (the analytic occupancy grid among them) as
        # initialised, empty optimizer moments, the initial ray count and the
        # same global step, then its own warm-up steps.  Without this, each
        # pass would train the field further, and the grid refresh every 16
        # steps (re-derived from the field) would change the samples per ray
        # from one pass to the next.
        snap = {k: v.detach().clone() for k, v in model.state_dict().items()}
        start = (tr.train_num_rays, tr.global_step)

        def reset():
            with torch.no_grad():
                for k, v in model.state_dict().items():
                    v.copy_(snap[k])
            tr.optimizer.state.clear()
            tr.train_num_rays, tr.global_step = start
            gen.manual_seed(1234 + rank)   # the same ray batches as the first pass

        gen = torch.Generator(device=dev).manual_seed(1234 + rank)
        # `value` is the median of VALUE_PASSES passes, each from the same
        # state with the same ray batches (so the same samples), each after
        # its own W warm-up steps: a pass that meets a one-off cost (a first
        # kernel load, an allocator growth, a clock ramp) does not set it
        runs = []
        with Clocks(local) as clk:
            for p in range(VALUE_PASSES):
                reset()
                for _ in range(args.warmup):
                    step_device(tr, views, gen)
                # profiler range (cudaProfilerStart/Stop) marks the timed
                # steps for a capture started with --profile-from-start off;
                # the backward kernels launch from autograd's own thread,
                # which an NVTX range of this thread would not cover
                torch.cuda.profiler.start()
                runs.append(timed(lambda: step_device(tr, views, gen), args.steps, dev, world,
                                  clk if p == 0 else None))
                torch.cuda.profiler.stop()
            clk.mark(1)
        torch.cuda.synchronize(dev)
        pass_ms = [r[0] for r in runs]
        ms, acc = sorted(runs, key=lambda r: r[0])[len(runs) // 2]
        # per-call CUDA events (roofline, kernel shares, launch count) over a
        # second timed pass of as many steps: recording them costs host time,
        # so they stay out of the pass that gives `value`
        reset()
        for _ in range(args.warmup):
            step_device(tr, views, gen)
        _lib.PROFILER.start()
        timed(lambda: step_device(tr, views, gen), args.steps, dev, world)
        _lib.PROFILER.stop()
        torch.cuda.synchronize(dev)
        summ = _lib.PROFILER.summary()
        launches = _lib.PROFILER.launches
        rays = sum(a[0] for a in acc)
        samples = sum(a[1] for a in acc)
        rl, shares = roofline(summ, hbm_peak, peak_kind, tensor_peak)
        # host-fed end-to-end through the public API; median of E2E_PASSES
        # passes, each from the same state with the same host batches
        runs_e = []
        for p in range(E2E_PASSES):
            feed = HostFeed(views, seed=77 + rank)
            reset()
            for _ in range(args.warmup):
                step_host(tr, feed, dev)
            feed.read_result()
            runs_e.append(timed(lambda: step_host(tr, feed, dev), args.steps, dev, world))
            feed.read_result()
            assert len(feed.losses) >= args.steps and all(np.isfinite(feed.losses[-args.steps:]))
        pass_ms_e2e = [r[0] for r in runs_e]
        ms_e2e, acc_e = sorted(runs_e, key=lambda r: r[0])[len(runs_e) // 2]
        rays_e = sum(a[0] for a in acc_e)
        samples_e = sum(a[1] for a in acc_e)
        rays, rays_e, samples = sum_over_ranks([rays, rays_e, samples], dev, world)
        call_gbs = {}
        for name in ("angelo_sdf_stencil_fwd", "angelo_sdf_stencil_bwd", "angelo_hashgrid_fwd",
                     "angelo_hashgrid_bwd"):
            if name in summ:
                c_, t_, u_ = summ[name]
                b_ = [algorithmic_bytes(name, u) for u in u_]
                if all(x is not None for x in b_):
                    call_gbs[name] = round(sum(b_) / (t_ * 1e-3) / 1e9, 1)
        results[form] = dict(
            call_ms_per_step={k: round(v[1] / args.steps, 4) for k, v in summ.items()},
            call_gbs=call_gbs,
            value=rays / (ms * 1e-3), ms_per_step=ms / args.steps, rays_per_step=rays / args.steps
            / world, samples_per_step=samples / args.steps / world, roofline=rl,
            pass_ms_per_step=[round(t / args.steps, 3) for t in pass_ms],
            e2e_pass_ms_per_step=[round(t / args.steps, 3) for t in pass_ms_e2e],
            kernel_ms=shares, gpu_launches=launches, clocks=clk.summary(),
            samples_target=tr.train_num_samples,
            e2e=dict(value=round(rays_e / (ms_e2e * 1e-3), 1), unit="rays/s",
                     h2d_bytes_per_step=int(np.mean([a[2] for a in acc_e])),
                     d2h_bytes_per_step=int(np.mean([a[3] for a in acc_e])),
                     ms_per_step=round(ms_e2e / args.steps, 3),
                     samples_per_step=round(samples_e / args.steps, 1)))
        del model, tr
        torch.cuda.empty_cache()
    head = "fused" if "fused" in results else forms[0]
    R = results[head]
    line = {
        "metric": "train rays/s", "value": round(R["value"], 1), "unit": "rays/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(R["ms_per_step"], 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32/bf16x3" if head != "plain" else "f32",
        "data": "synthetic: 8 seeded 1600x1200 views of an "
        "analytic torus/box/sphere union, Gaussian noise 0.01",
        "config": {"workload": "neuralangelo-sparse-train (16 lv x 2^22, 128^3 grid, 2^18 "
                   "samples/step target, FD + curvature)", "form": head,
                   "rays_per_step": round(R["rays_per_step"], 1),
                   "samples_per_step": round(R["samples_per_step"], 1),
                   "global_step": GLOBAL_STEP, "parallelism": f"replicas x{world}",
                   "precision": "hash table, encodings, alpha, transmittance, loss and AdamW in "
                   "fp32; the geometry and radiance MLPs on tcgen05 with every operand split into "
                   "a bf16 hi + lo pair (three products, ~16 significant bits per operand) and "
                   "fp32 accumulation in tensor memory" if head != "plain" else "fp32",
                   "l2": "inputs larger than L2 (hash table 0.37 GB + AdamW state 0.73 GB)",
                   "per_call_events": "roofline, kernel_ms and gpu_launches from a second "
                   "timed pass of the same number of steps",
                   "passes": "each pass (value, per-call events, e2e) starts from the same "
                   "initial model, empty optimizer moments, the analytic occupancy grid, 8192 "
                   "rays and the same global step, then W warm-up steps; the per-call pass "
                   "replays the value pass's ray batches, e2e draws its own on the host"},
        # rays/s follows the samples per ray (the ray count is resized toward
        # 2^18 samples); the per-sample figures are the steadier comparison
        "samples_per_s": round(R["samples_per_step"] * world / (R["ms_per_step"] * 1e-3), 1),
        "ns_per_sample": round(R["ms_per_step"] * 1e6 / max(R["samples_per_step"], 1.0), 3),
        "e2e": R["e2e"], "roofline": R["roofline"], "clocks": R["clocks"],
        "gpu_launches": R["gpu_launches"], "kernel_ms": R["kernel_ms"],
        "forms": {f: {"value": round(v["value"], 1), "ms_per_step": round(v["ms_per_step"], 3),
                      "rays_per_step": round(v["rays_per_step"], 1),
                      "samples_per_step": round(v["samples_per_step"], 1),
                      "samples_target": v["samples_target"],
                      "ns_per_sample": round(v["ms_per_step"] * 1e6 / max(v["samples_per_step"], 1.0), 3),
                      "pass_ms_per_step": v["pass_ms_per_step"],
                      "e2e": v["e2e"]["value"], "e2e_ms_per_step": v["e2e"]["ms_per_step"],
                      "e2e_samples_per_step": v["e2e"]["samples_per_step"],
                      "e2e_pass_ms_per_step": v["e2e_pass_ms_per_step"],
                      "call_ms_per_step": v["call_ms_per_step"],
                      "call_algorithmic_gbs": v["call_gbs"]}
                  for f, v in results.items()},
    }
    if "fused" in results and "plain" in results:
        line["fused_vs_plain"] = round(results["fused"]["value"] / results["plain"]["value"], 3)
        ns = {f: results[f]["ms_per_step"] / max(results[f]["samples_per_step"], 1.0)
              for f in ("fused", "plain")}
        line["fused_vs_plain_per_sample"] = round(ns["plain"] / ns["fused"], 3)
        line["fused_vs_plain_e2e"] = round(results["fused"]["e2e"]["value"] /
                                           results["plain"]["e2e"]["value"], 3)
    if rank == 0 and not args.no_serving and "fused" in forms:
        line["serving"] = run_serving(dev, seed=1000 + rank)
    if rank == 0 and not args.no_mesh:
        line["mesh"] = run_mesh(dev, hbm_peak)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


# ------------------------------------------------------------------ serving

SERVE_RES = ((256, 256), (512, 512), (800, 600), (1920, 1080))
SERVE_GRIDS = (64, 128, 256, 512)


def serving_requests(n_render, n_grid, rate, seed):
    """Poisson arrivals (rate per second) of renders with resolutions drawn
    uniformly from SERVE_RES and random poses on a radius-2.5 sphere,
    interleaved with SDF grids of SERVE_GRIDS points per axis."""
    from angelo_gb.scenes import look_at_c2w
    from angelo_gb.serve import RenderRequest, SdfGridRequest
    g = np.random.default_rng(seed)
    reqs = []
    t = 0.0
    kinds = ["r"] * n_render + ["g"] * n_grid
    g.shuffle(kinds)
    gi = 0
    for i, k in enumerate(kinds):
        t += g.exponential(1.0 / rate)
        if k == "r":
            v = g.normal(size=3)
            eye = tuple(2.5 * v / np.linalg.norm(v))
            W, H = SERVE_RES[g.integers(len(SERVE_RES))]
            reqs.append(RenderRequest(i, look_at_c2w(eye), int(W), int(H), arrival=t))
        else:
            reqs.append(SdfGridRequest(i, SERVE_GRIDS[gi % len(SERVE_GRIDS)], arrival=t))
            gi += 1
    return reqs


def serving_model(dev, fused):
    """The small model's architecture (8 levels x 2^16, 1 hidden layer,
    radiance MLP, near/far 0.5-4.5, 128 samples per ray) with seeded weights:
    sphere-initialised geometry and a U(-0.05, 0.05) table."""
    from angelo_gb import models, workloads
    torch.manual_seed(0)
    m = models.make("neus", workloads.model_config("small", fused=fused)).to(dev)
    m.update_step(0, 5000)
    with torch.no_grad():
        gen = torch.Generator(device="cpu").manual_seed(7)
        p = m.geometry.hashgrid.encoding.params
        p.copy_((torch.rand(p.shape, generator=gen) * 0.1 - 0.05).to(dev))
    return m.eval()


SERVE_RATES = (2.0, 4.0)   # offered loads below and near what one GPU completes (req/s)


def _serve_stats(reqs, serve, t_wall):
    renders = [q for q in reqs if isinstance(q, serve.RenderRequest)]
    grids = [q for q in reqs if isinstance(q, serve.SdfGridRequest)]
    rays = sum(q.n for q in renders)
    pts = sum(q.n for q in grids)
    makespan = max(q.done for q in reqs) - min(q.arrival for q in reqs)
    p50, p99 = serve.latency_stats(reqs)
    r50, r99 = serve.latency_stats(renders)
    return {"served_mrays_per_s": round(rays / makespan / 1e6, 3),
            "served_mpts_per_s_sdf": round(pts / makespan / 1e6, 3),
            "p50_ms": round(p50, 2), "p99_ms": round(p99, 2),
            "render_p50_ms": round(r50, 2), "render_p99_ms": round(r99, 2),
            "rays": rays, "sdf_points": pts, "makespan_s": round(makespan, 3),
            "wall_s": round(t_wall, 3)}


def run_serving(dev, seed, n_render=12, n_grid=3, rate=50.0):
    """Served Mrays/s and p50/p99 latency of the persistent loop on Poisson
    request streams: the same requests (renders of SERVE_RES at random poses,
    SDF grids of SERVE_GRIDS) offered at SERVE_RATES (below and near what the
    GPU completes) and at `rate` (the configured 50 req/s, an overload: its
    latencies are queueing).  The reference's sequential eval path (plain
    kernels, one request at a time in arrival order, 2048-ray chunks moved to
    the host) serves the same stream at the highest sweep rate."""
    from angelo_gb import serve
    m = serving_model(dev, fused=True)
    srv = serve.Server(m, ray_bucket=1 << 14, max_samples_per_ray=128, point_bucket=1 << 21,
                       hbm_reserve=8 << 30)
    warm = serving_requests(2, 1, rate, seed + 1)
    srv.run(warm, realtime=False)
    rows = {}
    for lam in SERVE_RATES + (rate,):
        reqs = serving_requests(n_render, n_grid, lam, seed)
        srv.buckets = srv.overflows = 0
        t0 = time.perf_counter()
        srv.run(reqs, realtime=True)
        rows[f"{lam:g}"] = dict(_serve_stats(reqs, serve, time.perf_counter() - t0),
                                buckets=srv.buckets, overflows=srv.overflows)
    head = rows[f"{rate:g}"]
    out = {"workload": f"small-model field, {n_render} renders {SERVE_RES} + {n_grid} SDF grids "
                       f"{SERVE_GRIDS[:n_grid]}^3, Poisson arrivals, 128 samples/ray, "
                       f"{len(srv.rbs)} render streams + 1 SDF stream",
           **head, "by_rate_req_per_s": rows}
    del srv
    torch.cuda.empty_cache()
    # the reference's serving path on the same stream (the highest sweep rate)
    plain = serving_model(dev, fused=False)
    lam = SERVE_RATES[-1]
    seq = serving_requests(n_render, n_grid, lam, seed)
    t0 = time.perf_counter()
    serve.sequential_plain(plain, seq)
    st = _serve_stats(seq, serve, time.perf_counter() - t0)
    out["plain_sequential"] = dict(st, stream=f"the same {len(seq)} requests at {lam:g} req/s")
    fast = rows[f"{lam:g}"]
    out["served_vs_plain"] = round(fast["served_mrays_per_s"] / st["served_mrays_per_s"], 2)
    out["p99_vs_plain"] = round(st["p99_ms"] / max(fast["p99_ms"], 1e-3), 2)
    del plain
    torch.cuda.empty_cache()
    return out


MESH_RES = 512


def run_mesh(dev, hbm_peak, res=MESH_RES):
    """Mesh extraction (models/geometry.py:79-113, export.py:57-78), measured
    three ways: marching cubes on a resident res^3 lattice of the union
    scene's analytic SDF (device time, CUDA events, the lattice larger than
    L2); the same from a pinned host lattice with the mesh read back (wall
    clock); and the full model's export at isosurface resolution 512 (field
    lattice + triangulation + vertex colours and normals, to host tensors).
    The CPU figure is the oracle's numpy restatement on a 128^3 block of the
    same lattice that the torus tube's inner wall crosses."""
    from angelo_gb import mesh, models, scenes, workloads
    from angelo_gb.config import to_config
    ax = torch.linspace(-0.5, 0.5, res, device=dev)
    X, Y, Z = torch.meshgrid(ax, ax, ax, indexing="ij")
    lat = scenes.UnionScene().sdf(torch.stack([X, Y, Z], -1)).contiguous()
    del X, Y, Z
    sp = 1.0 / (res - 1)
    org, spc = (-0.5, -0.5, -0.5), (sp, sp, sp)
    for _ in range(3):
        v, f = mesh.marching_cubes(lat, 0.0, org, spc)
    times = []
    for _ in range(10):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record()
        v, f = mesh.marching_cubes(lat, 0.0, org, spc)
        e1.record()
        torch.cuda.synchronize(dev)
        times.append(e0.elapsed_time(e1))
    ms = statistics.median(times)
    cells = (res - 1) ** 3
    nbytes = lat.numel() * 4 + v.shape[0] * 12 + f.shape[0] * 24
    out = {"workload": f"marching cubes, {res}^3 lattice of the torus/box/sphere union SDF at "
                       "level 0", "vertices": int(v.shape[0]), "triangles": int(f.shape[0]),
           "ms": round(ms, 3), "gcells_per_s": round(cells / ms / 1e6, 3),
           "roofline": {"bound": "hbm", "achieved": round(nbytes / ms / 1e6, 1),
                        "peak": hbm_peak, "unit": "GB/s",
                        "frac": round(nbytes / ms / 1e6 / hbm_peak, 4),
                        "bytes": int(nbytes), "note": "lattice read once + mesh written once"}}
    lat_h = lat.cpu().pin_memory()
    walls = []
    for i in range(4):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        v2, f2 = mesh.marching_cubes(lat_h.to(dev, non_blocking=True), 0.0, org, spc)
        v2, f2 = v2.cpu(), f2.cpu()
        walls.append(time.perf_counter() - t0)
    out["e2e"] = {"ms": round(1e3 * statistics.median(walls[1:]), 2),
                  "h2d_bytes": lat_h.numel() * 4, "d2h_bytes": v2.numel() * 4 + f2.numel() * 8}
    del lat, v, f, v2, f2
    torch.cuda.empty_cache()
    # the reference's export path on the full model (isosurface resolution 512)
    torch.manual_seed(0)
    m = models.make("neus", workloads.model_config("full", fused=True)).to(dev).eval()
    m.update_step(0, GLOBAL_STEP)
    ecfg = to_config({"chunk_size": 2097152, "export_vertex_color": True})
    m.export(ecfg)
    walls = []
    for _ in range(2):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        msh = m.export(ecfg)
        walls.append(time.perf_counter() - t0)
    out["export"] = {"ms": round(1e3 * min(walls), 1), "resolution": 512,
                     "vertices": int(msh["v_pos"].shape[0]), "triangles": int(msh["t_pos_idx"].shape[0]),
                     "what": "full model (16 lv x 2^22, untrained: the geometric-init sphere): SDF "
                             "lattice, triangulation, vertex colours and normals, to host tensors"}
    del m, msh
    torch.cuda.empty_cache()
    # the oracle's whole-array numpy form on a bounded block
    from oracle import mcubes as mc_oracle
    b = 128
    i0 = int(round((0.2 + 0.5) / sp)) - b // 2   # the torus tube's inner wall at x = 0.2
    j0 = k0 = res // 2 - b // 2
    blk = lat_h[i0:i0 + b, j0:j0 + b, k0:k0 + b].numpy()
    t0 = time.perf_counter()
    vb, fb = mc_oracle.marching_cubes_vec(blk, 0.0)
    dt = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": round((b - 1) ** 3 / dt / 1e6, 4), "unit": "Mcells/s",
                           "cores": 1, "kind": "port", "sample": f"{b}^3 block of the lattice "
                           f"({len(fb)} triangles), the oracle's numpy restatement"}
    return out


def run_reference(args):
    """The reference arm: the reference's training step restated on the host
    cores (oracle/cpu_step.py: vectorised float32 torch over the C
    restatement of nerfacc's march), one 1024-ray sub-batch per step (fewer
    only if a step would take longer than a few seconds), W untimed and K
    timed steps.  The reference itself is Python over tcnn / nerfacc CUDA
    kernels that have no CPU implementation, and its source tree is not
    present where the benchmark runs.  No GPU work: neither CUDA nor
    libangelo_gb.so is touched."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    budget = max(2.0, min(8.0, 150.0 / max(1, args.steps + args.warmup)))
    cs = CpuStep(seed=0)
    n = cpu_sub_batch(cs, budget)
    for _ in range(args.warmup):
        cs.step(n)
    t_tot, r_tot, s_tot = 0.0, 0, 0
    for _ in range(args.steps):
        dt, s = cs.step(n)
        t_tot += dt
        r_tot += n
        s_tot += s
    v = r_tot / t_tot
    print(json.dumps({
        "impl": "reference", "metric": "train rays/s", "value": round(v, 2), "unit": "rays/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * t_tot / args.steps, 2), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "neuralangelo-sparse-train (16 lv x 2^22, 128^3 grid, 2^18 "
                   "samples/step target, FD + curvature)", "rays_per_step": n,
                   "samples_per_step": round(s_tot / args.steps, 1), "global_step": GLOBAL_STEP},
        "samples_per_s": round(s_tot / t_tot, 1),
        "cpu_baseline": {"value": round(v, 2), "unit": "rays/s", "cores": torch.get_num_threads(),
                         "kind": "port", "sample": f"{args.steps} steps of {n} rays "
                         f"({s_tot} samples), forward + backward + AdamW, in the oracle's "
                         "vectorised float32 CPU restatement (oracle/cpu_step.py)"},
        "e2e": {"value": round(v, 2), "unit": "rays/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}), flush=True)


def run_sdf_case(n):
    """A small standalone case of the fused VolumeSDF forward + backward of the
    full model (for kernel captures): N points in the inner box, table and
    first-layer weights randomised so that every gradient path is non-zero."""
    from angelo_gb import models, workloads
    torch.manual_seed(0)
    dev = torch.device("cuda:0")
    m = models.make("neus", workloads.model_config("full", fused=True)).to(dev).train()
    m.update_step(0, GLOBAL_STEP)
    g = m.geometry
    with torch.no_grad():
        g.hashgrid.encoding.params.uniform_(-0.05, 0.05)
        g.network.layers[0].weight_v[:, 3:].normal_(0, 0.05)
    pts = (torch.rand(n, 3, device=dev) - 0.5) * 0.8
    for _ in range(3):
        g.zero_grad()
        sdf, grad, feat, lap = g(pts, True, True, True)
        (sdf.sum() + grad.sum() + feat.sum() + lap.sum()).backward()
    torch.cuda.synchronize()
    print(json.dumps({"sdf_case": n, "ok": True}), flush=True)


def run_sdf_timing(steps, warmup):
    """Median CUDA-event time of angelo_sdf_stencil_fwd and _bwd on a fixed
    sample set: the march of 8192 camera rays (seeded) through the analytic
    occupancy grid of the full workload, the model at the benchmark's state
    with the table U(-0.05, 0.05) and the first layer's hash columns
    N(0, 0.05^2).  The same work on every build, for comparing kernels."""
    from angelo_gb import _lib, scenes
    dev = torch.device("cuda:0")
    model, tr = make_trainer("fused", dev)
    model.update_step(0, GLOBAL_STEP)
    g = model.geometry
    with torch.no_grad():
        gen = torch.Generator(device="cpu").manual_seed(7)
        p = g.hashgrid.encoding.params
        p.copy_((torch.rand(p.shape, generator=gen) * 0.1 - 0.05).to(dev))
        wv = g.network.layers[0].weight_v
        wv[:, 3:].copy_((torch.randn(wv[:, 3:].shape, generator=gen) * 0.05).to(dev))
    poses = scenes.sphere_poses(N_VIEWS, CAM_R, 0).float().to(dev)
    dirs = scenes.pixel_directions(W, H, FOV, device=dev).reshape(-1, 3)
    rg = torch.Generator(device=dev).manual_seed(3)
    pix = torch.randint(0, W * H, (MAX_RAYS,), device=dev, generator=rg)
    cam = torch.randint(0, N_VIEWS, (MAX_RAYS,), device=dev, generator=rg)
    rays = scenes.rays_from(dirs[pix], poses[cam]).contiguous()
    model.randomized = False
    o, d = rays[:, :3].contiguous(), rays[:, 3:].contiguous()
    ri, t0, t1, _ = model.march_rays(o, d)
    pos = (o[ri.long()] + d[ri.long()] * ((t0 + t1) * 0.5)[:, None]).contiguous()
    n = pos.shape[0]
    rd = torch.randn(n, 3, device=dev, generator=torch.Generator(device=dev).manual_seed(5))
    g.curvature_dirs_fn = lambda t: rd
    times = {"angelo_sdf_stencil_fwd": [], "angelo_sdf_stencil_bwd": []}
    for it in range(warmup + steps):
        g.zero_grad()
        _lib.PROFILER.start()
        sdf, grad, feat, lap = g(pos, True, True, True)
        (sdf.sum() + grad.sum() + feat.sum() + lap.sum()).backward()
        _lib.PROFILER.stop()
        torch.cuda.synchronize(dev)
        if it >= warmup:
            for name, (c, ms, _) in _lib.PROFILER.summary().items():
                if name in times:
                    times[name].append(ms)
    out = {"samples": n, "passes": steps}
    for name, t in times.items():
        out[name + "_ms"] = round(statistics.median(t), 4)
        out[name + "_ns_per_sample"] = round(statistics.median(t) * 1e6 / n, 3)
    print(json.dumps({"sdf_timing": out}), flush=True)


def main():
    global MAX_RAYS
    args = parse()
    MAX_RAYS = args.max_rays
    if args.sdf_case:
        run_sdf_case(args.sdf_case)
        return
    if args.sdf_timing:
        run_sdf_timing(args.steps, args.warmup)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
