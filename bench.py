"""Benchmark: the Plenoxels training step at scale (256^3 grid, 20% occupancy,
SH degree 2, 1,000,000 rays per step) on GB300.

One step = volume_render_fused (ray march + MSE adjoint, gradients scattered
into the grid) + inplace_tv_grad on density (lambda 1e-5) and on SH (1e-3),
1% contiguous cell window each + RMSprop on density (lr 30) and SH (lr 1e-2),
beta 0.95 — the order of the reference's training loop (opt/opt.py:499-595).
Inputs are seeded synthetic data with the configuration's distributions
(svox2_gb300/synthetic.py); the grid and its gradient/RMS state (1.2 GB)
exceed the 129 MB L2, so no flush is needed between steps.

Prints ONE JSON line.  `value` = rays/s with rays already in HBM; `e2e` =
the same step through the public SparseGrid API with each step's rays copied
from pinned host memory and the rendered colours copied back.  `roofline` is
for the fused render kernel (the dominant kernel): algorithmic bytes =
3648 B per evaluated sample (8 corners x (link + density + 27 SH) gathered
twice + 8 x 28 float gradients read-modify-written) + 48 B per ray.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm's CPU restatement (oracle/,
all host threads) on a bounded sample of the same step.
N > 1 (torchrun): independent replicas, one per GPU (the path has no
exchange step); value = total rays / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np
import torch

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

RESO = 256
OCC = 0.20
N_BALLS = 8
Q = 1_000_000
BYTES_PER_SAMPLE = 3648
BYTES_PER_RAY = 48
# DRAM bytes (read + write) per evaluated sample of the fused step on this workload (its two
# kernels, render_kernel<9, float, kFusedFwd> and <9, float, kFusedRev>): one ncu capture of
# three full 1M-ray steps (dram__bytes_read.sum and dram__bytes_write.sum only, a single replay
# pass per launch) measured 25.19 GB (forward) + 38.50 GB (reverse) per step over 155.83 M
# evaluated samples per step.
DRAM_BYTES_PER_SAMPLE = 408.7
# launches of this library per training step: ray_keys_kernel, 6 CUB radix-sort kernels,
# render_kernel twice (the fused step's forward and reverse kernels), add_accum_kernel,
# 2 x tv_sparse_kernel, 2 x step_mask_kernel
LAUNCHES_PER_STEP = 14
METRIC = "fused fwd+bwd rays/s at 256^3 SH9 (train step: render+MSE adjoint, TV, RMSprop)"
WORKLOAD = "train step 256^3 20% occupancy SH9 FP32, 1M rays/step, fused fwd+bwd + TV + RMSprop"


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_model() -> str:
    """The host CPU's model name (/proc/cpuinfo, else lscpu)."""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.TimeoutExpired):
        pass
    return platform.processor() or platform.machine()


def reference_grid(svox2, g, device, opt_kw=None):
    """The reference's own SparseGrid (oracle/_ref/src, its unmodified package) holding the
    synthetic tables of g: links, density and SH replace the constructor's tables."""
    grid = svox2.SparseGrid(reso=2, basis_dim=9, device=device)
    grid.links = g.links.to(device)
    grid.density_data = torch.nn.Parameter(g.density.to(device))
    grid.sh_data = torch.nn.Parameter(g.sh.to(device))
    grid.capacity = int(g.density.shape[0])
    grid.opt.step_size = 0.5
    grid.opt.sigma_thresh = 1e-8
    grid.opt.stop_thresh = 1e-7
    grid.opt.background_brightness = 1.0
    for k, v in (opt_kw or {}).items():
        setattr(grid.opt, k, v)
    return grid


def reference_cpu_step(svox2, grid, o, d, gt) -> float:
    """One step of the reference's own pure-PyTorch path: volume_render(use_kernel=False) and the
    MSE loss's autograd backward (svox2/svox2.py:658-884).  Returns seconds."""
    for p in (grid.density_data, grid.sh_data):
        p.grad = None
    t0 = time.perf_counter()
    rgb = grid.volume_render(svox2.Rays(o, d), use_kernel=False)
    torch.nn.functional.mse_loss(rgb, gt).backward()
    return time.perf_counter() - t0


def reference_cpu_64(budget_runs: int = 3):
    """The reference's own CPU path on the 64^3 dense configuration in full (4096 rays, seed 0):
    median of budget_runs steps after one warm-up, or None when its package is not staged."""
    from oracle import ref_cuda
    from svox2_gb300 import synthetic as S

    svox2 = ref_cuda.import_reference_package(with_extension=False)
    if svox2 is None:
        return None
    g = S.make_grid(64, occupancy=None, seed=0)
    grid = reference_grid(svox2, g, "cpu")
    o, d, gt = S.make_rays(4096, seed=0)
    reference_cpu_step(svox2, grid, o, d, gt)
    times = [reference_cpu_step(svox2, grid, o, d, gt) for _ in range(budget_runs)]
    t = statistics.median(times)
    return {"value": 4096 / t, "unit": "rays/s", "threads": torch.get_num_threads(),
            "sample": "the reference's own volume_render(use_kernel=False) + MSE backward (its unmodified "
                      "package), 64^3 dense SH9 FP32, 4096 rays in full, median of "
                      f"{budget_runs} after a warm-up: {t:.2f} s per step"}


def max_over_ranks(ms: float, dist, device) -> float:
    """The slowest replica's time (the job's time); ms itself without torch.distributed."""
    if dist is None:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world: int, rays_per_step: int, steps: int, ms: float) -> float:
    """Rays/s of the whole job: every replica processes rays_per_step rays per step (weak scaling)."""
    return world * rays_per_step * steps / (ms / 1e3)


def build_workload(device, seed_rays: int, n_batches: int):
    from svox2_gb300 import synthetic as S
    from svox2_gb300 import SparseGrid

    g = S.make_grid(RESO, occupancy=OCC, n_balls=N_BALLS, seed=0, device=device)
    grid = SparseGrid.from_tables(g.links.to(device), g.density.to(device), g.sh.to(device))
    grid.opt.sigma_thresh = 1e-8
    grid.opt.stop_thresh = 1e-7
    grid.opt.background_brightness = 1.0
    grid.opt.step_size = 0.5
    batches = [S.make_rays(Q, seed=seed_rays + i) for i in range(n_batches)]
    return g, grid, batches


def reset_state(grid, snapshot):
    """Restore the grid tables and clear gradients and optimiser state."""
    with torch.no_grad():
        grid.density_data.copy_(snapshot[0])
        grid.sh_data.copy_(snapshot[1])
    for p in (grid.density_data, grid.sh_data):
        if p.grad is not None:
            p.grad.zero_()
    grid.density_rms = None
    grid.sh_rms = None
    grid.sparse_grad_indexer = None
    grid.sparse_sh_grad_indexer = None


def train_step(grid, rays_o, rays_d, gt, stats=None, ev=None):
    """One step of the training loop; ev = (start, stop) events that the library records
    around the ray-march kernel of the fused render."""
    from svox2_gb300 import Rays
    from svox2_gb300 import csrc as C

    if stats is None and ev is None:
        rgb = grid.volume_render_fused(Rays(rays_o, rays_d), gt)
    else:
        gd, gs = grid._get_data_grads()
        rgb = torch.empty_like(gt)
        grid.sparse_grad_indexer = torch.zeros((grid.density_data.size(0),), dtype=torch.bool,
                                               device=gt.device)
        holder = C.GridOutputGrads()
        holder.grad_density_out = gd
        holder.grad_sh_out = gs
        holder.mask_out = grid.sparse_grad_indexer
        r = C.RaysSpec()
        r.origins, r.dirs = rays_o, rays_d
        st = dict(stats or {})
        if ev is not None:      # recorded by the library just around the ray-march kernel
            st["march_start"], st["march_stop"] = ev
        C.volume_render_cuvol_fused(grid._to_cpp(), r, grid.opt._to_cpp(), gt, 0.0, 0.0, rgb, holder, stats=st)
        grid.sparse_sh_grad_indexer = grid.sparse_grad_indexer.clone()
    grid.inplace_tv_grad(grid.density_data.grad, scaling=1e-5, sparse_frac=0.01, contiguous=True)
    grid.inplace_tv_color_grad(grid.sh_data.grad, scaling=1e-3, sparse_frac=0.01, contiguous=True)
    grid.optim_density_step(30.0, beta=0.95, epsilon=1e-8)
    grid.optim_sh_step(1e-2, beta=0.95, epsilon=1e-8)
    return rgb


def cpu_sample(g, budget_s: float = 12.0, threads: int | None = None):
    """The oracle's fused fwd+bwd on a bounded sample of the same workload, plus the
    TV + RMSprop work on a proportional slice of the grid.  Returns (rays/s, cores, desc)."""
    from oracle import oracle as O
    from svox2_gb300 import synthetic as S

    threads = threads or (os.cpu_count() or 1)
    off, scl = S.grid_transform(g.reso)
    og = O.Grid(g.links.numpy(), g.density.numpy(), g.sh.numpy(), 9, off, scl)
    opt = O.Opt(1.0, 0.5, 1e-8, 1e-7)
    N = g.density.shape[0]

    def step(n):
        o, d, gt = S.make_rays(n, seed=12345)
        t0 = time.perf_counter()
        r = O.render(og, opt, o.numpy(), d.numpy(), mode=1, rgb_gt=gt.numpy(), nthreads=threads)
        rows = max(int(N * n / Q), 1)
        dd = g.density.numpy()[:rows]
        O.optim(True, dd, np.zeros_like(dd), r["grad_density"][:rows].astype(np.float32), 2, r["mask"][:rows])
        ss = g.sh.numpy()[:rows]
        O.optim(True, ss, np.zeros_like(ss), r["grad_sh"][:rows].astype(np.float32), 2, r["mask"][:rows])
        cells = max(int(0.01 * g.links.numel() * n / Q), 1)
        cl = np.arange(cells, dtype=np.int32) + g.links.numel() // 3
        O.tv_grad(g.links.numpy(), g.density.numpy(), 0, 1, 1e-5, False, cells=cl)
        O.tv_grad(g.links.numpy(), g.sh.numpy(), 0, 27, 1e-3, True, cells=cl)
        return time.perf_counter() - t0

    n = 512
    t = step(n)
    n = int(max(512, min(1 << 20, n * budget_s / max(t, 1e-3))))
    t = step(n)
    return n / t, threads, f"{n} rays of the 256^3 workload fused fwd+bwd + TV/RMSprop on {n}/{Q} of the grid"


def bg_cpu_sample(g, bg_links, bg_data, o, d, gt, budget_s: float = 10.0, threads: int | None = None):
    """The oracle's fused fwd+bwd with the MSI background on a bounded sample of the background
    workload's rays (the same half-and-half mix).  Returns (rays/s, cores, desc)."""
    from oracle import oracle as O
    from svox2_gb300 import synthetic as S

    threads = threads or (os.cpu_count() or 1)
    off, scl = S.grid_transform(g.reso)
    og = O.Grid(g.links.numpy(), g.density.numpy(), g.sh.numpy(), 9, off, scl, bg_links=bg_links, bg_data=bg_data)
    opt = O.Opt(1.0, 0.5, 1e-8, 1e-7)
    q = o.shape[0]

    def step(n):
        idx = np.concatenate([np.arange(n // 2), q // 2 + np.arange(n - n // 2)])
        t0 = time.perf_counter()
        O.render(og, opt, o[idx], d[idx], mode=1, rgb_gt=gt[idx], nthreads=threads)
        return time.perf_counter() - t0

    n = 512
    t = step(n)
    n = int(max(512, min(q, n * budget_s / max(t, 1e-3))))
    t = step(n)
    return n / t, threads, f"{n} rays of the background workload, fused fwd+bwd with the background (no TV/optimiser)"


def run_reference(args, rank, world):
    """Reference arm: the CPU restatement of the reference algorithm, all host threads."""
    if rank != 0:
        return
    from svox2_gb300 import synthetic as S

    g = S.make_grid(RESO, occupancy=OCC, n_balls=N_BALLS, seed=0)
    # size each step to ~1 s so that warmup + steps ends within a few minutes
    per_step_s = min(1.0, 150.0 / max(args.steps + args.warmup, 1))
    rate, cores, _ = cpu_sample(g, budget_s=per_step_s)
    n = max(256, int(rate * per_step_s))
    from oracle import oracle as O

    off, scl = S.grid_transform(g.reso)
    og = O.Grid(g.links.numpy(), g.density.numpy(), g.sh.numpy(), 9, off, scl)
    opt = O.Opt(1.0, 0.5, 1e-8, 1e-7)
    times = []
    for i in range(args.warmup + args.steps):
        o, d, gt = S.make_rays(n, seed=100 + i)
        t0 = time.perf_counter()
        O.render(og, opt, o.numpy(), d.numpy(), mode=1, rgb_gt=gt.numpy(), nthreads=cores)
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    tot = sum(times)
    val = n * len(times) / tot
    line = {
        "metric": METRIC, "value": val, "unit": "rays/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * Q / val, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": {"workload": WORKLOAD, "reso": RESO, "occupancy": OCC, "rays_per_step": Q},
        "cpu_baseline": {"value": val, "unit": "rays/s", "cores": cores, "kind": "port",
                         "sample": f"{n} rays per step, fused fwd+bwd of the 256^3 workload (CPU restatement)"},
        "e2e": {"value": val, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_mixed(args):
    """Mixed-precision configuration: 512^3 grid, 8% occupancy (32 balls), SH stored
    as bfloat16 or float16 (density float32, all arithmetic float32) against the
    float32 form: PSNR of an 800x800 render from a fixed camera, relative error of
    the fused-step gradients over 4M rays, fused-step throughput and forward-only render
    throughput over the same rays."""
    from svox2_gb300 import Camera, Rays, SparseGrid
    from svox2_gb300 import synthetic as S

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    reso, occ, n_balls, q = 512, 0.08, 32, 4_000_000
    g = S.make_grid(reso, occupancy=occ, n_balls=n_balls, seed=0, device=dev)
    o, d, gt = [t.to(dev) for t in S.make_rays(q, seed=2000)]
    c2w = S.look_at_c2w((0.0, 0.0, -4.0)).to(dev)
    cam = Camera(c2w, fx=1111.0, fy=1111.0, cx=400.0, cy=400.0, width=800, height=800)
    res = {}
    ref_img = ref_gd = ref_gs = None
    for name, dt in (("fp32", torch.float32), ("bf16", torch.bfloat16), ("fp16", torch.float16)):
        grid = SparseGrid.from_tables(g.links.to(dev), g.density.to(dev), g.sh.to(dev).to(dt))
        grid.opt.sigma_thresh, grid.opt.stop_thresh = 1e-8, 1e-7
        with torch.no_grad():
            img = grid.volume_render_image(cam)
        rays = Rays(o, d)
        grid.volume_render_fused(rays, gt)          # gradients of one step (from zero)
        gd, gs = [t.clone() for t in grid._get_data_grads()]
        # throughput: fused render + TV + RMSprop, as the training step
        for _ in range(2):
            train_step(grid, o, d, gt)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            train_step(grid, o, d, gt)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        # forward-only render of the same rays (what a render request runs)
        with torch.no_grad():
            grid.volume_render(rays)
            torch.cuda.synchronize()
            f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            f0.record()
            for _ in range(args.steps):
                grid.volume_render(rays)
            f1.record()
            torch.cuda.synchronize()
        fwd_ms = f0.elapsed_time(f1) / args.steps
        entry = {"rays_per_s": q / (ms / 1e3), "ms_per_step": ms,
                 "render_rays_per_s": q / (fwd_ms / 1e3), "render_ms": fwd_ms,
                 "sh_bytes": int(grid.sh_data.numel() * grid.sh_data.element_size())}
        if ref_img is None:
            ref_img, ref_gd, ref_gs = img, gd, gs
        else:
            mse = float(torch.mean((img - ref_img) ** 2))
            entry["psnr_vs_fp32_db"] = float("inf") if mse == 0 else -10.0 * np.log10(mse)
            entry["grad_density_rel_err"] = float(torch.norm(gd - ref_gd) / torch.norm(ref_gd))
            entry["grad_sh_rel_err"] = float(torch.norm(gs - ref_gs) / torch.norm(ref_gs))
        res[name] = entry
        del grid
        torch.cuda.empty_cache()
    line = {"metric": "mixed-precision SH storage at 512^3 8% occupancy: render PSNR and gradient error vs FP32, "
                      "train-step rays/s", "unit": "rays/s", "steps": args.steps, "data": "synthetic",
            "config": {"workload": "512^3, 32 balls, 8% occupancy, SH9; 4M rays/step; 800x800 image fx=fy=1111 "
                                   "from (0,0,-4)", "n_voxels": int(g.density.shape[0]),
                       "occupancy": float(g.occupancy)}, "results": res}
    print(json.dumps(line), flush=True)


def run_render(args):
    """Forward-only render of the 256^3 workload (what a render request runs): args.rays rays
    per step through the grid API (no gradient), SH stored FP32 and BF16.  Reports rays/s and the
    forward kernel's roofline: 928 B (FP32) or 496 B (BF16) per evaluated sample + 24 B per ray."""
    from svox2_gb300 import Rays, SparseGrid
    from svox2_gb300 import synthetic as S
    from svox2_gb300 import csrc as C

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    q = args.rays
    g = S.make_grid(RESO, occupancy=OCC, n_balls=N_BALLS, seed=0, device=dev)
    o, d, _ = [t.to(dev) for t in S.make_rays(q, seed=1000)]
    peak, peak_kind = _peaks()
    res = {}
    for name, dt, per_sample in (("fp32", torch.float32, 928), ("bf16", torch.bfloat16, 496)):
        grid = SparseGrid.from_tables(g.links.to(dev), g.density.to(dev), g.sh.to(dev).to(dt))
        grid.opt.sigma_thresh, grid.opt.stop_thresh = 1e-8, 1e-7
        spec, optc = grid._to_cpp(), grid.opt._to_cpp()
        rays = C.RaysSpec()
        rays.origins, rays.dirs = o, d
        with torch.no_grad():
            for _ in range(args.warmup):
                grid.volume_render(Rays(o, d))
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(args.steps):
                grid.volume_render(Rays(o, d))
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / args.steps
            # the march kernel alone, with its evaluated-sample count
            st = {"eval_samples": torch.zeros(1, dtype=torch.int64, device=dev),
                  "march_start": torch.cuda.Event(enable_timing=True),
                  "march_stop": torch.cuda.Event(enable_timing=True)}
            C.volume_render_cuvol(spec, rays, optc, stats=st)
            torch.cuda.synchronize()
        kms = st["march_start"].elapsed_time(st["march_stop"])
        n_eval = int(st["eval_samples"].item())
        achieved = (n_eval * per_sample + 24 * q) / (kms / 1e3) / 1e9
        res[name] = {"rays_per_s": q / (ms / 1e3), "ms_per_step": ms, "kernel_ms": kms, "eval_samples": n_eval,
                     "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                  "frac": achieved / peak, "peak_kind": peak_kind}}
        del grid
    line = {"metric": "forward render rays/s at 256^3 SH9 (render_kernel fwd), FP32 and BF16 SH storage",
            "unit": "rays/s", "value": res["fp32"]["rays_per_s"], "steps": args.steps, "data": "synthetic",
            "config": {"workload": f"256^3 20% occupancy SH9, {q} rays per step, no gradient"}, "results": res}
    print(json.dumps(line), flush=True)


def run_background(args):
    """Training step with the MSI background model at the T&T configuration (64 layers,
    equirectangular 2048 x 1024 cells, 2.1 GB of background table) on the 256^3 workload:
    fused render + MSE adjoint with the background composited and differentiated in the same
    kernel, density / SH / background TV, RMSprop on all three.  Half of the rays leave the
    grid in random directions (a camera that sees the sky).  Reports rays/s, the same step on
    the same rays without the background, and the march kernel's roofline: 3648 B per evaluated
    foreground sample + 48 B per ray + 552 B per background sample (the sample's four corner
    links and 2 x 4 corner-layer rows gathered twice, 16 B per row, and the rows' gradients read,
    added and written with their two mask bytes)."""
    from svox2_gb300 import Rays, SparseGrid
    from svox2_gb300 import synthetic as S
    from svox2_gb300 import csrc as C

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    q = args.rays
    g = S.make_grid(RESO, occupancy=OCC, n_balls=N_BALLS, seed=0, device=dev)
    o, d, gt = S.make_rays(q, seed=2000)
    gen = torch.Generator().manual_seed(2001)
    dr = torch.randn((q // 2, 3), generator=gen)
    d[q // 2:] = dr / dr.norm(dim=-1, keepdim=True)
    o, d, gt = o.to(dev), d.to(dev), gt.to(dev)
    nl, bg_reso = args.bg_layers, args.bg_reso
    peak, peak_kind = _peaks()
    res = {}
    for name, with_bg in (("background", True), ("no_background", False)):
        grid = SparseGrid.from_tables(g.links.to(dev), g.density.to(dev), g.sh.to(dev))
        grid.opt.sigma_thresh, grid.opt.stop_thresh = 1e-8, 1e-7
        if with_bg:
            grid.background_nlayers, grid.background_reso = nl, bg_reso
            grid.background_links = torch.arange(2 * bg_reso * bg_reso, dtype=torch.int32,
                                                  device=dev).view(2 * bg_reso, bg_reso)
            bgd = torch.randn((2 * bg_reso * bg_reso, nl, 4), generator=torch.Generator(device=dev).manual_seed(3),
                              device=dev) * 0.3
            bgd[..., 3] = 0.1          # the reference's init_sigma_bg
            grid.background_data = torch.nn.Parameter(bgd)
        rays = Rays(o, d)

        def step():
            grid.volume_render_fused(rays, gt)
            grid.inplace_tv_grad(grid.density_data.grad, scaling=5e-5, sparse_frac=0.01, contiguous=True)
            grid.inplace_tv_color_grad(grid.sh_data.grad, scaling=5e-3, sparse_frac=0.01, contiguous=True)
            if with_bg:
                grid.inplace_tv_background_grad(grid.background_data.grad, scaling=1e-3, scaling_density=1e-3,
                                                sparse_frac=0.01, contiguous=True)
            grid.optim_density_step(30.0, beta=0.95)
            grid.optim_sh_step(1e-2, beta=0.95)
            if with_bg:
                grid.optim_background_step(3.0, 0.1, beta=0.95)

        for _ in range(max(args.warmup, 3)):
            step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            step()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        # the march kernel alone, with its sample counts
        st = {"eval_samples": torch.zeros(1, dtype=torch.int64, device=dev),
              "background_samples": torch.zeros(1, dtype=torch.int64, device=dev),
              "march_start": torch.cuda.Event(enable_timing=True),
              "march_stop": torch.cuda.Event(enable_timing=True)}
        holder = C.GridOutputGrads()
        gd, gs = grid._get_data_grads()
        holder.grad_density_out, holder.grad_sh_out = gd, gs
        if with_bg:
            holder.grad_background_out = grid._grad_buffer(grid.background_data)
        r = C.RaysSpec()
        r.origins, r.dirs = o, d
        out = torch.empty_like(gt)
        C.volume_render_cuvol_fused(grid._to_cpp(), r, grid.opt._to_cpp(), gt, 0.0, 0.0, out, holder, stats=st)
        torch.cuda.synchronize()
        kms = st["march_start"].elapsed_time(st["march_stop"])
        n_fg, n_bg = int(st["eval_samples"].item()), int(st["background_samples"].item())
        achieved = (3648 * n_fg + 48 * q + 552 * n_bg) / (kms / 1e3) / 1e9
        res[name] = {"rays_per_s": q / (ms / 1e3), "ms_per_step": ms, "kernel_ms": kms, "eval_samples": n_fg,
                     "background_samples": n_bg,
                     "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                  "frac": achieved / peak, "peak_kind": peak_kind}}
        if with_bg and not args.no_cpu_baseline:
            v, cores, desc = bg_cpu_sample(g, grid.background_links.cpu().numpy(),
                                           grid.background_data.data.cpu().numpy(), o.cpu().numpy(),
                                           d.cpu().numpy(), gt.cpu().numpy())
            res["cpu_baseline"] = {"value": v, "unit": "rays/s", "cores": cores, "kind": "port", "sample": desc}
        del grid
        torch.cuda.empty_cache()
    line = {"metric": f"fused fwd+bwd rays/s at 256^3 SH9 with the MSI background ({nl} layers, {bg_reso} reso)",
            "unit": "rays/s", "value": res["background"]["rays_per_s"], "steps": args.steps, "dtype": "f32",
            "data": "synthetic", "higher_is_better": True,
            "config": {"workload": f"train step 256^3 20% occupancy SH9 FP32 + MSI background {nl} x {2 * bg_reso} x {bg_reso}, "
                                   f"{q} rays per step, half leaving the grid in random directions"},
            "roofline": res["background"]["roofline"], "cpu_baseline": res.pop("cpu_baseline", None),
            "results": res}
    print(json.dumps(line), flush=True)


def run_serve(args):
    """Serving configuration: a Poisson stream (2000 requests/s) of render requests (square
    images, side U{64..800}, cameras on a radius-4 sphere looking at the origin) and train-step
    requests (rays ~ logU[4096, 262144]) against 16 resident grids (128^3..256^3, 5-25%
    occupancy, BF16 SH) admitted under a 150 GB budget.  The same stream runs through the
    continuous-batching RenderServer and through serial plain launches (one request at a
    time, the plain grid API), each from identical initial grids; reported are throughput
    and p50/p99 latency (arrival to result on the host) of both."""
    from svox2_gb300 import Camera, Rays, SparseGrid
    from svox2_gb300 import synthetic as S
    from svox2_gb300.serving import RenderRequest, RenderServer, TrainRequest, latency_stats

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(7)
    n_req = args.requests
    datas = {}
    for i in range(16):
        reso = int(rng.integers(128, 257))
        occ = float(rng.uniform(0.05, 0.25))
        datas[f"g{i}"] = S.make_grid(reso, occupancy=occ, n_balls=8, seed=100 + i, device=dev)

    def fresh(g):
        grid = SparseGrid.from_tables(g.links.to(dev), g.density.to(dev), g.sh.to(dev).to(torch.bfloat16))
        grid.opt.sigma_thresh, grid.opt.stop_thresh = 1e-8, 1e-7
        return grid

    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, size=n_req))
    reqs = []
    for i in range(n_req):
        gid = f"g{int(rng.integers(16))}"
        if rng.random() < 0.5:
            side = int(rng.integers(64, 801))
            v = rng.normal(size=3)
            eye = 4.0 * v / np.linalg.norm(v)
            reqs.append(RenderRequest(gid, S.look_at_c2w(tuple(eye)), side, side, fx=1.389 * side))
        else:
            q = int(np.exp(rng.uniform(np.log(4096), np.log(262144))))
            o, d, gt = S.make_rays(q, seed=5000 + i)
            reqs.append(TrainRequest(gid, o.pin_memory(), d.pin_memory(), gt.pin_memory(), tv_seed=i))
    total_rays = sum(r.width * r.height if isinstance(r, RenderRequest) else r.origins.shape[0] for r in reqs)

    # ---- continuous batching
    server = RenderServer(device=dev, hbm_budget=150e9, batch_rays=args.batch_rays, chunk_rays=args.chunk_rays)
    server.lane_depth = args.lane_depth
    for k, g in datas.items():
        server.add_grid(k, fresh(g), trainable=True)
    # warm-up: one request of each kind (graphs captured, kernels loaded), not timed
    warm = [server.submit(RenderRequest("g0", S.look_at_c2w((0.0, 0.0, -4.0)), 64, 64, fx=90.0)),
            server.submit(TrainRequest("g0", *S.make_rays(4096, seed=1), tv_seed=0)),
            server.submit(TrainRequest("g1", *S.make_rays(65536, seed=2), tv_seed=0))]
    server.run_until_idle()
    for k, g in datas.items():          # back to the initial grids
        server.remove_grid(k)
        server.add_grid(k, fresh(g), trainable=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tickets = []
    i = 0
    while i < n_req or not server.idle():
        now = time.perf_counter() - t0
        while i < n_req and arrivals[i] <= now:
            tickets.append(server.submit(reqs[i], now=t0 + arrivals[i]))
            i += 1
        server.step()
    span_b = time.perf_counter() - t0
    stats_b = latency_stats(tickets)

    # ---- serial plain launches
    grids = {k: fresh(g) for k, g in datas.items()}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lat = []
    for r, a in zip(reqs, arrivals):
        now = time.perf_counter() - t0
        if now < a:
            time.sleep(a - now)
        grid = grids[r.grid_id]
        if isinstance(r, RenderRequest):
            with torch.no_grad():
                grid.volume_render_image(Camera(r.c2w.to(dev), fx=r.fx, width=r.width, height=r.height)).cpu()
        else:
            rgb = grid.volume_render_fused(Rays(r.origins.to(dev), r.dirs.to(dev)), r.rgb_gt.to(dev))
            np.random.seed(r.tv_seed)
            grid.inplace_tv_grad(grid._grad_buffer(grid.density_data), scaling=r.tv_density, sparse_frac=r.tv_frac)
            grid.inplace_tv_color_grad(grid._grad_buffer(grid.sh_data), scaling=r.tv_sh, sparse_frac=r.tv_frac)
            grid.optim_density_step(r.lr_density, beta=r.rms_beta)
            grid.optim_sh_step(r.lr_sh, beta=r.rms_beta)
            rgb.cpu()
        lat.append(time.perf_counter() - t0 - a)
    span_s = time.perf_counter() - t0
    lat = np.array(lat)
    stats_s = {"n": int(lat.size), "p50_ms": float(np.percentile(lat, 50) * 1e3),
               "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3)}
    for kind, cls in (("render", RenderRequest), ("train", TrainRequest)):
        lk = np.array([x for x, r in zip(lat, reqs) if isinstance(r, cls)])
        if lk.size:
            stats_s[f"{kind}_p50_ms"] = float(np.percentile(lk, 50) * 1e3)
            stats_s[f"{kind}_p99_ms"] = float(np.percentile(lk, 99) * 1e3)
    line = {"metric": "serving: requests/s and p50/p99 latency, continuous batching vs serial plain launches",
            "unit": "requests/s", "value": n_req / span_b, "data": "synthetic",
            "config": {"workload": "Poisson %.0f req/s, %d requests, 50%% renders (side U{64..800}) / 50%% train "
                                   "steps (logU[4096, 262144] rays), 16 grids 128^3..256^3 5-25%% occupancy BF16 SH, "
                                   "150 GB budget" % (args.rate, n_req), "total_rays": int(total_rays),
                       "batch_rays": args.batch_rays, "chunk_rays": args.chunk_rays, "lane_depth": args.lane_depth},
            "batched": {"requests_per_s": n_req / span_b, "rays_per_s": total_rays / span_b, "makespan_s": span_b,
                        **stats_b, "batches": server.batches},
            "serial": {"requests_per_s": n_req / span_s, "rays_per_s": total_rays / span_s, "makespan_s": span_s,
                       **stats_s}}
    print(json.dumps(line), flush=True)


def run_refgpu(args):
    """The reference's own CUDA training step on the 256^3 training workload, beside this
    library's, on the same GPU in the same process: its unmodified package (oracle/_ref/src) on
    its own compiled extension (oracle/_ref), SparseGrid.volume_render_fused + inplace_tv_grad +
    inplace_tv_color_grad + optim_density_step + optim_sh_step, 1M rays per step, CUDA events.
    The plain-FP32 GPU form that this library's kernels replace."""
    from oracle import ref_cuda

    svox2 = ref_cuda.import_reference_package(with_extension=True)
    if svox2 is None or svox2.svox2._C is None:
        print(json.dumps({"config": "refgpu", "unavailable": "the reference's extension is not built here"}))
        return
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    steps, warm = min(args.steps, 10), max(args.warmup, 3)
    g, grid, batches = build_workload(dev, seed_rays=1000, n_batches=4)
    dev_batches = [tuple(t.to(dev) for t in b) for b in batches]
    rgrid = reference_grid(svox2, g, dev)

    def ref_step(o, d, gt, fused_ev=None):
        if fused_ev is not None:
            fused_ev[0].record()
        rgb = rgrid.volume_render_fused(svox2.Rays(o, d), gt)
        if fused_ev is not None:
            fused_ev[1].record()
        rgrid.inplace_tv_grad(rgrid.density_data.grad, scaling=1e-5, sparse_frac=0.01, contiguous=True)
        rgrid.inplace_tv_color_grad(rgrid.sh_data.grad, scaling=1e-3, sparse_frac=0.01, contiguous=True)
        rgrid.optim_density_step(30.0, beta=0.95, epsilon=1e-8)
        rgrid.optim_sh_step(1e-2, beta=0.95, epsilon=1e-8)
        return rgb

    def timed(step_fn, fused_evs):
        for i in range(warm):
            step_fn(*dev_batches[i % 4])
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for i in range(steps):
            step_fn(*dev_batches[i % 4], fused_evs[i])
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / steps, sum(x.elapsed_time(y) for x, y in fused_evs) / steps

    mk = lambda: [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with ClockSampler(0) as clk_ref:
        ref_ms, ref_fused_ms = timed(ref_step, mk())

    def our_step(o, d, gt, ev=None):
        return train_step(grid, o, d, gt, ev=ev)

    with ClockSampler(0) as clk_ours:
        our_ms, our_fused_ms = timed(our_step, mk())
    line = {"config": "refgpu", "workload": WORKLOAD, "rays_per_step": Q, "steps": steps, "warmup": warm,
            "reference": {"ms_per_step": ref_ms, "rays_per_s": Q / ref_ms * 1e3, "fused_render_ms": ref_fused_ms,
                          "what": "sxyu/svox2's own SparseGrid training step on its own CUDA extension, "
                                  "built unmodified for sm_103a", "clocks": clk_ref.summary()},
            "ours": {"ms_per_step": our_ms, "rays_per_s": Q / our_ms * 1e3, "fused_render_ms": our_fused_ms,
                     "clocks": clk_ours.summary()},
            "speedup_step": ref_ms / our_ms, "speedup_fused_render": ref_fused_ms / our_fused_ms}
    print(json.dumps(line), flush=True)


def run_refcpu(args):
    """The reference's own pure-PyTorch path (volume_render(use_kernel=False) + MSE backward,
    its unmodified package) on the host cores: the 64^3 dense configuration in full, and the
    256^3 training workload at the ray counts of --refcpu-rays, with a fit t = a + b Q and the
    1M-ray step it extrapolates to."""
    from oracle import ref_cuda
    from svox2_gb300 import synthetic as S

    svox2 = ref_cuda.import_reference_package(with_extension=False)
    if svox2 is None:
        print(json.dumps({"config": "refcpu", "unavailable": "the reference's package is not staged here"}))
        return
    out = {"config": "refcpu", "cpu_model": cpu_model(), "torch_threads": torch.get_num_threads(),
           "cores": os.cpu_count(), "dense64": reference_cpu_64(3)}
    g = S.make_grid(RESO, occupancy=OCC, n_balls=N_BALLS, seed=0)
    grid = reference_grid(svox2, g, "cpu")
    pts = []
    for q in [int(x) for x in args.refcpu_rays.split(",")]:
        o, d, gt = S.make_rays(q, seed=12345)
        t = reference_cpu_step(svox2, grid, o, d, gt)
        pts.append((q, t))
        print(json.dumps({"refcpu_point": {"rays": q, "seconds": t}}), flush=True)
    (q0, t0), (q1, t1) = pts[0], pts[-1]
    b = (t1 - t0) / (q1 - q0) if q1 != q0 else 0.0
    a = t0 - b * q0
    out["train256"] = {"points": [{"rays": q, "seconds": t, "rays_per_s": q / t} for q, t in pts],
                       "fit": {"a_s": a, "b_s_per_ray": b},
                       "extrapolated_1M_ray_step_s": a + b * 1_000_000,
                       "extrapolated_rays_per_s": 1_000_000 / (a + b * 1_000_000),
                       "note": "extrapolated from the fit, not measured"}
    print(json.dumps(out), flush=True)


def main():
    global Q
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--rays", type=int, default=1_000_000, help="rays per step (profiling runs use a smaller case)")
    ap.add_argument("--skip-e2e", action="store_true", help="leave out the host-copy arm (profiling runs)")
    ap.add_argument("--config", default="train",
                    choices=["train", "mixed", "serve", "render", "background", "refgpu", "refcpu"],
                    help="train: the 256^3 training step (default); mixed: 512^3 BF16/FP16 SH vs FP32; "
                         "serve: continuous-batching server vs serial launches; "
                         "render: forward-only render of the 256^3 workload, FP32 and BF16 SH; "
                         "background: the training step with the T&T MSI background; "
                         "refgpu: the reference's own CUDA training step beside this library's; "
                         "refcpu: the reference's own CPU path (64^3 in full, 256^3 ray subsets + fit)")
    ap.add_argument("--refcpu-rays", default="256,1024", help="refcpu: ray counts of the 256^3 subsets")
    ap.add_argument("--requests", type=int, default=600, help="serve: number of requests in the stream")
    ap.add_argument("--bg-layers", type=int, default=64, help="background: MSI layers (the T&T configuration's 64)")
    ap.add_argument("--bg-reso", type=int, default=1024, help="background: MSI resolution (T&T: 1024)")
    ap.add_argument("--rate", type=float, default=2000.0, help="serve: Poisson arrival rate (requests/s)")
    ap.add_argument("--rates", default="", help="serve: comma-separated arrival rates, one line each (overrides --rate)")
    ap.add_argument("--chunk-rays", type=int, default=1 << 18, help="serve: rays of a render request per batch")
    ap.add_argument("--batch-rays", type=int, default=1 << 20, help="serve: rays per lane and iteration")
    ap.add_argument("--lane-depth", type=int, default=2, help="serve: batches a lane may have queued")
    args = ap.parse_args()
    if args.config == "mixed":
        run_mixed(args)
        return
    if args.config == "serve":
        for rate in ([float(x) for x in args.rates.split(",")] if args.rates else [args.rate]):
            args.rate = rate
            run_serve(args)
        return
    if args.config == "render":
        run_render(args)
        return
    if args.config == "background":
        run_background(args)
        return
    if args.config == "refgpu":
        run_refgpu(args)
        return
    if args.config == "refcpu":
        run_refcpu(args)
        return
    Q = args.rays
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist_mod

        dist = dist_mod
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")

    if args.impl == "reference":
        run_reference(args, rank, world)
        if dist is not None:
            dist.destroy_process_group()
        return

    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    from svox2_gb300 import Rays

    n_batches = min(args.steps + args.warmup, 8)
    g, grid, host_batches = build_workload(device, seed_rays=1000 + 97 * rank, n_batches=n_batches)
    dev_batches = [tuple(t.to(device) for t in b) for b in host_batches]
    stats = {"eval_samples": torch.zeros(1, dtype=torch.int64, device=device)}
    snapshot = (grid.density_data.detach().clone(), grid.sh_data.detach().clone())

    # ---- warmup (from the initial grid; the timed arm continues from the warmed-up state)
    for i in range(args.warmup):
        o, d, gt = dev_batches[i % n_batches]
        train_step(grid, o, d, gt)
    torch.cuda.synchronize()

    # ---- timed: device-resident inputs
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t_start, t_stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stats["eval_samples"].zero_()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(device.index if device.index is not None else 0) as clk:
        t_start.record()
        for i in range(args.steps):
            o, d, gt = dev_batches[i % n_batches]
            train_step(grid, o, d, gt, stats=stats, ev=evs[i])
        t_stop.record()
        torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    total_ms = t_start.elapsed_time(t_stop)
    kern_ms = sum(a.elapsed_time(b) for a, b in evs)
    n_eval = int(stats["eval_samples"].item())
    total_ms = max_over_ranks(total_ms, dist, device)

    # ---- e2e: public API, rays from pinned host memory, colours back to the host
    if args.skip_e2e:
        e2e_ms = float("nan")
    else:
        reset_state(grid, snapshot)   # both arms train from the same initial grid
        e2e_ms = run_e2e(args, grid, host_batches, device, n_batches, dist)
    value = whole_job_rate(world, Q, args.steps, total_ms)
    e2e_val = whole_job_rate(world, Q, args.steps, e2e_ms)
    emit(args, rank, world, g, value, e2e_val, total_ms, kern_ms, n_eval, clk)
    if dist is not None:
        dist.destroy_process_group()


def run_e2e(args, grid, host_batches, device, n_batches, dist):
    """The training step through the public grid API with host buffers: every step copies its
    rays and targets from pinned host memory and reads its colours back.  The copies run on a
    copy stream, double-buffered, so the next step's upload and the previous step's download
    overlap the current step's kernels, as a training loop feeding the GPU would do."""
    pinned = [tuple(t.pin_memory() for t in b) for b in host_batches]
    dbuf = [tuple(torch.empty((Q, 3), device=device) for _ in range(3)) for _ in range(2)]
    hout = [torch.empty((Q, 3), dtype=torch.float32).pin_memory() for _ in range(2)]
    main = torch.cuda.current_stream(device)
    copy = torch.cuda.Stream(device=device)
    ev_in = [torch.cuda.Event() for _ in range(2)]      # inputs of a buffer have landed
    ev_free = [torch.cuda.Event() for _ in range(2)]    # the step using a buffer has finished
    ev_out = [torch.cuda.Event() for _ in range(2)]     # colours of a step are on the host

    def upload(i):
        k = i % 2
        with torch.cuda.stream(copy):
            copy.wait_event(ev_free[k])
            for dst, src in zip(dbuf[k], pinned[i % n_batches]):
                dst.copy_(src, non_blocking=True)
            ev_in[k].record(copy)

    def run(n):
        upload(0)
        for i in range(n):
            k = i % 2
            main.wait_event(ev_in[k])
            if i + 1 < n:
                upload(i + 1)
            rgb = train_step(grid, *dbuf[k])
            ev_free[k].record(main)
            with torch.cuda.stream(copy):
                copy.wait_event(ev_free[k])
                hout[k].copy_(rgb, non_blocking=True)
                rgb.record_stream(copy)
                ev_out[k].record(copy)
        main.wait_event(ev_out[(n - 1) % 2])          # the last read-back ends the job

    run(args.warmup)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    e_start, e_stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e_start.record(main)
    run(args.steps)
    e_stop.record(main)
    torch.cuda.synchronize()
    e2e_ms = e_start.elapsed_time(e_stop)
    e2e_ms = max_over_ranks(e2e_ms, dist, device)
    return e2e_ms


def emit(args, rank, world, g, value, e2e_val, total_ms, kern_ms, n_eval, clk):
    peak, peak_kind = _peaks()
    per_launch_s = kern_ms / 1e3 / args.steps
    alg_bytes = (n_eval / args.steps) * BYTES_PER_SAMPLE + BYTES_PER_RAY * Q
    achieved = alg_bytes / per_launch_s / 1e9

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        rate, cores, desc = cpu_sample(g)
        cpu = {"value": rate, "unit": "rays/s", "cores": cores, "kind": "port", "sample": desc,
               "cpu_model": cpu_model(), "torch_threads": torch.get_num_threads()}
        ref_cpu = reference_cpu_64()
        if ref_cpu is not None:
            cpu["reference_cpu_path"] = ref_cpu

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "reso": RESO, "occupancy": float(g.occupancy), "n_voxels": int(
                g.density.shape[0]), "rays_per_step": Q, "l2": "no flush: grid + grads + RMS state 1.2 GB > L2",
                "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": DRAM_BYTES_PER_SAMPLE * n_eval / args.steps,
                         "traffic_note": "DRAM bytes per step of the fused step's two kernels: ncu capture "
                                         "of full 1M-ray steps (dram__bytes_read.sum + dram__bytes_write.sum), "
                                         "per evaluated sample x this step's evaluated samples",
                         "frac_note": "achieved counts the algorithmic bytes (every corner gathered twice, every "
                                      "gradient row read and written); corner reuse along a ray and between "
                                      "rays serves most of them from L1/L2, so it can exceed the DRAM peak. "
                                      "dram_achieved / dram_frac are the kernel's real DRAM traffic over its time",
                         "dram_achieved": DRAM_BYTES_PER_SAMPLE * n_eval / args.steps / per_launch_s / 1e9,
                         "dram_frac": DRAM_BYTES_PER_SAMPLE * n_eval / args.steps / per_launch_s / 1e9 / peak,
                         "peak_kind": peak_kind,
                         "kernel": "the fused step: render_kernel<9,float,kFusedFwd> (forward march, MSE "
                                   "residual, per-ray records) + render_kernel<9,float,kFusedRev> (adjoint)",
                         "kernel_ms": kern_ms / args.steps, "eval_samples_per_step": n_eval / args.steps,
                         "algorithmic_bytes_per_launch": alg_bytes},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_val, "unit": "rays/s", "h2d_bytes_per_step": 3 * Q * 3 * 4,
                    "d2h_bytes_per_step": Q * 3 * 4},
            "gpu_launches": LAUNCHES_PER_STEP * args.steps,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
