"""Continuous-batching serving loop over resident grids.

Requests:
  * RenderRequest(grid_id, camera)      -> the image [H, W, 3] (what volume_render_image renders)
  * TrainRequest(grid_id, rays, rgb_gt) -> one training step on the grid (fused render + MSE
    adjoint, TV on density and SH, RMSprop on both, as the reference's training loop), and the
    rendered colours [Q, 3].

How requests run (``RenderServer``):
  * Grids stay resident on the device.  ``add_grid`` admits a grid only if its bytes (tables,
    and for trainable grids gradients, RMSprop state and mask) fit the HBM budget with the
    grids already resident; otherwise it raises ``AdmissionError``.
  * ``submit`` validates a request on the host (unknown grid, shapes, dtypes, sizes) and raises
    ``ValueError`` for a malformed one before anything is launched.
  * Each iteration of the loop (``step``) admits queued requests while request slots and
    device memory allow (their ray and output buffers count against the budget), fails
    requests that waited longer than their timeout (``RequestTimeout``), and plans one batch
    per lane: render rays (large images are cut into chunks so that new arrivals join at the
    next iteration) and train steps (one per grid).  Rays of different requests and grids go
    into one persistent kernel launch per lane (svx_render_batch), replayed from a captured
    CUDA graph; the render lane and the train lane run on two streams and overlap.
  * Each grid sees its requests in arrival order: a render waits for earlier train steps on its
    grid, a train step waits for every earlier request on its grid.  So every result equals
    what serial execution in arrival order gives (renders bit for bit; train steps up to the
    order of atomic additions).

The host-side logic (``Scheduler``) has no CUDA dependency and is tested on the CPU with a fake
executor; ``RenderServer`` executes its plans on the GPU.
"""
from __future__ import annotations

import ctypes as C
import itertools
import time
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Tuple

import numpy as np
import torch


class AdmissionError(RuntimeError):
    """A grid or request does not fit the device-memory budget."""


class RequestTimeout(TimeoutError):
    """A request waited longer than its timeout before it could be admitted."""


# ---------------------------------------------------------------- requests

@dataclass
class RenderRequest:
    grid_id: str
    c2w: torch.Tensor                 # [3|4, 4] OpenCV camera-to-world
    width: int
    height: int
    fx: float
    fy: Optional[float] = None
    cx: Optional[float] = None
    cy: Optional[float] = None


@dataclass
class TrainRequest:
    grid_id: str
    origins: torch.Tensor             # [Q, 3] float32 (host or device)
    dirs: torch.Tensor                # [Q, 3] float32, unit
    rgb_gt: torch.Tensor              # [Q, 3] float32
    lr_density: float = 30.0
    lr_sh: float = 1e-2
    rms_beta: float = 0.95
    tv_density: float = 1e-5
    tv_sh: float = 1e-3
    tv_frac: float = 0.01
    tv_seed: int = 0                  # start of the TV cell windows (host RNG, as the reference)
    # grids with an MSI background (the reference's opt/opt.py defaults, 113-127 and 226-229)
    lr_sigma_bg: float = 3.0
    lr_color_bg: float = 0.1
    tv_background_sigma: float = 1e-2
    tv_background_color: float = 1e-2
    tv_background_frac: float = 0.01


@dataclass
class Ticket:
    """Handle of a submitted request."""
    id: int
    kind: str                         # "render" | "train"
    grid_id: str
    n_rays: int
    arrival: float
    deadline: Optional[float]
    request: object
    state: str = "queued"             # queued -> admitted -> done | failed
    bytes: int = 0
    rays_launched: int = 0
    rays_done_event: list = field(default_factory=list)
    result: Optional[torch.Tensor] = None
    error: Optional[BaseException] = None
    finish: Optional[float] = None
    # executor-owned buffers
    buf: dict = field(default_factory=dict)

    @property
    def done(self) -> bool:
        return self.state in ("done", "failed")

    @property
    def latency(self) -> Optional[float]:
        return None if self.finish is None else self.finish - self.arrival


# ---------------------------------------------------------------- host-side scheduler

@dataclass
class Chunk:
    ticket: Ticket
    start: int                        # first ray of the request in this chunk
    count: int


class Scheduler:
    """Admission, per-grid ordering and batch planning (no CUDA).

    budget_bytes: device memory available to resident grids and in-flight requests.
    max_inflight: request slots.  batch_rays: rays per lane and iteration.
    chunk_rays: largest piece of one render request per iteration.
    """

    def __init__(self, budget_bytes: float, max_inflight: int = 64, batch_rays: int = 262144,
                 chunk_rays: int = 65536, default_timeout: Optional[float] = None,
                 work_done: Optional[Callable[[Ticket], bool]] = None):
        # work_done(t): the request's device work has completed (its results may still be on
        # their way to the host); later conflicting requests on its grid may then start.
        self.work_done = work_done or (lambda t: t.done)
        self.budget = int(budget_bytes)
        self.max_inflight = max_inflight
        self.batch_rays = batch_rays
        self.chunk_rays = chunk_rays
        self.default_timeout = default_timeout
        self.grid_bytes: Dict[str, int] = {}
        self.queue: List[Ticket] = []          # arrival order
        self.active: List[Ticket] = []         # admitted, not done, arrival order
        self.pending: Dict[str, List[Ticket]] = {}   # per grid: queued + active tickets, arrival order
        self._ids = itertools.count()

    # -- grids
    def used_bytes(self) -> int:
        return sum(self.grid_bytes.values()) + sum(t.bytes for t in self.active)

    def add_grid(self, grid_id: str, nbytes: int) -> None:
        if grid_id in self.grid_bytes:
            raise ValueError(f"grid {grid_id!r} already resident")
        if self.used_bytes() + nbytes > self.budget:
            raise AdmissionError(f"grid {grid_id!r} needs {nbytes} B; {self.budget - self.used_bytes()} B of the "
                                 f"{self.budget} B budget are free")
        self.grid_bytes[grid_id] = int(nbytes)
        self.pending.setdefault(grid_id, [])

    def remove_grid(self, grid_id: str) -> None:
        if self.pending.get(grid_id):
            raise RuntimeError(f"grid {grid_id!r} has requests in flight")
        self.grid_bytes.pop(grid_id)
        self.pending.pop(grid_id, None)

    # -- requests
    def new_ticket(self, kind: str, grid_id: str, n_rays: int, nbytes: int, request, now: float,
                   timeout: Optional[float]) -> Ticket:
        if grid_id not in self.grid_bytes:
            raise ValueError(f"unknown grid {grid_id!r}")
        if n_rays <= 0:
            raise ValueError("a request needs at least one ray")
        if kind == "train" and n_rays > self.batch_rays:
            raise ValueError(f"a train step of {n_rays} rays exceeds the batch of {self.batch_rays} rays")
        if nbytes + sum(self.grid_bytes.values()) > self.budget:
            raise AdmissionError(f"request needs {nbytes} B, more than the budget leaves beside the grids")
        timeout = self.default_timeout if timeout is None else timeout
        t = Ticket(next(self._ids), kind, grid_id, n_rays, now, None if timeout is None else now + timeout, request,
                   bytes=int(nbytes))
        self.queue.append(t)
        self.pending[grid_id].append(t)
        return t

    def expire(self, now: float) -> List[Ticket]:
        """Fail queued requests past their deadline."""
        out = []
        for t in list(self.queue):
            if t.deadline is not None and now > t.deadline:
                self.queue.remove(t)
                self.pending[t.grid_id].remove(t)
                t.state = "failed"
                t.error = RequestTimeout(f"request {t.id} waited {now - t.arrival:.3f} s")
                t.finish = now
                out.append(t)
        return out

    def admit(self) -> List[Ticket]:
        """Admit queued requests in arrival order while slots and memory allow."""
        out = []
        while self.queue and len(self.active) < self.max_inflight:
            t = self.queue[0]
            if self.used_bytes() + t.bytes > self.budget:
                break
            self.queue.pop(0)
            t.state = "admitted"
            self.active.append(t)
            out.append(t)
        return out

    def _ready(self, t: Ticket) -> bool:
        """Per-grid arrival order: a render waits for earlier train steps on its grid; a train
        step waits for every earlier request on its grid."""
        for u in self.pending[t.grid_id]:
            if u is t:
                return True
            if u.done:
                continue
            if (t.kind == "train" or u.kind == "train") and not self.work_done(u):
                return False
        return True

    def plan(self, train_busy: bool = False, render_busy: bool = False) -> Tuple[List[Chunk], List[Ticket]]:
        """One iteration: render chunks (arrival order, up to batch_rays) and train steps
        (one per grid, up to batch_rays); a busy lane gets nothing this iteration."""
        chunks: List[Chunk] = []
        room = 0 if render_busy else self.batch_rays
        for t in self.active:
            if t.kind != "render" or t.rays_launched >= t.n_rays or room <= 0 or not self._ready(t):
                continue
            n = min(self.chunk_rays, t.n_rays - t.rays_launched, room)
            chunks.append(Chunk(t, t.rays_launched, n))
            t.rays_launched += n
            room -= n
        trains: List[Ticket] = []
        if not train_busy:
            room = self.batch_rays
            grids = set()
            for t in self.active:
                if t.kind != "train" or t.rays_launched > 0 or t.grid_id in grids or t.n_rays > room:
                    continue
                if not self._ready(t):
                    continue
                trains.append(t)
                grids.add(t.grid_id)
                t.rays_launched = t.n_rays
                room -= t.n_rays
        return chunks, trains

    def finish(self, t: Ticket, now: float, error: Optional[BaseException] = None) -> None:
        t.state = "failed" if error is not None else "done"
        t.error = error
        t.finish = now
        self.active.remove(t)
        self.pending[t.grid_id].remove(t)

    def idle(self) -> bool:
        return not self.queue and not self.active


# ---------------------------------------------------------------- GPU executor

def grid_bytes(grid, trainable: bool) -> int:
    n = grid.links.numel() * 4 + grid.density_data.numel() * 4 + grid.sh_data.numel() * grid.sh_data.element_size()
    if trainable:
        N, Cc = grid.sh_data.shape
        n += 2 * (N * 4 + N * Cc * 4) + N          # gradients, RMSprop state, mask
        n += N * ((Cc + 1 + 3) // 4 * 4) * 4       # padded accumulation rows
    if grid.use_background:
        n += grid.background_links.numel() * 4 + grid.background_data.numel() * 4
        if trainable:
            n += 2 * grid.background_data.numel() * 4 + grid.background_data[..., 0].numel()
    return int(n)


class RenderServer:
    """Continuous-batching server on one GPU (see the module docstring)."""

    def __init__(self, device="cuda", hbm_budget: float = 150e9, batch_rays: int = 262144, chunk_rays: int = 65536,
                 max_inflight: int = 64, default_timeout: Optional[float] = None, use_graphs: bool = True,
                 step_size: float = 0.5, sigma_thresh: float = 1e-8, stop_thresh: float = 1e-7,
                 background_brightness: float = 1.0, max_grids: int = 64):
        from . import _lib
        self._lib = _lib
        _lib.load()
        self.device = torch.device(device)
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.sched = Scheduler(hbm_budget, max_inflight, batch_rays, chunk_rays, default_timeout,
                               work_done=self._work_done)
        self.grids: Dict[str, dict] = {}
        self.opt = _lib.SvxRenderOpts(background_brightness, step_size, sigma_thresh, stop_thresh, 0.0, 0, 0)
        self.use_graphs = use_graphs
        self.dtype = None
        self.desc_size = C.sizeof(_lib.SvxBatchGrid)
        self.desc_host = np.zeros((max_grids, self.desc_size), dtype=np.uint8)
        B = batch_rays
        dev = self.device
        self.lanes = {}
        for name in ("render", "train"):
            self.lanes[name] = {
                "stream": torch.cuda.Stream(device=dev),
                "origins": torch.zeros((B, 3), device=dev), "dirs": torch.zeros((B, 3), device=dev),
                "ray_grid": torch.zeros((B,), dtype=torch.int32, device=dev),
                "rgb_gt": torch.zeros((B, 3), device=dev), "rgb_out": torch.zeros((B, 3), device=dev),
                "order": torch.zeros((B,), dtype=torch.int32, device=dev),
                "n_rays": torch.zeros((1,), dtype=torch.int64, device=dev),
                "work": torch.zeros((4,), dtype=torch.int64, device=dev),
                "desc": torch.zeros((max_grids, self.desc_size), dtype=torch.uint8, device=dev),
                "desc_version": -1,      # version of desc_host last uploaded to this lane
                "graph": None,
            }
        # the train lane's records for the two-kernel fused step: each ray's per-sample colour,
        # transmittance, t and sigma, up to 1024 evaluated samples (the longest ray of a 256^3
        # grid at step 0.5 has 887; longer rays are redone by the one-kernel step)
        cache_bytes = int(_lib.load().svx_batch_record_bytes(B, 1024))
        self.lanes["train"]["colour_cache"] = torch.empty((cache_bytes // 4,), dtype=torch.float32, device=dev)
        lane_bytes = sum(t.numel() * t.element_size() for lane in self.lanes.values() for t in lane.values()
                         if isinstance(t, torch.Tensor))
        self.sched.budget -= lane_bytes
        self.slots_free = list(range(max_grids))
        # desc_host versions: any change (train steps rewrite their grid's loss scale) and changes
        # of the grids themselves (the render lane reads only those)
        self.desc_version = 0
        self.grid_version = 0
        self.with_bg = False             # some resident grid has an MSI background
        self.batches = {"render": 0, "train": 0}
        self.accum_min_rays = 1 << 15  # train steps this large accumulate into padded rows (vector atomics)
        self.lane_depth = 2          # batches a lane may have queued on the device
        # pinned staging for host->device updates (a pageable source would make the copy wait
        # for everything queued on the stream); a slot is reused once its copy has completed
        self.ring = [{"buf": torch.zeros((max_grids * self.desc_size,), dtype=torch.uint8).pin_memory(),
                      "event": None} for _ in range(16)]
        self.ring_pos = 0

    # -- grids
    def add_grid(self, grid_id: str, grid, trainable: bool = False) -> None:
        """Make a grid resident (its tables must already be on the server's device)."""
        if grid.sh_data.device != self.device:
            raise ValueError("the grid must live on the server's device")
        if grid.basis_dim != 9:
            raise ValueError("the server batches basis_dim 9 grids")
        if self.dtype is not None and grid.sh_data.dtype != self.dtype:
            raise ValueError("all grids of a server share one SH storage type")
        if not self.slots_free:
            raise AdmissionError("no grid slots left")
        self.sched.add_grid(grid_id, grid_bytes(grid, trainable))
        self.dtype = grid.sh_data.dtype
        slot = self.slots_free.pop(0)
        from . import csrc
        g = {"grid": grid, "slot": slot, "trainable": trainable, "struct": csrc._grid_struct(grid._to_cpp())}
        if trainable:
            N, Cc = grid.sh_data.shape
            g["mask"] = torch.zeros((N,), dtype=torch.bool, device=self.device)
            g["accum"] = torch.zeros((N, (Cc + 1 + 3) // 4 * 4), dtype=torch.float32, device=self.device)
            grid._get_data_grads()
            if grid.use_background:
                g["mask_bg"] = torch.zeros(grid.background_data.shape[:2], dtype=torch.bool, device=self.device)
                grid._grad_buffer(grid.background_data)
        self.grids[grid_id] = g
        self._set_desc(grid_id, 0.0)
        self.grid_version += 1
        self._update_background_flag()

    def remove_grid(self, grid_id: str) -> None:
        self.sched.remove_grid(grid_id)
        self.slots_free.append(self.grids.pop(grid_id)["slot"])
        self.grid_version += 1
        self._update_background_flag()

    def _update_background_flag(self) -> None:
        """Batches run the background kernel while some resident grid has an MSI background;
        the lanes' captured graphs are dropped when that changes."""
        flag = any(g["grid"].use_background for g in self.grids.values())
        if flag != self.with_bg:
            for lane in self.lanes.values():
                lane["graph"] = None
        self.with_bg = flag

    def _set_desc(self, grid_id: str, norm: float, use_accum: bool = False) -> None:
        _lib = self._lib
        g = self.grids[grid_id]
        d = _lib.SvxBatchGrid()
        d.grid = g["struct"]
        if g["trainable"]:
            gd, gs = g["grid"]._get_data_grads()
            d.grads = _lib.SvxGridGrads(gd.data_ptr(), gs.data_ptr(), g["mask"].data_ptr())
            if "mask_bg" in g:
                d.grads.grad_background_out = g["grid"]._grad_buffer(g["grid"].background_data).data_ptr()
                d.grads.mask_background_out = g["mask_bg"].data_ptr()
            if use_accum:
                d.accum = g["accum"].data_ptr()
                d.accum_stride = g["accum"].size(1)
        d.norm = norm
        self.desc_host[g["slot"]] = np.frombuffer(bytes(d), dtype=np.uint8)
        self.desc_version += 1

    # -- requests
    def submit(self, req, now: Optional[float] = None, timeout: Optional[float] = None) -> Ticket:
        """Queue a request; malformed requests raise ValueError here, before any launch."""
        now = time.perf_counter() if now is None else now
        if isinstance(req, RenderRequest):
            if req.grid_id not in self.grids:
                raise ValueError(f"unknown grid {req.grid_id!r}")
            if req.width <= 0 or req.height <= 0:
                raise ValueError("image size must be positive")
            c2w = torch.as_tensor(req.c2w)
            if c2w.ndim != 2 or c2w.shape[-1] != 4 or c2w.shape[0] not in (3, 4) or not c2w.is_floating_point():
                raise ValueError("c2w must be a float [3|4, 4] matrix")
            if not (req.fx > 0):
                raise ValueError("focal length must be positive")
            n = req.width * req.height
            return self.sched.new_ticket("render", req.grid_id, n, n * 9 * 4, req, now, timeout)
        if isinstance(req, TrainRequest):
            if req.grid_id not in self.grids:
                raise ValueError(f"unknown grid {req.grid_id!r}")
            if not self.grids[req.grid_id]["trainable"]:
                raise ValueError(f"grid {req.grid_id!r} was added without trainable=True")
            o, d, gt = req.origins, req.dirs, req.rgb_gt
            if not (o.ndim == 2 and o.shape[1] == 3 and d.shape == o.shape and gt.shape == o.shape):
                raise ValueError("origins, dirs and rgb_gt must be [Q, 3]")
            if not all(t.dtype == torch.float32 for t in (o, d, gt)):
                raise ValueError("train rays must be float32")
            n = o.shape[0]
            return self.sched.new_ticket("train", req.grid_id, n, n * 12 * 4, req, now, timeout)
        raise ValueError(f"unknown request type {type(req).__name__}")

    # -- execution
    def _prepare(self, t: Ticket) -> None:
        """Device buffers of an admitted request, filled on its lane's stream."""
        _lib = self._lib
        r = t.request
        lane = self.lanes[t.kind]
        with torch.cuda.stream(lane["stream"]):
            # the result lands in pinned host memory, copied from the lane's output buffer right
            # after the launch that computed it
            t.buf["host"] = torch.empty((t.n_rays, 3), dtype=torch.float32, pin_memory=True)
            if t.kind == "render":
                n = t.n_rays
                t.buf["origins"] = torch.empty((n, 3), device=self.device)
                t.buf["dirs"] = torch.empty((n, 3), device=self.device)
                m = np.ascontiguousarray(torch.as_tensor(r.c2w, dtype=torch.float32).cpu().numpy())
                c2w = torch.empty(m.shape, dtype=torch.float32, device=self.device)
                self._upload(c2w.view(-1).view(torch.uint8), m)
                t.buf["c2w"] = c2w
                fy = r.fx if r.fy is None else r.fy
                cx = r.width * 0.5 if r.cx is None else r.cx
                cy = r.height * 0.5 if r.cy is None else r.cy
                cam = _lib.SvxCamera(c2w.data_ptr(), c2w.size(0), float(r.fx), float(fy), float(cx), float(cy),
                                     int(r.width), int(r.height), -1.0, -1.0)
                _lib.call("svx_camera_rays", C.byref(cam), t.buf["origins"].data_ptr(), t.buf["dirs"].data_ptr(),
                          lane["stream"].cuda_stream)
            else:
                for k in ("origins", "dirs", "rgb_gt"):
                    t.buf[k] = getattr(r, k).to(self.device, non_blocking=True).contiguous()

    def _launch(self, name: str, n: int) -> None:
        """One batched kernel launch on the lane's current stream: replay of the lane's captured
        graph (captured on first use, when the launch itself does the work)."""
        lane = self.lanes[name]
        _lib = self._lib
        lane["n_rays"].fill_(n)
        # the descriptors are uploaded only when they changed since this lane's last upload (the
        # render lane reads only the grids' tables, not the train steps' loss scales)
        version = self.desc_version if name == "train" else self.grid_version
        if lane["desc_version"] != version:
            self._upload(lane["desc"].view(-1), self.desc_host)
            lane["desc_version"] = version
        dt = {torch.float32: _lib.SVX_F32, torch.bfloat16: _lib.SVX_BF16, torch.float16: _lib.SVX_F16}[self.dtype]
        mode = 0 if name == "render" else 1

        order = lane["order"].data_ptr() if name == "train" else None

        cache = lane.get("colour_cache")

        def call():
            _lib.call("svx_render_batch", mode, lane["desc"].data_ptr(), 9, dt, int(self.with_bg),
                      lane["origins"].data_ptr(),
                      lane["dirs"].data_ptr(), lane["ray_grid"].data_ptr(), order, lane["n_rays"].data_ptr(),
                      self.sched.batch_rays, C.byref(self.opt), lane["rgb_gt"].data_ptr(),
                      lane["rgb_out"].data_ptr(), lane["work"].data_ptr(),
                      None if cache is None else cache.data_ptr(),
                      0 if cache is None else cache.numel() * 4, torch.cuda.current_stream().cuda_stream)

        self.batches[name] += 1
        if not self.use_graphs:
            call()
            return
        if lane["graph"] is None:
            call()
            torch.cuda.current_stream().synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=lane["stream"]):
                call()
            lane["graph"] = g
            return
        lane["graph"].replay()

    def _upload(self, dst: torch.Tensor, data: np.ndarray) -> None:
        """Copy host bytes into the device tensor dst (uint8, same size) on the current stream,
        through a pinned staging slot that is reused only after its copy has completed."""
        slot = self.ring[self.ring_pos]
        self.ring_pos = (self.ring_pos + 1) % len(self.ring)
        if slot["event"] is not None:
            slot["event"].synchronize()
        raw = np.ascontiguousarray(data).view(np.uint8).reshape(-1)
        if slot["buf"].numel() < raw.size:
            slot["buf"] = torch.zeros((raw.size,), dtype=torch.uint8).pin_memory()
        view = slot["buf"][:raw.size]
        view.numpy()[:] = raw
        dst.copy_(view, non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream())
        slot["event"] = ev

    def step(self, now: Optional[float] = None) -> List[Ticket]:
        """One scheduler iteration; returns the tickets that finished in it."""
        now = time.perf_counter() if now is None else now
        finished = self.sched.expire(now)
        for t in self.sched.admit():
            self._prepare(t)
        for lane in self.lanes.values():
            lane["queued"] = [e for e in lane.get("queued", []) if not e.query()]
        chunks, trains = self.sched.plan(render_busy=len(self.lanes["render"]["queued"]) >= self.lane_depth,
                                         train_busy=len(self.lanes["train"]["queued"]) >= self.lane_depth)
        if chunks:
            self._run_render(chunks)
        if trains:
            self._run_train(trains)
        finished += self._collect()
        return finished

    def _run_render(self, chunks: List[Chunk]) -> None:
        lane = self.lanes["render"]
        st = lane["stream"]
        with torch.cuda.stream(st):
            off = 0
            for ch in chunks:
                t = ch.ticket
                sl = slice(off, off + ch.count)
                lane["origins"][sl].copy_(t.buf["origins"][ch.start:ch.start + ch.count])
                lane["dirs"][sl].copy_(t.buf["dirs"][ch.start:ch.start + ch.count])
                lane["ray_grid"][sl].fill_(self.grids[t.grid_id]["slot"])
                off += ch.count
            self._launch("render", off)
            off = 0
            for ch in chunks:
                t = ch.ticket
                t.buf["host"][ch.start:ch.start + ch.count].copy_(lane["rgb_out"][off:off + ch.count],
                                                                  non_blocking=True)
                off += ch.count
            ev = torch.cuda.Event()
            ev.record(st)
        for ch in chunks:
            ch.ticket.rays_done_event.append(ev)
        lane["queued"].append(ev)

    @staticmethod
    def _work_done(t: Ticket) -> bool:
        if t.done:
            return True
        return t.rays_launched >= t.n_rays and bool(t.rays_done_event) and all(e.query() for e in t.rays_done_event)

    def _run_train(self, trains: List[Ticket]) -> None:
        _lib = self._lib
        lane = self.lanes["train"]
        st = lane["stream"]
        with torch.cuda.stream(st):
            off = 0
            for t in trains:
                g = self.grids[t.grid_id]
                sl = slice(off, off + t.n_rays)
                lane["origins"][sl].copy_(t.buf["origins"])
                lane["dirs"][sl].copy_(t.buf["dirs"])
                lane["rgb_gt"][sl].copy_(t.buf["rgb_gt"])
                lane["ray_grid"][sl].fill_(g["slot"])
                # each train step's rays run in coherence order (outputs stay at their own index)
                rays = _lib.SvxRays(lane["origins"][sl].data_ptr(), lane["dirs"][sl].data_ptr(), t.n_rays)
                _lib.call("svx_ray_order", C.byref(g["struct"]), C.byref(rays), C.byref(self.opt),
                          off, lane["order"][sl].data_ptr(), st.cuda_stream)
                g["mask"].zero_()
                if "mask_bg" in g:
                    g["mask_bg"].zero_()
                use_accum = t.n_rays >= self.accum_min_rays
                if use_accum:
                    g["accum"].zero_()
                self._set_desc(t.grid_id, 2.0 / (3 * t.n_rays), use_accum)
                t.buf["accum"] = use_accum
                off += t.n_rays
            self._launch("train", off)
            off = 0
            for t in trains:
                g = self.grids[t.grid_id]
                grid, r = g["grid"], t.request
                t.buf["host"].copy_(lane["rgb_out"][off:off + t.n_rays], non_blocking=True)
                off += t.n_rays
                if t.buf["accum"]:
                    # padded accumulation rows -> the grid's gradients
                    gd, gs = grid._get_data_grads()
                    acc = g["accum"]
                    _lib.call("svx_add_accum", acc.data_ptr(), acc.size(1), grid.sh_data.size(1), acc.size(0),
                              gs.data_ptr(), gd.data_ptr(), st.cuda_stream)
                # the rest of the reference's training step on this grid (opt/opt.py:557-595)
                grid.sparse_grad_indexer = g["mask"]
                grid.sparse_sh_grad_indexer = g["mask"].clone()
                np.random.seed(r.tv_seed)
                grid.inplace_tv_grad(grid._grad_buffer(grid.density_data), scaling=r.tv_density,
                                     sparse_frac=r.tv_frac)
                grid.inplace_tv_color_grad(grid._grad_buffer(grid.sh_data), scaling=r.tv_sh, sparse_frac=r.tv_frac)
                if "mask_bg" in g:
                    grid.sparse_background_indexer = g["mask_bg"]
                    if r.tv_background_sigma > 0.0 or r.tv_background_color > 0.0:
                        grid.inplace_tv_background_grad(grid._grad_buffer(grid.background_data),
                                                        scaling=r.tv_background_color,
                                                        scaling_density=r.tv_background_sigma,
                                                        sparse_frac=r.tv_background_frac, contiguous=True)
                grid.optim_density_step(r.lr_density, beta=r.rms_beta)
                grid.optim_sh_step(r.lr_sh, beta=r.rms_beta)
                if "mask_bg" in g:
                    grid.optim_background_step(r.lr_sigma_bg, r.lr_color_bg, beta=r.rms_beta)
                    grid.sparse_background_indexer = None
                grid.sparse_grad_indexer = None
                grid.sparse_sh_grad_indexer = None
                # the request is complete once its grid's step is: an event of its own, so that
                # it does not wait for the optimiser steps of the batch's later grids
                ev = torch.cuda.Event()
                ev.record(st)
                t.rays_done_event.append(ev)
        lane["queued"].append(ev)

    def _collect(self) -> List[Ticket]:
        """Finish requests whose work completed: each launch copied its part of a result into the
        request's pinned host buffer on the lane's stream, so the result is there once every
        launch of the request has completed."""
        done = []
        for t in list(self.sched.active):
            if t.rays_launched < t.n_rays or not t.rays_done_event:
                continue
            if not all(e.query() for e in t.rays_done_event):
                continue
            out = t.buf["host"]
            t.result = out.view(t.request.height, t.request.width, 3) if t.kind == "render" else out
            t.buf.clear()
            t.rays_done_event.clear()
            self.sched.finish(t, time.perf_counter())
            done.append(t)
        return done

    def idle(self) -> bool:
        return self.sched.idle()

    def run_until_idle(self) -> List[Ticket]:
        out = []
        while not self.idle():
            out += self.step()
        return out


def latency_stats(tickets: List[Ticket]) -> dict:
    """Latency percentiles of the finished tickets, over all and per kind (render / train)."""
    lat = np.array([t.latency for t in tickets if t.state == "done"], dtype=np.float64)
    if lat.size == 0:
        return {"n": 0}
    out = {"n": int(lat.size), "p50_ms": float(np.percentile(lat, 50) * 1e3),
           "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
           "max_ms": float(lat.max() * 1e3)}
    for kind in ("render", "train"):
        lk = np.array([t.latency for t in tickets if t.state == "done" and t.kind == kind], dtype=np.float64)
        if lk.size:
            out[f"{kind}_p50_ms"] = float(np.percentile(lk, 50) * 1e3)
            out[f"{kind}_p99_ms"] = float(np.percentile(lk, 99) * 1e3)
    return out
