"""The serving loop on the GPU: a mixed stream of render and train-step requests on
several resident BF16 grids runs through RenderServer (continuous batching, CUDA
graph replays, two overlapping lanes) and every result is compared with a serial
replay of the same requests in arrival order through the plain grid API.

Tolerance: renders of grids no train step touched are bit-identical; results that
depend on a train step differ only by the order of atomic additions in the
gradients, held to 1e-3 absolute (learning rates of 1e-2 / 1e-3 bound what a
rounding-level change of a gradient can do to the next RMSprop step)."""
import numpy as np
import pytest
import torch

from svox2_gb300 import Camera, Rays, SparseGrid
from svox2_gb300 import synthetic as S
from svox2_gb300.serving import AdmissionError, RenderRequest, RenderServer, TrainRequest, latency_stats

pytestmark = pytest.mark.gpu


def _grid(g):
    grid = SparseGrid.from_tables(g.links.cuda(), g.density.cuda(), g.sh.cuda().to(torch.bfloat16))
    grid.opt.sigma_thresh, grid.opt.stop_thresh = 1e-8, 1e-7
    return grid


def _requests(n, grid_ids, trainable, seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        gid = grid_ids[int(rng.integers(len(grid_ids)))]
        if gid in trainable and rng.random() < 0.4:
            q = int(rng.integers(256, 4096))
            o, d, gt = S.make_rays(q, seed=1000 + i)
            reqs.append(TrainRequest(gid, o, d, gt, lr_density=1e-2, lr_sh=1e-3, tv_seed=i))
        else:
            w, h = int(rng.integers(8, 96)), int(rng.integers(8, 96))
            v = rng.normal(size=3)
            eye = 4.0 * v / np.linalg.norm(v)
            reqs.append(RenderRequest(gid, S.look_at_c2w(tuple(eye)), w, h, fx=1.3 * max(w, h)))
    return reqs


def test_serving_matches_serial_replay():
    spec = {"g0": (32, 0.3), "g1": (40, 0.2), "g2": (24, 0.4)}
    data = {k: S.make_grid(r, occupancy=o, seed=70 + i) for i, (k, (r, o)) in enumerate(spec.items())}
    trainable = {"g0", "g1"}
    server = RenderServer(hbm_budget=8e9, batch_rays=16384, chunk_rays=2048, use_graphs=True)
    live = {k: _grid(g) for k, g in data.items()}
    for k, grid in live.items():
        server.add_grid(k, grid, trainable=k in trainable)
    reqs = _requests(40, list(spec), trainable, seed=5)
    tickets = [server.submit(r) for r in reqs]
    server.run_until_idle()
    assert all(t.state == "done" for t in tickets)
    n_chunks = sum(-(-t.n_rays // 2048) for t in tickets if t.kind == "render")
    assert server.batches["render"] < n_chunks          # several requests shared launches

    # serial replay through the plain API, in arrival order, from the same initial grids
    ref = {k: _grid(g) for k, g in data.items()}
    touched = set()
    for r, t in zip(reqs, tickets):
        grid = ref[r.grid_id]
        if isinstance(r, RenderRequest):
            with torch.no_grad():
                img = grid.volume_render_image(Camera(r.c2w.cuda(), fx=r.fx, width=r.width, height=r.height)).cpu()
            if r.grid_id in touched:
                assert float((img - t.result).abs().max()) <= 1e-3
            else:
                assert torch.equal(img, t.result), "render differs from the same render alone"
        else:
            rgb = grid.volume_render_fused(Rays(r.origins.cuda(), r.dirs.cuda()), r.rgb_gt.cuda())
            np.random.seed(r.tv_seed)
            grid.inplace_tv_grad(grid._grad_buffer(grid.density_data), scaling=r.tv_density, sparse_frac=r.tv_frac)
            grid.inplace_tv_color_grad(grid._grad_buffer(grid.sh_data), scaling=r.tv_sh, sparse_frac=r.tv_frac)
            grid.optim_density_step(r.lr_density, beta=r.rms_beta)
            grid.optim_sh_step(r.lr_sh, beta=r.rms_beta)
            rgb = rgb.cpu()
            if r.grid_id in touched:
                assert float((rgb - t.result).abs().max()) <= 1e-3
            else:
                assert torch.equal(rgb, t.result)
            touched.add(r.grid_id)
    for k in trainable:
        assert float((ref[k].density_data.detach() - live[k].density_data.detach()).abs().max()) <= 1e-3
    print("latency", latency_stats(tickets), "batches", server.batches)


def test_admission_rejects_over_budget_grid():
    server = RenderServer(hbm_budget=16e6, batch_rays=4096, chunk_rays=1024)
    g = S.make_grid(48, seed=80)
    with pytest.raises(AdmissionError):
        server.add_grid("big", _grid(g), trainable=True)
    with pytest.raises(ValueError):
        server.submit(RenderRequest("missing", torch.eye(4), 8, 8, fx=10.0))


def _bg_grid(g, seed):
    grid = _grid(g)
    gen = torch.Generator().manual_seed(seed)
    reso, nl = 12, 6
    grid.background_nlayers, grid.background_reso = nl, reso
    grid.background_links = torch.arange(2 * reso * reso, dtype=torch.int32, device="cuda").view(2 * reso, reso)
    bd = torch.randn((2 * reso * reso, nl, 4), generator=gen) * 0.5
    bd[..., 3] = torch.rand((2 * reso * reso, nl), generator=gen) * 2.0
    grid.background_data = torch.nn.Parameter(bd.cuda())
    return grid


def test_serving_with_background_matches_serial_replay():
    """A resident grid with an MSI background next to one without: the batch launches render
    and train both, and every result equals the plain API's (background TV and optimiser step
    included in the train step)."""
    spec = {"b0": (32, 0.3), "g1": (24, 0.4)}
    data = {k: S.make_grid(r, occupancy=o, seed=90 + i) for i, (k, (r, o)) in enumerate(spec.items())}
    trainable = {"b0", "g1"}

    def make(k):
        return _bg_grid(data[k], 7) if k == "b0" else _grid(data[k])

    server = RenderServer(hbm_budget=8e9, batch_rays=16384, chunk_rays=2048, use_graphs=True)
    live = {k: make(k) for k in spec}
    for k, grid in live.items():
        server.add_grid(k, grid, trainable=k in trainable)
    assert server.with_bg
    reqs = _requests(24, list(spec), trainable, seed=9)
    tickets = [server.submit(r) for r in reqs]
    server.run_until_idle()
    assert all(t.state == "done" for t in tickets)

    ref = {k: make(k) for k in spec}
    touched = set()
    for r, t in zip(reqs, tickets):
        grid = ref[r.grid_id]
        if isinstance(r, RenderRequest):
            with torch.no_grad():
                img = grid.volume_render_image(Camera(r.c2w.cuda(), fx=r.fx, width=r.width, height=r.height)).cpu()
            if r.grid_id in touched:
                assert float((img - t.result).abs().max()) <= 1e-3
            else:
                assert torch.equal(img, t.result), "render differs from the same render alone"
        else:
            rgb = grid.volume_render_fused(Rays(r.origins.cuda(), r.dirs.cuda()), r.rgb_gt.cuda())
            np.random.seed(r.tv_seed)
            grid.inplace_tv_grad(grid._grad_buffer(grid.density_data), scaling=r.tv_density, sparse_frac=r.tv_frac)
            grid.inplace_tv_color_grad(grid._grad_buffer(grid.sh_data), scaling=r.tv_sh, sparse_frac=r.tv_frac)
            if grid.use_background:
                grid.inplace_tv_background_grad(grid._grad_buffer(grid.background_data),
                                                scaling=r.tv_background_color, scaling_density=r.tv_background_sigma,
                                                sparse_frac=r.tv_background_frac, contiguous=True)
            grid.optim_density_step(r.lr_density, beta=r.rms_beta)
            grid.optim_sh_step(r.lr_sh, beta=r.rms_beta)
            if grid.use_background:
                grid.optim_background_step(r.lr_sigma_bg, r.lr_color_bg, beta=r.rms_beta)
            rgb = rgb.cpu()
            if r.grid_id in touched:
                assert float((rgb - t.result).abs().max()) <= 1e-3
            else:
                assert torch.equal(rgb, t.result)
            touched.add(r.grid_id)
    assert "b0" in touched
    d = float((ref["b0"].background_data.detach() - live["b0"].background_data.detach()).abs().max())
    assert d <= 1e-3, d
    assert float((ref["b0"].background_data.detach() - _bg_grid(data["b0"], 7).background_data.detach()).abs().max()) > 0
    server.remove_grid("b0")
    assert not server.with_bg
