"""Host-side serving logic (svox2_gb300.serving.Scheduler), no GPU: admission by
memory budget, rejection of malformed and oversized requests, timeouts, per-grid
arrival order, and continuous batching (new requests join the next iteration
while earlier ones are still in flight)."""
import pytest

from svox2_gb300.serving import AdmissionError, RequestTimeout, Scheduler


def _sched(**kw):
    args = dict(budget_bytes=10_000, max_inflight=8, batch_rays=1000, chunk_rays=300)
    args.update(kw)
    return Scheduler(**args)


def test_grid_admission_by_budget():
    s = _sched()
    s.add_grid("a", 6000)
    with pytest.raises(AdmissionError):
        s.add_grid("b", 5000)
    s.add_grid("b", 3000)
    with pytest.raises(ValueError):
        s.add_grid("a", 1)
    s.remove_grid("b")
    s.add_grid("c", 3500)


def test_malformed_and_oversized_requests_are_rejected():
    s = _sched()
    s.add_grid("a", 6000)
    with pytest.raises(ValueError):
        s.new_ticket("render", "nope", 10, 10, None, 0.0, None)
    with pytest.raises(ValueError):
        s.new_ticket("render", "a", 0, 10, None, 0.0, None)
    with pytest.raises(ValueError):
        s.new_ticket("train", "a", 5000, 10, None, 0.0, None)      # more rays than one batch
    with pytest.raises(AdmissionError):
        s.new_ticket("render", "a", 10, 5000, None, 0.0, None)     # can never fit beside the grid
    assert s.idle()


def test_memory_gated_admission_and_timeout():
    s = _sched(max_inflight=8)
    s.add_grid("a", 6000)
    t1 = s.new_ticket("render", "a", 100, 3000, None, 0.0, None)
    t2 = s.new_ticket("render", "a", 100, 3000, None, 0.0, 0.5)
    assert s.admit() == [t1]                 # t2 would exceed the budget while t1 holds its buffers
    assert s.expire(0.4) == []
    assert s.expire(0.6) == [t2]
    assert isinstance(t2.error, RequestTimeout) and t2.state == "failed"
    s.finish(t1, 1.0)
    assert s.idle()


def test_slots_bound_inflight_requests():
    s = _sched(max_inflight=2)
    s.add_grid("a", 100)
    ts = [s.new_ticket("render", "a", 10, 10, None, 0.0, None) for _ in range(3)]
    assert s.admit() == ts[:2]
    s.finish(ts[0], 1.0)
    assert s.admit() == [ts[2]]


def test_per_grid_arrival_order():
    s = _sched()
    s.add_grid("a", 100)
    s.add_grid("b", 100)
    r1 = s.new_ticket("render", "a", 200, 10, None, 0.0, None)
    t1 = s.new_ticket("train", "a", 200, 10, None, 0.1, None)
    r2 = s.new_ticket("render", "a", 200, 10, None, 0.2, None)
    r3 = s.new_ticket("render", "b", 200, 10, None, 0.3, None)
    s.admit()
    chunks, trains = s.plan()
    assert [c.ticket for c in chunks] == [r1, r3] and trains == []   # t1 waits for r1, r2 for t1
    s.finish(r1, 1.0)
    chunks, trains = s.plan()
    assert chunks == [] and trains == [t1]
    s.finish(t1, 2.0)
    chunks, trains = s.plan()
    assert [c.ticket for c in chunks] == [r2]
    s.finish(r2, 3.0)
    s.finish(r3, 3.0)
    assert s.idle()


def test_continuous_batching_chunks_and_late_arrivals():
    s = _sched(batch_rays=1000, chunk_rays=300)
    s.add_grid("a", 100)
    s.add_grid("b", 100)
    big = s.new_ticket("render", "a", 1000, 10, None, 0.0, None)
    s.admit()
    c1, _ = s.plan()
    assert [(c.ticket, c.start, c.count) for c in c1] == [(big, 0, 300)]
    # a request arriving while the first chunk is in flight joins the next batch
    small = s.new_ticket("render", "b", 50, 10, None, 0.01, None)
    tr = s.new_ticket("train", "b", 400, 10, None, 0.02, None)
    s.admit()
    c2, trains = s.plan()
    assert [(c.ticket, c.start, c.count) for c in c2] == [(big, 300, 300), (small, 0, 50)]
    assert trains == []                      # the train step on b waits for the earlier render on b
    c3, _ = s.plan()
    assert [(c.ticket, c.start, c.count) for c in c3] == [(big, 600, 300)]
    c4, _ = s.plan()
    assert [(c.ticket, c.start, c.count) for c in c4] == [(big, 900, 100)]
    s.finish(small, 0.5)
    _, trains = s.plan()
    assert trains == [tr]
    s.finish(big, 0.6)
    s.finish(tr, 0.7)
    assert s.idle()


def test_one_train_step_per_grid_per_batch():
    s = _sched(batch_rays=1000)
    s.add_grid("a", 100)
    s.add_grid("b", 100)
    ta1 = s.new_ticket("train", "a", 300, 10, None, 0.0, None)
    ta2 = s.new_ticket("train", "a", 300, 10, None, 0.1, None)
    tb1 = s.new_ticket("train", "b", 300, 10, None, 0.2, None)
    s.admit()
    _, trains = s.plan()
    assert trains == [ta1, tb1]
    s.finish(ta1, 1.0)
    _, trains = s.plan()
    assert trains == [ta2]


def test_grid_removal_waits_for_its_requests_and_memory_returns():
    s = _sched()
    s.add_grid("a", 4000)
    base = s.used_bytes()
    t = s.new_ticket("render", "a", 100, 1500, None, 0.0, None)
    with pytest.raises(RuntimeError):
        s.remove_grid("a")                    # a request is queued on it
    assert s.admit() == [t]
    assert s.used_bytes() == base + 1500      # the admitted request holds its buffers
    s.plan()
    s.finish(t, 1.0)
    assert s.used_bytes() == base             # ... and returns them when it finishes
    s.remove_grid("a")
    assert s.used_bytes() == 0 and s.idle()


def test_default_timeout_applies_and_failed_requests_unblock_their_grid():
    s = _sched(default_timeout=0.5, max_inflight=1)
    s.add_grid("a", 100)
    r0 = s.new_ticket("render", "a", 10, 10, None, 0.0, None)
    tr = s.new_ticket("train", "a", 10, 10, None, 0.1, None)
    r1 = s.new_ticket("render", "a", 10, 10, None, 0.2, timeout=5.0)
    assert s.admit() == [r0]                  # one slot: the others wait in the queue
    expired = s.expire(0.7)                   # the train step's default 0.5 s deadline passed
    assert expired == [tr] and tr.state == "failed"
    assert r1.state == "queued"               # its own 5 s timeout still runs
    s.plan()
    s.finish(r0, 0.8)
    assert s.admit() == [r1]
    chunks, _ = s.plan()                      # the failed train step no longer orders r1
    assert [c.ticket for c in chunks] == [r1]


def test_train_step_waits_for_device_work_not_host_readback():
    done = set()
    s = _sched(work_done=lambda t: t.done or t.id in done)
    s.add_grid("a", 100)
    r = s.new_ticket("render", "a", 100, 10, None, 0.0, None)
    tr = s.new_ticket("train", "a", 100, 10, None, 0.1, None)
    s.admit()
    chunks, trains = s.plan()
    assert [c.ticket for c in chunks] == [r] and trains == []
    done.add(r.id)                            # the render's kernels finished; its colours are still
    _, trains = s.plan()                      # on their way to the host
    assert trains == [tr]


def test_grid_bytes_count_the_background_tables():
    """Admission charges a grid's MSI background: its tables, and when trainable its gradient,
    RMSprop state and mask."""
    from svox2_gb300 import SparseGrid
    from svox2_gb300.serving import grid_bytes
    plain = SparseGrid(reso=8, basis_dim=9)
    bg = SparseGrid(reso=8, basis_dim=9, background_nlayers=3, background_reso=4)
    tables = 2 * 4 * 4 * 4 + 2 * 4 * 4 * 3 * 4 * 4          # links + data [32, 3, 4] float32
    assert grid_bytes(bg, False) - grid_bytes(plain, False) == tables
    train_extra = 2 * (2 * 4 * 4 * 3 * 4 * 4) + 2 * 4 * 4 * 3  # gradient + RMSprop state + mask
    assert grid_bytes(bg, True) - grid_bytes(plain, True) == tables + train_extra
