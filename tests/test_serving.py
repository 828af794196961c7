"""Request server (continuous batching, admission by device memory).

CPU: the scheduler against a simulated executor and clock: arrival order, the memory budget
and the slot count are never exceeded, requests too large for the budget are rejected, jobs
that arrive while others run start as soon as memory frees, requests past their admission
deadline are cancelled unstarted, latency percentiles.
GPU: a mixed stream of ABO3 jobs of different sizes and frame counts, admitted under a budget
that forces queueing, gives every job the same S(Q) and E=const maps as the job run alone, bit
for bit (the executor's jobs take the reproducible in-tile order)."""
import numpy as np
import pytest

from mp_tools_gb300 import serve


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def clock(self):
        return self.t

    def sleep(self, dt):
        self.t += max(dt, 1e-4)


class FakeExecutor:
    """Each request carries .mem (bytes) and .dur (seconds on the device)."""

    def __init__(self, clk):
        self.clk = clk
        self.running = {}
        self.max_used = 0
        self.used = 0
        self.max_concurrent = 0

    def estimate(self, req):
        return req.mem

    def start(self, req):
        self.used += req.mem
        self.max_used = max(self.max_used, self.used)
        self.running[req.rid] = self.clk.t + req.dur
        self.max_concurrent = max(self.max_concurrent, len(self.running))
        return req

    def done(self, h):
        return self.clk.t >= self.running[h.rid]

    def finish(self, h):
        del self.running[h.rid]
        self.used -= h.mem
        return np.full(3, float(h.rid)), None


def _req(rid, arrival, mem, dur):
    r = serve.Request(rid, arrival, np.zeros((1, 10, 4), np.float32), [10], grid=None)
    r.mem, r.dur = mem, dur
    return r


def test_scheduler_budget_slots_and_rejection():
    clk = FakeClock()
    ex = FakeExecutor(clk)
    reqs = [_req(0, 0.00, 40, 1.0), _req(1, 0.01, 40, 1.0), _req(2, 0.02, 40, 0.5),
            _req(3, 0.03, 500, 0.1), _req(4, 0.04, 10, 0.2), _req(5, 3.0, 30, 0.1)]
    srv = serve.Server(ex, budget_bytes=100, max_active=3, clock=clk.clock, sleep=clk.sleep)
    res, st = srv.run(reqs)
    assert st["rejected_ids"] == [3]                       # larger than the whole budget
    assert sorted(res) == [0, 1, 2, 4, 5]
    assert ex.max_used <= 100 and st["peak_admitted_bytes"] <= 100
    assert ex.max_concurrent <= 3
    # 2 needs 40 more than 0 and 1 leave: it waits until one of them ends; 4 waits behind it
    assert res[2].admitted >= 1.0 - 1e-9 and res[4].admitted >= res[2].admitted
    assert st["queued"] >= 2 and st["max_queue"] >= 2
    assert res[5].admitted == pytest.approx(3.0, abs=1e-3)  # an idle server starts at once
    for r in res.values():
        assert np.all(r.sq == r.rid)
    lat = np.array([res[k].latency for k in sorted(res)])
    assert st["p50_s"] == pytest.approx(np.percentile(lat, 50))
    assert st["p99_s"] == pytest.approx(np.percentile(lat, 99))


def test_scheduler_overlaps_jobs_that_fit():
    clk = FakeClock()
    ex = FakeExecutor(clk)
    reqs = [_req(i, 0.001 * i, 10, 1.0) for i in range(4)]
    res, st = serve.Server(ex, budget_bytes=100, max_active=8, clock=clk.clock,
                           sleep=clk.sleep).run(reqs)
    assert ex.max_concurrent == 4 and st["queued"] == 0
    assert max(r.done for r in res.values()) < 1.1      # all four ran together


def test_scheduler_cancels_requests_past_their_admission_deadline():
    """A request still queued when its max_wait has passed is cancelled unstarted; one admitted
    in time runs to completion; the head of the queue leaving unblocks the requests behind."""
    clk = FakeClock()
    ex = FakeExecutor(clk)
    reqs = [_req(0, 0.00, 80, 2.0), _req(1, 0.01, 80, 0.5), _req(2, 0.02, 10, 0.5),
            _req(3, 0.03, 80, 0.5)]
    reqs[1].max_wait = 0.5            # 0 holds the memory until t = 2: 1 gives up at t = 0.51
    reqs[2].max_wait = 5.0            # behind 1 in the queue, admitted once 1 has left
    reqs[3].max_wait = 3.0            # admitted when 0 ends at t = 2
    res, st = serve.Server(ex, budget_bytes=100, max_active=4, clock=clk.clock,
                           sleep=clk.sleep).run(reqs)
    assert st["cancelled_ids"] == [1] and st["cancelled"] == 1
    assert sorted(res) == [0, 2, 3]
    assert 0.5 <= res[2].admitted < 0.6      # right after 1 left the head of the queue
    assert res[3].admitted == pytest.approx(2.0, abs=1e-3)
    assert ex.max_used <= 100


def test_scheduler_metrics_json_lines():
    """One JSON line per completed, rejected and cancelled request, then the summary."""
    import io
    import json
    clk = FakeClock()
    ex = FakeExecutor(clk)
    reqs = [_req(0, 0.0, 80, 1.0), _req(1, 0.01, 500, 0.1), _req(2, 0.02, 80, 0.1)]
    reqs[2].max_wait = 0.2
    sink = io.StringIO()
    res, st = serve.Server(ex, budget_bytes=100, max_active=4, clock=clk.clock, sleep=clk.sleep,
                           metrics=sink).run(reqs)
    lines = [json.loads(x) for x in sink.getvalue().splitlines()]
    ev = {(d["event"], d.get("rid")) for d in lines}
    assert ev == {("rejected", 1), ("cancelled", 2), ("completed", 0), ("summary", None)}
    done = next(d for d in lines if d["event"] == "completed")
    assert done["latency_s"] == pytest.approx(res[0].latency) and done["nu_points"] == 10
    summary = lines[-1]
    assert summary["event"] == "summary" and summary["completed"] == 1
    assert summary["rejected_ids"] == [1] and summary["cancelled_ids"] == [2]


@pytest.mark.gpu
def test_gpu_results_same_alone_and_in_the_mix(cuda):
    from mp_tools_gb300 import _lib
    rng = np.random.default_rng(7)
    specs = [(0.000, 4, 8, 2), (0.002, 6, 1, 2), (0.004, 5, 16, 2), (0.006, 8, 4, 2),
             (0.008, 4, 6, 3), (0.010, 6, 12, 2)]
    reqs = [serve.abo3_request(i, t, e, f, z, rng) for i, (t, e, f, z) in enumerate(specs)]
    ex = serve.GpuExecutor()
    est = [ex.estimate(r) for r in reqs]
    budget = int(2.2 * max(est))                          # forces some queueing
    mixed, st = serve.Server(ex, budget_bytes=budget, max_active=4).run(reqs)
    assert st["completed"] == len(reqs) and st["rejected"] == 0
    assert st["peak_admitted_bytes"] <= budget
    alone = {}
    for r in reqs:                                         # one job at a time
        a, _ = serve.Server(ex, budget_bytes=budget, max_active=1).run(
            [serve.Request(r.rid, 0.0, r.frames, r.counts, r.grid, r.job_kwargs)])
        alone[r.rid] = a[r.rid]
    for k in alone:
        m, a = mixed[k], alone[k]
        assert np.array_equal(m.sq, a.sq), k
        if a.sqw is None:
            assert m.sqw is None
        else:
            assert np.array_equal(m.sqw, a.sqw), k
    # and against the plain (job-at-a-time) API
    from mp_tools_gb300.sqom import SqomJob
    r = reqs[2]
    job = SqomJob(r.grid, species_counts=r.counts, n_frames=r.n_frames, **r.job_kwargs)
    try:
        job.set_option(_lib.OPT_REPRODUCIBLE, 1)
        job.set_frames(r.frames)
        job.transform()
        sq = job.sq_total()
    finally:
        job.close()
    assert np.array_equal(mixed[2].sq, sq)
    assert _lib.load().mpsq_launch_count() > 0


@pytest.mark.gpu
def test_gpu_job_larger_than_the_budget_runs_by_q_slabs(cuda):
    """A request whose whole amplitude store does not fit in the budget is admitted with the
    largest kz slab that does and runs slab by slab; its S(Q) and E=const maps equal those of
    the same job with the whole store (relative l2 1e-5)."""
    rng = np.random.default_rng(11)
    r = serve.abo3_request(0, 0.0, 8, 8, 4, rng)            # 32^3 modes, 8 frames
    ex = serve.GpuExecutor()
    full, slab4 = ex._bytes(r, 0), ex._bytes(r, 4)
    assert slab4 < full
    budget = (full + slab4) // 2
    res, st = serve.Server(ex, budget_bytes=budget, max_active=2).run([r])
    assert st["completed"] == 1 and st["rejected"] == 0
    assert 4 <= r._q_slab < r.grid.n_q[2]
    assert st["peak_admitted_bytes"] <= budget
    whole = serve.Request(1, 0.0, r.frames, r.counts, r.grid, r.job_kwargs)
    ref, st2 = serve.Server(serve.GpuExecutor(), budget_bytes=4 * full, max_active=1).run([whole])
    assert whole._q_slab == 0
    a, b = res[0], ref[1]
    assert np.linalg.norm(a.sq - b.sq) <= 1e-5 * np.linalg.norm(b.sq)
    assert np.linalg.norm(a.sqw - b.sqw) <= 1e-5 * np.linalg.norm(b.sqw)


def test_scheduler_reports_a_job_that_fails_to_start():
    """A request whose executor start() raises is reported as failed (with its error) and the
    other requests of the stream still complete; its memory is not held."""
    import io
    import json
    clk = FakeClock()
    ex = FakeExecutor(clk)
    orig = ex.start

    def start(req):
        if req.rid == 1:
            raise RuntimeError("plan creation failed")
        return orig(req)

    ex.start = start
    reqs = [_req(0, 0.0, 60, 0.5), _req(1, 0.01, 60, 0.5), _req(2, 0.02, 60, 0.5)]
    sink = io.StringIO()
    res, st = serve.Server(ex, budget_bytes=130, max_active=4, clock=clk.clock, sleep=clk.sleep,
                           metrics=sink).run(reqs)
    assert st["failed_ids"] == [1] and st["failed"] == 1
    assert sorted(res) == [0, 2]
    assert res[2].admitted < 0.1             # 1's memory was never counted
    ev = [json.loads(x) for x in sink.getvalue().splitlines()]
    assert any(d["event"] == "failed" and "plan creation" in d["error"] for d in ev)
