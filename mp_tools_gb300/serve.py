"""Request server for S(Q,omega) jobs on one GPU: continuous batching with admission by device
memory.

Requests arrive over time, each an MD trajectory (host memory) with its Q grid and weights.  A
request is admitted as soon as an execution slot is free and its device footprint
(``mpsq_job_estimate_bytes``: trajectory, fine grids, records, amplitude store) fits in what
the admitted jobs leave of the budget; requests that could never fit are rejected, the others
wait in arrival order, and a request that is still waiting when its ``max_wait`` has passed is
cancelled without being started (an admitted job always runs to completion; one whose job
cannot be created — a library limit its estimate did not foresee — is reported as failed and
the stream goes on).  Every admitted
job runs on its own CUDA stream with stream-ordered device memory, so creating and closing a
job never waits for the device, and the kernels of jobs that are in flight together overlap on
the GPU (a job that arrives while others run starts at once instead of after them).  The host loop only launches work, polls completion events and
admits the next requests.

Per job: upload of the trajectory, the NUFFT of every frame and species with the species
weights, total S(Q) and, for runs of at least 4 frames, E=const maps of the first frequency bins
(mp_sqom's sliding-window form), all copied back to pinned host memory; the job's latency is the
time from its arrival to the moment its results are on the host.  ``Server.run`` returns the
results and the stream's statistics: p50/p99 latency, throughput in nonuniform points per
second, completed / rejected / cancelled counts and the longest queue.
"""
from __future__ import annotations

import json
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .sqom import QGrid, SqomJob, TimeAxis


@dataclass
class Request:
    rid: int
    arrival: float                 # seconds after the start of the stream
    frames: object                 # (F, N, 4) float32 host array / tensor (pinned: overlapped
                                   # copy), or a FrameSource that makes the frames on the device
    counts: list                   # atoms per species (species-major order of the frames)
    grid: QGrid
    job_kwargs: dict = field(default_factory=dict)   # SqomJob arguments (precision, eps, weights)
    t_step: float = 0.01           # ps between frames (E=const maps)
    n_econst: int = 4              # E=const bins returned when the run has >= 4 frames
    max_wait: float | None = None  # seconds it may wait for admission; cancelled after that

    @property
    def n_frames(self) -> int:
        return int(self.frames.shape[0])

    @property
    def n_atoms(self) -> int:
        return int(self.frames.shape[1])

    @property
    def nu_points(self) -> int:
        return int(sum(self.counts)) * self.n_frames


@dataclass
class Result:
    rid: int
    sq: np.ndarray
    sqw: np.ndarray | None        # (n_bins, n_Q) E=const maps, or None
    arrival: float
    admitted: float
    done: float

    @property
    def latency(self) -> float:
        return self.done - self.arrival


class FrameSource:
    """A trajectory made on the device when its job starts (synthetic clients whose requests
    are too large to hold in host memory while they wait): make(stream) returns the (F, N, 4)
    float32 device tensor; shape gives its size for admission."""

    def __init__(self, shape, make):
        self.shape = tuple(shape)
        self.make = make


class GpuExecutor:
    """Runs a request as a stream-ordered SqomJob on its own stream.  A request whose whole
    amplitude store would not fit in the budget runs slab by slab along kz (q_slab: the largest
    slab that fits), recomputing the transform of every frame per slab.  Jobs run with the
    reproducible in-tile order (a request's results do not depend on what else shares the GPU)
    unless `reproducible` is set False."""

    budget = None                  # set by the server: the device memory admissions share
    pin_limit = 256 << 20          # map bytes up to which results go to pinned host buffers
    reproducible = True

    def _describe(self, req, q_slab):
        return SqomJob.describe(req.grid, species_counts=req.counts, n_frames=req.n_frames,
                                n_atoms_frame=req.n_atoms, stream_ordered=True, q_slab=q_slab,
                                **req.job_kwargs)

    def _bytes(self, req, q_slab):
        n_bins = self._n_bins(req)
        plane = req.grid.n_q[0] * req.grid.n_q[1]
        kept = plane * (min(q_slab, req.grid.n_q[2]) if q_slab else req.grid.n_q[2])
        full = req.grid.n_modes * (1 + n_bins) * 4
        out = kept * (1 + n_bins) * 4 if full <= self.pin_limit else full
        made = 16 * req.n_frames * req.n_atoms if isinstance(req.frames, FrameSource) else 0
        return SqomJob.estimate_bytes(self._describe(req, q_slab)) + out + made

    @staticmethod
    def _n_bins(req):
        if req.n_frames < 4:
            return 0
        return min(req.n_econst, TimeAxis(nfile=req.n_frames, t_step=req.t_step).n_freq_max)

    def plan(self, req: Request):
        """(bytes, q_slab): the whole store when it fits in the budget, else the largest kz slab
        that does (q_slab 0 = whole store); the whole-store bytes when no slab fits."""
        full = self._bytes(req, 0)
        if self.budget is None or full <= self.budget or req.grid.ndim != 3:
            return full, 0
        lo, hi = 1, req.grid.n_q[2]
        if self._bytes(req, lo) > self.budget:
            return full, 0
        while lo < hi:                              # largest slab within the budget
            mid = (lo + hi + 1) // 2
            if self._bytes(req, mid) <= self.budget:
                lo = mid
            else:
                hi = mid - 1
        return self._bytes(req, lo), lo

    def estimate(self, req: Request) -> int:
        b, q_slab = self.plan(req)
        req._q_slab = q_slab
        return b

    def start(self, req: Request):
        import torch
        stream = torch.cuda.Stream()
        q_slab = getattr(req, "_q_slab", 0)
        job = SqomJob(req.grid, species_counts=req.counts, n_frames=req.n_frames,
                      n_atoms_frame=req.n_atoms, stream=stream.cuda_stream,
                      stream_ordered=True, q_slab=q_slab, **req.job_kwargs)
        job.set_option(_lib.OPT_REPRODUCIBLE, int(self.reproducible))
        nq = req.grid.n_modes
        F = req.n_frames
        n_bins = self._n_bins(req)
        ta = TimeAxis(nfile=F, t_step=req.t_step) if n_bins else None
        # small maps: slab-sized device buffers copied to pinned host memory after each slab;
        # large maps (pinning them would take longer than the job): full-size device maps, copied
        # to host memory when the job has finished
        pinned = nq * (1 + n_bins) * 4 <= self.pin_limit
        kept = job.store_modes if pinned else nq
        with torch.cuda.stream(stream):
            dev_sq = torch.empty(kept, dtype=torch.float32, device="cuda")
            dev_sqw = torch.empty((n_bins, kept), dtype=torch.float32, device="cuda") if n_bins else None
        host_sq = torch.empty(nq, dtype=torch.float32, pin_memory=True) if pinned else None
        host_sqw = (torch.empty((n_bins, nq), dtype=torch.float32, pin_memory=True)
                    if pinned and n_bins else None)
        frames = req.frames
        made = isinstance(frames, FrameSource)
        if made:
            with torch.cuda.stream(stream):
                frames = frames.make(stream)
        job.set_frames(frames)                     # pinned host -> device on the job's stream
        if made:
            frames = None        # the copy is queued on the stream that owns the tensor's memory
        for z0, planes, q0 in job.slabs():
            if q_slab:
                job.set_q_slab(z0)
            n = req.grid.n_q[0] * req.grid.n_q[1] * planes
            o = 0 if pinned else q0
            job.transform()
            job.sq_total(out=dev_sq[o:o + n])
            for b in range(n_bins):
                job.sqw_econst(ta, b + 1, out=dev_sqw[b, o:o + n])
            if pinned:
                with torch.cuda.stream(stream):    # after the slab's maps, before the next slab's
                    host_sq[q0:q0 + n].copy_(dev_sq[:n], non_blocking=True)
                    for b in range(n_bins):        # contiguous rows
                        host_sqw[b, q0:q0 + n].copy_(dev_sqw[b, :n], non_blocking=True)
        done = torch.cuda.Event()
        done.record(stream)
        return {"job": job, "stream": stream, "done": done, "sq": host_sq, "sqw": host_sqw,
                "dev": (dev_sq, dev_sqw), "frames": frames, "q_slab": q_slab}

    def done(self, h) -> bool:
        return h["done"].query()

    def finish(self, h):
        job = h["job"]
        job.sync()                                 # completed already: checks the error flag
        job.close()                                # stream-ordered frees, no device wait
        if h["sq"] is None:                        # large maps: copied now, from the device
            dev_sq, dev_sqw = h["dev"]
            return dev_sq.cpu().numpy(), dev_sqw.cpu().numpy() if dev_sqw is not None else None
        sq = h["sq"].numpy().copy()
        sqw = h["sqw"].numpy().copy() if h["sqw"] is not None else None
        return sq, sqw


class Server:
    """Admission by memory and execution slots, first come first served; see the module
    docstring.  `executor` provides estimate(req) -> bytes, start(req) -> handle,
    done(handle) -> bool and finish(handle) -> (sq, sqw).  `metrics`, a writable text file,
    receives one JSON line per completed, rejected or cancelled request and a summary line
    with the statistics that run() returns."""

    def __init__(self, executor=None, budget_bytes: int | None = None, max_active: int = 8,
                 poll_s: float = 2e-4, clock=time.perf_counter, sleep=time.sleep,
                 metrics=None, keep_results: bool = True):
        self.ex = executor if executor is not None else GpuExecutor()
        if budget_bytes is None:
            import torch
            free, total = torch.cuda.mem_get_info()
            budget_bytes = int(0.8 * free)
        self.budget = int(budget_bytes)
        if hasattr(self.ex, "budget"):
            self.ex.budget = self.budget
        self.max_active = int(max_active)
        self.poll_s = poll_s
        self.clock = clock
        self.sleep = sleep
        self.metrics = metrics         # file-like: one JSON line per request event + a summary
        self.keep_results = keep_results   # False: maps are dropped once delivered (statistics only)

    def _emit(self, record: dict):
        if self.metrics is not None:
            self.metrics.write(json.dumps(record) + "\n")

    def run(self, requests):
        pending = deque(sorted(requests, key=lambda r: (r.arrival, r.rid)))
        queue: deque = deque()
        active = []                # (req, handle, bytes, admitted)
        results: dict[int, Result] = {}
        rejected, cancelled, failed, waited = [], [], [], set()
        used = peak = 0
        max_queue = 0
        t0 = self.clock()
        first = pending[0].arrival if pending else 0.0
        while pending or queue or active:
            now = self.clock() - t0
            while pending and pending[0].arrival <= now:
                r = pending.popleft()
                b = self.ex.estimate(r)
                if b > self.budget:
                    rejected.append(r.rid)
                    self._emit({"event": "rejected", "rid": r.rid, "t_s": now, "bytes": b,
                                "budget_bytes": self.budget})
                else:
                    queue.append((r, b))
            # completions first: they free memory and slots
            still = []
            for r, h, b, adm in active:
                if self.ex.done(h):
                    sq, sqw = self.ex.finish(h)
                    t = self.clock() - t0
                    if not self.keep_results:
                        sq = sqw = None
                    results[r.rid] = Result(r.rid, sq, sqw, r.arrival, adm, t)
                    self._emit({"event": "completed", "rid": r.rid, "arrival_s": r.arrival,
                                "admitted_s": adm, "done_s": t, "latency_s": t - r.arrival,
                                "nu_points": r.nu_points, "bytes": b,
                                "nu_pts_per_s": r.nu_points / max(t - adm, 1e-12)})
                    used -= b
                else:
                    still.append((r, h, b, adm))
            active = still
            # requests whose admission deadline has passed leave the queue unstarted
            if any(r.max_wait is not None for r, _ in queue):
                keep = deque()
                for r, b in queue:
                    if r.max_wait is not None and now > r.arrival + r.max_wait:
                        cancelled.append(r.rid)
                        self._emit({"event": "cancelled", "rid": r.rid, "t_s": now,
                                    "waited_s": now - r.arrival})
                    else:
                        keep.append((r, b))
                queue = keep
            # admissions in arrival order (the head of the queue blocks the rest)
            while queue and len(active) < self.max_active and used + queue[0][1] <= self.budget:
                r, b = queue.popleft()
                adm = self.clock() - t0
                try:
                    h = self.ex.start(r)
                except Exception as e:   # e.g. a library limit the estimate did not foresee
                    failed.append(r.rid)
                    self._emit({"event": "failed", "rid": r.rid, "t_s": adm, "error": str(e)})
                    continue
                used += b
                peak = max(peak, used)
                active.append((r, h, b, adm))
            for r, _ in queue:            # could not start on arrival: waited for memory/slot
                waited.add(r.rid)
            max_queue = max(max_queue, len(queue))
            if not queue and not active and pending:
                self.sleep(max(0.0, min(pending[0].arrival - (self.clock() - t0), 0.05)))
            elif active or queue:
                self.sleep(self.poll_s)
        wall = (self.clock() - t0) - first
        lat = np.array([results[k].latency for k in sorted(results)])
        pts = sum(r.nu_points for r in requests if r.rid in results)
        stats = {
            "completed": len(results), "rejected": len(rejected), "rejected_ids": rejected,
            "cancelled": len(cancelled), "cancelled_ids": cancelled,
            "failed": len(failed), "failed_ids": failed,
            "queued": len(waited), "max_queue": max_queue, "budget_bytes": self.budget,
            "peak_admitted_bytes": peak, "max_active": self.max_active,
            "p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
            "mean_s": float(lat.mean()) if len(lat) else None,
            "wall_s": wall, "nu_pts_per_s": pts / wall if wall > 0 else None,
        }
        self._emit(dict(stats, event="summary"))
        return results, stats


# ------------------------------------------------------------------ synthetic request stream
ABO3_B = [0.507, 0.716, 0.5803, 0.5803, 0.5803]   # neutron b_coh (10^-12 cm): A, B, O, O, O


def abo3_request(rid, arrival, edge, n_frames, zones, rng, precision=_lib.FP32, eps=1e-5,
                 a=4.19, sigma=(0.05, 0.08), pinned=True):
    """One ABO3 supercell job: edge^3 cells (5 edge^3 atoms), n_frames frames of independent
    Gaussian displacements (sigma A/B and O in Angstrom) around the ideal sites, a Q volume of
    `zones` Brillouin zones per axis, neutron weights."""
    from . import synth
    cells, _ = synth.abo3_cells(edge)
    nc = len(cells)
    base = np.concatenate([cells + synth.ABO3_BASIS[s] for s in range(5)]).astype(np.float32)
    sig = np.repeat(np.array([sigma[0], sigma[0], sigma[1], sigma[1], sigma[1]]) / a, nc)
    fr = np.zeros((n_frames, 5 * nc, 4), np.float32)
    fr[:, :, :3] = base[None] + (rng.standard_normal((n_frames, 5 * nc, 3)) * sig[None, :, None])
    if pinned:
        import torch
        t = torch.from_numpy(fr).pin_memory()
    else:
        t = fr
    grid = QGrid(_lib.CELL, (edge,) * 3, n_bz=zones, a_par=(a,) * 3, ndim=3)
    kw = dict(precision=precision, eps=eps, weight_mode=_lib.WEIGHT_NEUTRON, b_coh=ABO3_B)
    return Request(rid, float(arrival), t, [nc] * 5, grid, kw)


def abo3_request_device(rid, arrival, edge, n_frames, zones, seed, precision=_lib.FP32, eps=1e-5,
                        a=4.19, dt_ps=0.01):
    """One ABO3 supercell job whose frames are made on the device when it starts: edge^3 cells,
    ideal sites displaced by a superposition of 48 seeded plane waves sampled every dt_ps (the
    inelastic benchmark's trajectories), a Q volume of `zones` Brillouin zones per axis, neutron
    weights.  For request streams whose trajectories are too large to hold in host memory."""
    nc = edge ** 3

    def make(stream):
        from . import synth
        fr, _, _ = synth.abo3_planewave_frames(edge, n_frames, dt_ps, a,
                                               np.random.default_rng(seed), device="cuda")
        return fr

    grid = QGrid(_lib.CELL, (edge,) * 3, n_bz=zones, a_par=(a,) * 3, ndim=3)
    kw = dict(precision=precision, eps=eps, weight_mode=_lib.WEIGHT_NEUTRON, b_coh=ABO3_B)
    return Request(rid, float(arrival), FrameSource((n_frames, 5 * nc, 4), make), [nc] * 5, grid,
                   kw, t_step=dt_ps)


def poisson_stream(n_jobs, rate_hz, seed, edge=(16, 100), frames=(1, 256), zones=(4, 8),
                   precision=_lib.FP32, eps=1e-5, pinned=True, device_frames=False):
    """The serving stream: n_jobs ABO3 requests with Poisson arrivals at rate_hz, edge, frame
    count and zones uniform in the given inclusive ranges (seeded).  device_frames: plane-wave
    trajectories made on the device at admission instead of Gaussian ones in host memory."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n_jobs):
        t += rng.exponential(1.0 / rate_hz)
        e = int(rng.integers(edge[0], edge[1] + 1))
        f = int(rng.integers(frames[0], frames[1] + 1))
        z = int(rng.integers(zones[0], zones[1] + 1))
        if device_frames:
            out.append(abo3_request_device(i, t, e, f, z, seed * 1000 + i, precision=precision,
                                           eps=eps))
        else:
            out.append(abo3_request(i, t, e, f, z, rng, precision=precision, eps=eps,
                                    pinned=pinned))
    return out
