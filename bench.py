"""Benchmark of the S(Q,omega) hot path on the batched amorphous-alloy workload.

Workload (one "step" = one whole job): a cubic box of 10^6 atoms (92% Al, 8% U) at 0.06 A^-3,
hard-sphere random sequential addition (d_min 2.2 A), 512 frames of Gaussian random walk
(sigma 0.1 A, periodic), per frame and species a 3D type-1 NUFFT onto 192^3 Q modes (Q-range
4.72 A^-1) in FP32 split precision (eps 1e-6), X-ray Cromer-Mann weights, then the whole-run
Gaussian window (FWHM 256 frames) + 512-point transform along time for every Q, |F|^2 into
257 non-negative frequency bins, and the total S(Q).

Arms
  default            : this library on the GPU (value = inputs resident in HBM; e2e = pinned
                       host trajectory in, S(Q,omega) + S(Q) maps back to pinned host memory)
  --impl reference   : the CPU restatement of the reference path (ES-kernel NUFFT + mp_sqom
                       loops, FP64, all host cores) on a bounded sample of frames

Metric: nonuniform points per second (atoms x species transforms x frames / wall time).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "NU pts/s S(Q,w) FP32 batched (amorphous Al92U8, 1e6 atoms, 512 frames, 192^3 Q)"
UNIT = "NU pts/s"
N_ATOMS, RHO, FRAC_U, DMIN = 1_000_000, 0.06, 0.08, 2.2
FRAMES, SIGMA, T_STEP = 512, 0.1, 0.01
Q_RANGE, EPS = 4.72, 1e-6
SEED = 20261205


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.rows = []
        self.proc = None
        self.gpu = gpu_index
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self._t:
            self._t.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(n)
        load = [s for s in sm if mx and s > 0.5 * mx] or sm
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ----------------------------------------------------------------------------- workload
SPREAD_KERNEL = "spread3_pair_mma_kernel<7>"
SPREAD_PROFILE = ROOT / "profiles" / "spread3_pair_mma_w7_alu1e6_192.txt"


def profiled_traffic():
    """DRAM bytes (read + write) per launch of the spread kernel, from the committed summary
    of an ncu capture of this workload (line 'traffic_bytes_per_launch: N')."""
    try:
        for line in SPREAD_PROFILE.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch:"):
                return int(line.split(":")[1]), SPREAD_PROFILE.name
    except OSError:
        pass
    return None, None


def make_workload(device="cuda"):
    from mp_tools_gb300 import synth
    t0 = time.time()
    pos0, counts, box = synth.amorphous_alloy(N_ATOMS, RHO, FRAC_U, DMIN, seed=SEED)
    log(f"[bench] hard-sphere box {box:.2f} A, {N_ATOMS} atoms in {time.time() - t0:.1f}s")
    frames = None
    if device is not None:
        frames = synth.random_walk_frames(pos0, FRAMES, SIGMA, box, SEED + 1, device=device)
    return pos0, counts, box, frames


def host_buffer(shape):
    """A float32 host tensor for the e2e leg: pinned (DMA copies that overlap the transform),
    or pageable when the host refuses to pin that much (many replicas on one node); returns
    (tensor, pinned)."""
    import torch
    try:
        return torch.empty(shape, dtype=torch.float32, pin_memory=True), True
    except RuntimeError as e:
        log(f"[bench] pinning {shape} refused ({e}); pageable host memory")
        return torch.empty(shape, dtype=torch.float32), False


def max_over_ranks(ms: float, dist, device) -> float:
    """Slowest rank's step time (the job is as fast as its slowest replica); the value a single
    process reports when dist is None."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world: int, pts_per_rank_step: float, ms: float) -> float:
    """Weak scaling: every rank processes its own replica, so the job rate is world times the
    per-replica work over the slowest rank's time."""
    return world * pts_per_rank_step / (ms / 1e3)


def make_grid(box):
    from mp_tools_gb300 import _lib
    from mp_tools_gb300.sqom import QGrid
    return QGrid(_lib.BULK, (1, 1, 1), n_bz=Q_RANGE, a_par=(box,) * 3, ndim=3)


def job_kwargs():
    from mp_tools_gb300 import _lib, synth
    return dict(weight_mode=_lib.WEIGHT_XRAY, xff=[synth.XFF["Al"], synth.XFF["U"]],
                ff_convention=_lib.FF_STANDARD, eps=EPS)


# ------------------------------------------------------------------------ CPU baseline
def cpu_port_frames(pos0, counts, box, grid, n_frames, rng_seed=SEED + 2):
    """Times the oracle's CPU port (ES NUFFT FP64 per species + weighting) on n_frames
    frames of the same random walk; returns (seconds, points, threads)."""
    import oracle
    from oracle import sqom_ref
    from mp_tools_gb300 import synth
    rng = np.random.default_rng(rng_seed)
    p = pos0[:, :3].astype(np.float32).copy()
    half = box / 2
    off = np.concatenate([[0], np.cumsum(counts)])
    origin, steps, _ = grid.qphys()
    k = [np.arange(n) - n // 2 for n in grid.n_q]
    kappa = 1.0 / (16 * np.pi ** 2)
    qx = origin[0] + k[0] * steps[0][0]
    qy = origin[1] + k[1] * steps[1][1]
    qz = origin[2] + k[2] * steps[2][2]
    q2 = (qz[:, None, None] ** 2 + qy[None, :, None] ** 2 + qx[None, None, :] ** 2)
    weights = [sqom_ref.xray_ff(synth.XFF[s], kappa * q2) for s in ("Al", "U")]
    weights = [np.ascontiguousarray(wt.ravel(), dtype=np.float64) for wt in weights]
    cs = np.empty(grid.n_modes, np.complex128)
    s_q = np.zeros(grid.n_modes, np.float64)
    axes = [grid.axis[a].astype(np.float64) * float(grid.tpe[a]) for a in range(3)]
    total_pts, elapsed = 0, 0.0
    for t in range(n_frames):
        if t > 0:
            p = p + rng.normal(0, SIGMA, p.shape).astype(np.float32)
            p = (np.remainder(p + half, box) - half).astype(np.float32)
        t0 = time.perf_counter()
        for s in range(len(counts)):
            r = p[off[s]:off[s + 1]].astype(np.float64)
            coords = [r @ axes[a] for a in range(3)]
            A = oracle.es_nufft(coords, np.ones(len(r)), -1, EPS, grid.n_q)
            oracle.weight_accumulate(cs, weights[s], A, first=(s == 0))
        oracle.abs2_accumulate(s_q, cs)   # the |F|^2 accumulation of the frame
        elapsed += time.perf_counter() - t0
        total_pts += int(off[-1])
    return elapsed, total_pts, oracle.num_threads()


def run_reference(args):
    rank = env_int("RANK", 0)
    if rank != 0:
        return
    pos0, counts, box, _ = make_workload(device=None)
    grid = make_grid(box)
    per_step = 1
    cpu_port_frames(pos0, counts, box, grid, 1)  # import/FFT-plan warm-up outside the timing
    times = []
    for i in range(args.warmup + args.steps):
        el, pts, thr = cpu_port_frames(pos0, counts, box, grid, per_step, rng_seed=SEED + 10 + i)
        if i >= args.warmup:
            times.append((el, pts, thr))
    el = sum(t[0] for t in times)
    pts = sum(t[1] for t in times)
    value = pts / el
    sample = (f"{per_step} frame(s) per step of the {FRAMES}-frame job (2 species x 1e6 atoms, "
              f"192^3 modes, FP64 ES NUFFT eps {EPS} + weights)")
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic", "config": config_dict(),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": times[0][2], "kind": "port",
                            "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def config_dict():
    return {"workload": "batched amorphous Al92U8: 1e6 atoms, 512 frames, 192^3 Q modes, "
                        "X-ray Cromer-Mann weights, Gaussian window FWHM 256 frames",
            "atoms": N_ATOMS, "frames": FRAMES, "species": 2, "modes": [192, 192, 192],
            "eps": EPS, "precision": "fp32 split (FP64-exact phase reduction)",
            "time_transform": "whole-run Gaussian window, 512-point DFT per Q, 257 bins + total S(Q)",
            "l2": "inputs larger than L2 (8.2 GB trajectory, 29 GB amplitude store)",
            "parallelism": "single GPU"}


# ------------------------------------------------------------------------------ GPU arm
def accuracy_sample(job, frames_dev, counts, grid, n_q=48, n_t=3):
    """Relative error of the weighted amplitudes and |F|^2 vs the FP64 direct-sum oracle on
    n_q random Q modes x n_t frames (all atoms)."""
    import oracle
    from oracle import sqom_ref
    from mp_tools_gb300 import synth
    rng = np.random.default_rng(7)
    nq = grid.n_modes
    qs = rng.choice(nq, n_q, replace=False)
    ts = np.linspace(0, FRAMES - 1, n_t).astype(int)
    cs = job.amplitudes()
    off = np.concatenate([[0], np.cumsum(counts)])
    origin, steps, extra = grid.qphys()
    m0, m1, m2 = grid.n_q
    kq = np.stack([qs % m0 - m0 // 2, (qs // m0) % m1 - m1 // 2, qs // (m0 * m1) - m2 // 2], 1)
    Qv = origin[None] + kq[:, :1] * steps[0] + kq[:, 1:2] * steps[1] + kq[:, 2:3] * steps[2]
    s2 = ((Qv ** 2).sum(1) + extra) / (16 * np.pi ** 2)
    w = [sqom_ref.xray_ff(synth.XFF[s], s2) for s in ("Al", "U")]
    got, ref = [], []
    for t in ts:
        r_all = frames_dev[t, :, :3].double().cpu().numpy()
        acc = np.zeros(n_q, np.complex128)
        for s in range(2):
            r = r_all[off[s]:off[s + 1]]
            x = [r @ grid.axis[a].astype(np.float64) * float(grid.tpe[a]) for a in range(3)]
            acc += w[s] * oracle.dirft_modes(x[0], x[1], x[2], np.ones(len(r)), -1, kq)
        ref.append(acc)
        got.append(cs[t, qs])
    out = error_metrics(np.array(got), np.array(ref))
    out["sample"] = f"{n_q} random Q x {n_t} frames, FP64 direct sum over all 1e6 atoms"
    return out


def error_metrics(got, ref):
    """Relative l2 errors of amplitudes and of |F|^2, and the largest relative |F|^2 error over
    the samples whose oracle |F|^2 exceeds 1e-3 of the sample maximum."""
    got = np.asarray(got, np.complex128).ravel()
    ref = np.asarray(ref, np.complex128).ravel()
    s_got, s_ref = np.abs(got) ** 2, np.abs(ref) ** 2
    strong = s_ref > 1e-3 * s_ref.max()
    return {"rel_l2_amplitude": float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
            "rel_l2_S": float(np.linalg.norm(s_got - s_ref) / np.linalg.norm(s_ref)),
            "max_rel_S": (float(np.max(np.abs(s_got[strong] - s_ref[strong]) / s_ref[strong]))
                          if strong.any() else None)}


def run_gpu(args):
    import torch

    from mp_tools_gb300 import _lib
    from mp_tools_gb300.sqom import SqomJob

    rank = env_int("RANK", 0)
    world = env_int("WORLD_SIZE", 1)
    local = env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    L = _lib.load()
    pos0, counts, box, frames = make_workload(device="cuda")
    grid = make_grid(box)
    stream = torch.cuda.current_stream()
    job = SqomJob(grid, species_counts=counts, n_frames=FRAMES, precision=_lib.FP32,
                  stream=stream.cuda_stream, **job_kwargs())
    job.set_frames(frames)
    n_freq = FRAMES // 2 + 1
    sqw = torch.empty((n_freq, grid.n_modes), dtype=torch.float32, device="cuda")
    sq = torch.empty(grid.n_modes, dtype=torch.float32, device="cuda")

    def step():
        job.transform()
        job.sq_total(out=sq)
        job.sqw_gauss(fwhm_frames=FRAMES / 2, n_freq=n_freq, t_step=T_STEP, out=sqw)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
            torch.cuda.synchronize()

    for _ in range(args.warmup):
        step()
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = L.mpsq_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.nvtx.range_push("bench_timed")   # lets a profiler select the timed launches
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    barrier()
    torch.cuda.nvtx.range_pop()
    launches = L.mpsq_launch_count() - launches0
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    ms = max_over_ranks(ms, dist, "cuda")
    pts_per_step = sum(counts) * FRAMES
    value = whole_job_rate(world, pts_per_step, ms)

    # e2e through the public API: pinned host trajectory in, maps out to pinned host memory
    host_frames, pin_f = host_buffer(frames.shape)
    host_frames.copy_(frames)
    host_sqw, pin_w = host_buffer(sqw.shape)
    host_sq, pin_s = host_buffer(sq.shape)

    def step_e2e():
        # chunked upload overlapping the transform; the maps land in pinned host memory by
        # copies that overlap the next step's transform (the job orders buffer reuse)
        job.transform_from_host(host_frames)
        job.sq_total(out=host_sq)
        job.sqw_gauss(fwhm_frames=FRAMES / 2, n_freq=n_freq, t_step=T_STEP, out=host_sqw)

    step_e2e()
    job.sync()
    barrier()
    e_steps = max(1, min(args.steps, 3))
    e0.record(stream)
    for _ in range(e_steps):
        step_e2e()
    job.wait_outputs()          # every step's maps are on the host before the end event
    e1.record(stream)
    job.sync()
    barrier()
    ms_e2e = e0.elapsed_time(e1) / e_steps
    ms_e2e = max_over_ranks(ms_e2e, dist, "cuda")
    e2e = {"value": whole_job_rate(world, pts_per_step, ms_e2e), "unit": UNIT,
           "h2d_bytes_per_step": int(host_frames.numel() * 4),
           "d2h_bytes_per_step": int((host_sqw.numel() + host_sq.numel()) * 4),
           "ms_per_step": ms_e2e,
           "host_memory": "pinned" if (pin_f and pin_w and pin_s) else "pageable (pinning refused)"}

    # per-stage kernel durations (CUDA events on the job's stream), one profiled pass
    job.profile(True)
    job.stage_ms(reset=True)
    job.transform()
    barrier()
    st, nfr = job.stage_ms()
    job.profile(False)
    stage = dict(zip(["bin", "spread", "fft", "deconv"], [s / nfr for s in st]))
    peak, peak_kind = measured_peaks()
    n_fine = 384 ** 3
    spread_bytes = sum(counts) * 16 + n_fine * 8
    achieved = spread_bytes / (stage["spread"] / 1e3) / 1e9
    traffic, traffic_src = profiled_traffic()
    roofline = {"bound": "hbm", "kernel": SPREAD_KERNEL, "achieved": achieved,
                "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": traffic, "traffic_source": traffic_src,
                "algorithmic_bytes_per_launch": spread_bytes,
                "ms_per_launch": stage["spread"],
                "stages_ms_per_frame": stage}

    acc = accuracy_sample(job, frames, counts, grid) if rank == 0 and not args.no_accuracy else None

    # FP64 plain path on a few frames, issued per frame (one job per frame), for the ratio
    fp64 = None
    if rank == 0 and not args.no_fp64:
        nf64 = 4
        j64 = SqomJob(grid, species_counts=counts, n_frames=1, precision=_lib.FP64,
                      stream=stream.cuda_stream, no_pack=True, **job_kwargs())
        j64.set_frames(frames[0:1])
        j64.transform()
        barrier()
        e0.record(stream)
        for t in range(nf64):
            j64.set_frames(frames[t:t + 1])
            j64.transform()
            j64.sq_total(out=sq)
        e1.record(stream)
        barrier()
        ms64 = e0.elapsed_time(e1) / nf64
        fp64 = {"value": sum(counts) / (ms64 / 1e3), "unit": UNIT, "ms_per_frame": ms64,
                "frames": nf64, "note": "per-frame FP64 plain job (no species packing)"}
        j64.close()

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu_port_frames(pos0, counts, box, grid, 1)  # thread pool / FFT warm-up, not timed
        el, pts, thr = cpu_port_frames(pos0, counts, box, grid, args.cpu_frames)
        cpu = {"value": pts / el, "unit": UNIT, "cores": thr, "kind": "port",
               "sample": f"{args.cpu_frames} frame(s) x 2 species of the same workload, "
                         f"FP64 ES NUFFT (eps {EPS}) + X-ray weights, {el:.1f} s"}

    job.close()
    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32",
               "data": "synthetic (seeded hard-sphere Al92U8 box + Gaussian random walk)",
               "config": config_dict(), "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
               "gpu_launches": int(launches), "clocks": clk, "accuracy": acc, "fp64_plain": fp64}
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_profile_case(args):
    """The per-frame pipeline of the benchmark job on a few frames only (for ncu captures:
    same atoms, grid and kernels per frame; bounded device memory and launch count)."""
    import torch

    from mp_tools_gb300 import _lib
    from mp_tools_gb300.sqom import SqomJob
    global FRAMES
    FRAMES = args.frames
    pos0, counts, box, frames = make_workload(device="cuda")
    grid = make_grid(box)
    job = SqomJob(grid, species_counts=counts, n_frames=FRAMES, precision=_lib.FP32,
                  stream=torch.cuda.current_stream().cuda_stream, **job_kwargs())
    job.set_frames(frames)
    job.transform()
    job.profile(True)
    job.transform()
    job.sync()
    st, nfr = job.stage_ms()
    print(json.dumps({"profile_case": "ok", "frames": FRAMES, "modes": grid.n_q,
                      "stage_ms_per_frame": dict(zip(["bin", "spread", "fft", "deconv"],
                                                     [s / max(nfr, 1) for s in st])),
                      "launches": int(_lib.load().mpsq_launch_count())}), flush=True)
    job.close()


def run_serving(args):
    """Serving stream (C3 shape, scaled so that it finishes in about a minute): ABO3 jobs with
    Poisson arrivals, edge / frames / zones uniform in the given ranges, FP32 at eps 1e-5,
    through the request server (continuous batching, admission by device memory), then the
    same jobs one at a time in FP64 on a bounded subset.  One JSON line with p50/p99 latency,
    throughput and the completed / rejected / queued counts."""
    import torch
    from mp_tools_gb300 import _lib, serve
    import dataclasses
    edge = tuple(int(x) for x in args.serving_edge.split(","))
    frames = tuple(int(x) for x in args.serving_frames.split(","))
    zones = tuple(int(x) for x in args.serving_zones.split(","))
    reqs = serve.poisson_stream(args.serving_jobs, 1.0, SEED + 3, edge=edge, frames=frames,
                                zones=zones)
    warm = serve.poisson_stream(2, 100.0, SEED + 4, edge=(edge[0], edge[0]), frames=(4, 4),
                                zones=(zones[0], zones[0]))
    serve.Server(max_active=args.serving_slots).run(warm)          # builds, pools, streams
    torch.cuda.synchronize()
    # capacity: the whole stream at once; then Poisson arrivals at load x capacity
    _, cap = serve.Server(max_active=args.serving_slots).run(
        [dataclasses.replace(r, arrival=0.0) for r in reqs])
    capacity = cap["nu_pts_per_s"]
    rate = args.serving_load * capacity / float(np.mean([r.nu_points for r in reqs]))
    if args.serving_rate > 0:
        rate = args.serving_rate
    rng = np.random.default_rng(SEED + 5)
    t = np.cumsum(rng.exponential(1.0 / rate, len(reqs)))
    reqs = [dataclasses.replace(r, arrival=float(a)) for r, a in zip(reqs, t)]
    srv = serve.Server(max_active=args.serving_slots)
    res, st = srv.run(reqs)
    # the baseline of the config: one job at a time in FP64 (a bounded subset)
    sub = reqs[: args.serving_fp64_jobs]
    plain = [serve.Request(r.rid, 0.0, r.frames, r.counts, r.grid,
                           dict(r.job_kwargs, precision=_lib.FP64)) for r in sub]
    t0 = time.perf_counter()
    serve.Server(max_active=1).run(plain)
    t_fp64 = time.perf_counter() - t0
    pts_sub = sum(r.nu_points for r in sub)
    out = {"metric": "job latency p50/p99 (s), serving stream", "impl": "mpsq",
           "unit": "s", "data": "synthetic (seeded ABO3 supercells, Gaussian displacements)",
           "config": {"workload": f"{len(reqs)} ABO3 jobs, Poisson arrivals at {rate:.1f} /s "
                                  f"(offered load {args.serving_load:g} x the measured capacity "
                                  f"{capacity:.3g} NU pts/s), edge {edge}, frames {frames}, "
                                  f"zones {zones}, FP32 eps 1e-5, neutron weights, S(Q) + "
                                  f"up to 4 E=const maps per job",
                      "slots": args.serving_slots, "budget_bytes": st["budget_bytes"]},
           "capacity_nu_pts_s": capacity, "capacity_p50_s": cap["p50_s"],
           "capacity_p99_s": cap["p99_s"],
           "p50_s": st["p50_s"], "p99_s": st["p99_s"], "mean_s": st["mean_s"],
           "throughput_nu_pts_s": st["nu_pts_per_s"], "wall_s": st["wall_s"],
           "completed": st["completed"], "rejected": st["rejected"], "queued": st["queued"],
           "max_queue": st["max_queue"], "peak_admitted_bytes": st["peak_admitted_bytes"],
           "fp64_one_at_a_time": {"jobs": len(sub), "nu_pts_s": pts_sub / t_fp64,
                                  "wall_s": t_fp64}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--profile-case", action="store_true",
                    help="run the per-frame pipeline on --frames frames for profiler captures")
    ap.add_argument("--frames", type=int, default=2)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mpsq", choices=["mpsq", "reference"])
    ap.add_argument("--cpu-frames", type=int, default=10)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--serving", action="store_true",
                    help="run the serving stream (request server) instead of the batched job")
    ap.add_argument("--serving-jobs", type=int, default=40)
    ap.add_argument("--serving-rate", type=float, default=0.0,
                    help="arrivals per second (0: serving-load x the measured capacity)")
    ap.add_argument("--serving-load", type=float, default=1.0)
    ap.add_argument("--serving-edge", default="8,32")
    ap.add_argument("--serving-frames", default="1,64")
    ap.add_argument("--serving-zones", default="2,4")
    ap.add_argument("--serving-slots", type=int, default=8)
    ap.add_argument("--serving-fp64-jobs", type=int, default=6)
    args = ap.parse_args()
    if args.serving:
        run_serving(args)
    elif args.profile_case:
        run_profile_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
