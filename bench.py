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
Q_RANGE, EPS = 4.72, 1e-7
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
def spread_kernel_name(width):
    return f"spread3_pair_mma_kernel<{width}>"


def profiled_traffic(width):
    """DRAM bytes (read + write) per launch of the spread kernel at this width, from the
    committed summary of an ncu capture of this workload (line 'traffic_bytes_per_launch: N')."""
    path = ROOT / "profiles" / f"spread3_pair_mma_w{width}_alu1e6_192.txt"
    try:
        for line in path.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch:"):
                return int(line.split(":")[1]), path.name
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
    cs = job.amplitudes_at(qs, ts)
    off = np.concatenate([[0], np.cumsum(counts)])
    origin, steps, extra = grid.qphys()
    m0, m1, m2 = grid.n_q
    kq = np.stack([qs % m0 - m0 // 2, (qs // m0) % m1 - m1 // 2, qs // (m0 * m1) - m2 // 2], 1)
    Qv = origin[None] + kq[:, :1] * steps[0] + kq[:, 1:2] * steps[1] + kq[:, 2:3] * steps[2]
    s2 = ((Qv ** 2).sum(1) + extra) / (16 * np.pi ** 2)
    w = [sqom_ref.xray_ff(synth.XFF[s], s2) for s in ("Al", "U")]
    got, ref = [], []
    for i, t in enumerate(ts):
        r_all = frames_dev[t, :, :3].double().cpu().numpy()
        acc = np.zeros(n_q, np.complex128)
        for s in range(2):
            r = r_all[off[s]:off[s + 1]]
            x = [r @ grid.axis[a].astype(np.float64) * float(grid.tpe[a]) for a in range(3)]
            acc += w[s] * direct_sum(x, kq)
        ref.append(acc)
        got.append(cs[i])
    out = error_metrics(np.array(got), np.array(ref))
    out["sample"] = (f"{n_q} random Q x {n_t} frames, FP64 direct sum over all 1e6 atoms "
                     f"(strong samples: |F|^2 above 1e-3 of the sample maximum)")
    return out


def maps_accuracy(job, frames_dev, counts, grid, sq, sqw, fwhm, n_freq, n_q=40):
    """Relative error of the job's outputs — total S(Q) and the Gaussian-window S(Q, omega) —
    against the oracle at n_q random Q: the FP64 direct sum of every frame's weighted
    amplitude, then the same frame sum and time transform in FP64."""
    import torch

    from oracle import sqom_ref
    from mp_tools_gb300 import synth
    rng = np.random.default_rng(17)
    qs = rng.choice(grid.n_modes, n_q, replace=False)
    off = np.concatenate([[0], np.cumsum(counts)])
    origin, steps, extra = grid.qphys()
    kq = mode_index(grid, qs)
    Qv = origin[None] + kq[:, :1] * steps[0] + kq[:, 1:2] * steps[1] + kq[:, 2:3] * steps[2]
    s2 = ((Qv ** 2).sum(1) + extra) / (16 * np.pi ** 2)
    w = [sqom_ref.xray_ff(synth.XFF[s], s2) for s in ("Al", "U")]
    F = frames_dev.shape[0]
    ref = np.zeros((F, n_q), np.complex128)
    for t in range(F):
        r_all = frames_dev[t, :, :3].double().cpu().numpy()
        for s in range(2):
            r = r_all[off[s]:off[s + 1]]
            ref[t] += w[s] * direct_sum(grid_coords(grid, r), kq)
    norm2 = job.norm2()
    g = sqom_ref.gauss_window(F, fwhm)
    qt = torch.as_tensor(qs, device="cuda")
    out = {"sq_total": map_metrics(sq[qt].cpu().numpy(), sqom_ref.sq_total(ref, norm2)),
           "sqw_gauss": map_metrics(sqw[:, qt].cpu().numpy(),
                                    sqom_ref.gauss_spectrum(ref, fwhm, n_freq, None,
                                                            T_STEP / g.sum() / norm2)),
           "sample": f"{n_q} random Q x all {F} frames (S(Q), and {n_freq} bins each for S(Q,w)), "
                     f"FP64 direct sum over all atoms, FP64 frame sum and time transform"}
    return out


def host_link(dev_in, host_in, dev_out, host_out, stream):
    """Copy bandwidth between the host buffers of the e2e leg and the device, one copy at a time
    (GB/s), and the time the step's transfers take at those rates when they follow each other on
    one copy stream, as the e2e leg issues them: the floor of the e2e step."""
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {}
    for name, dst, src in (("h2d", dev_in, host_in), ("d2h", host_out, dev_out)):
        torch.cuda.synchronize()
        e0.record(stream)
        dst.copy_(src, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize()
        out[name + "_gbs"] = src.numel() * src.element_size() / (e0.elapsed_time(e1) * 1e6)
    out["transfer_ms_per_step"] = (host_in.numel() * 4 / (out["h2d_gbs"] * 1e6)
                                   + host_out.numel() * 4 / (out["d2h_gbs"] * 1e6))
    return out


def graph_vs_stream(job, frames):
    """ms per frame of transform(0, frames) issued launch by launch and replayed as a captured
    CUDA graph (each after one untimed call); the job's graph option is restored."""
    import torch
    from mp_tools_gb300 import _lib
    before = job.get_option(_lib.OPT_GRAPH)
    out = {}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    st = torch.cuda.current_stream()
    for g in (0, 1, 0, 1):
        job.set_option(_lib.OPT_GRAPH, g)
        job.transform(0, frames)
        e0.record(st)
        for _ in range(3):
            job.transform(0, frames)
        e1.record(st)
        torch.cuda.synchronize()
        out.setdefault("graph" if g else "stream", []).append(e0.elapsed_time(e1) / (3 * frames))
    job.set_option(_lib.OPT_GRAPH, before)
    return {"stream_ms_per_frame": min(out["stream"]), "graph_ms_per_frame": min(out["graph"]),
            "frames_per_call": frames}


def error_metrics(got, ref):
    """Relative l2 errors of amplitudes and of |F|^2, and the largest relative |F|^2 error over
    the samples whose oracle |F|^2 exceeds 1e-3 of the sample maximum."""
    got = np.asarray(got, np.complex128).ravel()
    ref = np.asarray(ref, np.complex128).ravel()
    s_got, s_ref = np.abs(got) ** 2, np.abs(ref) ** 2
    strong = s_ref > 1e-3 * s_ref.max()
    rel = np.abs(s_got - s_ref) / np.maximum(s_ref, 1e-300)
    worst = int(np.argmax(np.where(strong, rel, -1.0))) if strong.any() else None
    return {"rel_l2_amplitude": float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
            "rel_l2_S": float(np.linalg.norm(s_got - s_ref) / np.linalg.norm(s_ref)),
            "max_rel_S": float(rel[worst]) if worst is not None else None,
            "worst_S_over_max": float(s_ref[worst] / s_ref.max()) if worst is not None else None,
            "max_rel_S_above_1e-2_max": (float(rel[s_ref > 1e-2 * s_ref.max()].max())
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
    # run-time choices: graph replay vs stream-issued launches timed on 16 frames, then the
    # autotuner's pick over graph / spreading kernel / X-pass rows / lanes (what the steps use)
    graph_ab = graph_vs_stream(job, 16)
    tune = job.autotune(0, 16, cache=args.tune_cache or None)
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
    e_steps = args.steps
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
    e2e["host_link"] = host_link(frames, host_frames, sqw, host_sqw, stream)

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
    width = job.info()["width"]
    traffic, traffic_src = profiled_traffic(width)
    kernel = (spread_kernel_name(width) if tune["spread"] == "tensor-core"
              else f"spread3_f32_w_kernel<{width}>")
    if tune["spread"] != "tensor-core":
        traffic, traffic_src = None, None
    roofline = {"bound": "hbm", "kernel": kernel, "achieved": achieved,
                "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": traffic, "traffic_source": traffic_src,
                "algorithmic_bytes_per_launch": spread_bytes,
                "ms_per_launch": stage["spread"],
                "stages_ms_per_frame": stage}

    acc = None
    if rank == 0 and not args.no_accuracy:
        acc = {"frames": accuracy_sample(job, frames, counts, grid, n_q=args.acc_q, n_t=args.acc_t),
               "maps": maps_accuracy(job, frames, counts, grid, sq, sqw, FRAMES / 2, n_freq,
                                     n_q=args.acc_map_q)}

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
               "gpu_launches": int(launches), "clocks": clk, "accuracy": acc, "fp64_plain": fp64,
               "launch_forms": graph_ab, "autotune": tune}
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
    """Serving stream: ABO3 jobs with Poisson arrivals, edge / frames / zones uniform in the
    given ranges, FP32 at eps 1e-5, through the request server (continuous batching, admission
    by device memory, jobs larger than the budget run by Q slabs), then the same kind of jobs
    one at a time in FP64 on a bounded subset (the smallest).  --serving-c3 takes the serving
    configuration's own ranges (edge 16-100 cells, 1-256 frames, 4-8 zones) with plane-wave
    trajectories made on the device at admission; the default is a scaled-down mix with host
    trajectories.  The offered rate is --serving-load x the capacity measured on the first
    --serving-capacity-jobs jobs submitted at once.  One JSON line with p50/p99 latency,
    throughput and the completed / rejected / queued counts."""
    import torch
    from mp_tools_gb300 import _lib, serve
    import dataclasses
    if args.serving_c3:
        args.serving_edge, args.serving_frames, args.serving_zones = "16,100", "1,256", "4,8"
    edge = tuple(int(x) for x in args.serving_edge.split(","))
    frames = tuple(int(x) for x in args.serving_frames.split(","))
    zones = tuple(int(x) for x in args.serving_zones.split(","))
    dev = bool(args.serving_c3)
    free, _ = torch.cuda.mem_get_info()
    budget = int(args.serving_budget_frac * free)
    reqs = serve.poisson_stream(args.serving_jobs, 1.0, SEED + 3, edge=edge, frames=frames,
                                zones=zones, device_frames=dev)
    warm = serve.poisson_stream(2, 100.0, SEED + 4, edge=(edge[0], edge[0]), frames=(4, 4),
                                zones=(zones[0], zones[0]), device_frames=dev)
    serve.Server(budget_bytes=budget, max_active=args.serving_slots, keep_results=False).run(warm)
    torch.cuda.synchronize()
    # capacity: the first jobs of the stream at once; then Poisson arrivals at load x capacity
    k = args.serving_capacity_jobs or len(reqs)
    cap_reqs = [dataclasses.replace(r, arrival=0.0) for r in reqs[:k]]
    _, cap = serve.Server(budget_bytes=budget, max_active=args.serving_slots,
                          keep_results=False).run(cap_reqs)
    capacity = cap["nu_pts_per_s"]
    rate = args.serving_load * capacity / float(np.mean([r.nu_points for r in reqs]))
    if args.serving_rate > 0:
        rate = args.serving_rate
    rng = np.random.default_rng(SEED + 5)
    t = np.cumsum(rng.exponential(1.0 / rate, len(reqs)))
    reqs = [dataclasses.replace(r, arrival=float(a)) for r, a in zip(reqs, t)]
    srv = serve.Server(budget_bytes=budget, max_active=args.serving_slots, keep_results=False)
    res, st = srv.run(reqs)
    slabbed = sum(1 for r in reqs if getattr(r, "_q_slab", 0))
    # the baseline of the config: one job at a time in FP64 (the smallest jobs of the stream)
    sub = sorted(reqs, key=lambda r: r.nu_points * r.grid.n_modes)[: args.serving_fp64_jobs]
    plain = [serve.Request(r.rid, 0.0, r.frames, r.counts, r.grid,
                           dict(r.job_kwargs, precision=_lib.FP64), t_step=r.t_step) for r in sub]
    t0 = time.perf_counter()
    serve.Server(budget_bytes=budget, max_active=1, keep_results=False).run(plain)
    t_fp64 = time.perf_counter() - t0
    pts_sub = sum(r.nu_points for r in sub)
    t0 = time.perf_counter()
    serve.Server(budget_bytes=budget, max_active=1, keep_results=False).run(
        [dataclasses.replace(r, arrival=0.0) for r in sub])
    t_fp32_sub = time.perf_counter() - t0
    kind = ("plane-wave trajectories made on the device at admission" if dev
            else "Gaussian displacements, host trajectories")
    out = {"metric": "job latency p50/p99 (s), serving stream", "impl": "mpsq",
           "unit": "s", "data": f"synthetic (seeded ABO3 supercells, {kind})",
           "config": {"workload": f"{len(reqs)} ABO3 jobs, Poisson arrivals at {rate:.3g} /s "
                                  f"(offered load {args.serving_load:g} x the measured capacity "
                                  f"{capacity:.3g} NU pts/s), edge {edge}, frames {frames}, "
                                  f"zones {zones}, FP32 eps 1e-5, neutron weights, S(Q) + "
                                  f"up to 4 E=const maps per job",
                      "slots": args.serving_slots, "budget_bytes": st["budget_bytes"],
                      "capacity_jobs": k},
           "capacity_nu_pts_s": capacity, "capacity_p50_s": cap["p50_s"],
           "capacity_p99_s": cap["p99_s"],
           "p50_s": st["p50_s"], "p99_s": st["p99_s"], "mean_s": st["mean_s"],
           "throughput_nu_pts_s": st["nu_pts_per_s"], "wall_s": st["wall_s"],
           "completed": st["completed"], "rejected": st["rejected"], "queued": st["queued"],
           "failed": st["failed"],
           "max_queue": st["max_queue"], "peak_admitted_bytes": st["peak_admitted_bytes"],
           "jobs_run_by_q_slabs": slabbed,
           "fp64_one_at_a_time": {"jobs": len(sub), "nu_pts_s": pts_sub / t_fp64,
                                  "wall_s": t_fp64,
                                  "fp32_same_jobs_one_at_a_time_nu_pts_s": pts_sub / t_fp32_sub}}
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------------ further configurations
# Seeded synthetic inputs with the shapes, sizes and distributions of the other benchmark
# configurations (seed 20261203 + configuration index).  Each prints one JSON line of the same
# form as the default run: device-resident value, e2e through the public API from pinned host
# memory, the dominant kernel's roofline, the accuracy against the FP64 direct-sum oracle.
CFG_SEED = 20261203
ABO3_A = 4.19


def neutron_b():
    from mp_tools_gb300 import synth
    return [0.1 * b for b in synth.ABO3_B_COH_FM]


def grid_coords(grid, r):
    """NUFFT coordinates (radians, FP64) of positions r (N x 3) on a QGrid."""
    return [r @ grid.axis[a].astype(np.float64) * float(grid.tpe[a]) for a in range(3)]


def oracle_amplitudes(frame, counts, grid, weights, kq):
    """FP64 direct sum of the weighted amplitude sum_s w_s(Q) A_s(Q) of one frame (float32
    (N, 4)) at the integer modes kq (n x 3); weights: per species, a scalar or an array over
    the sampled modes."""
    import oracle
    off = np.concatenate([[0], np.cumsum(counts)])
    r_all = np.asarray(frame[:, :3], np.float64)
    acc = np.zeros(len(kq), np.complex128)
    for s in range(len(counts)):
        r = r_all[off[s]:off[s + 1]]
        x = grid_coords(grid, r)
        keep = ~((r[:, 0] == 0) & (r[:, 1] == 0) & (r[:, 2] == 0)) if grid.input_method == 0 else None
        if keep is not None and not keep.all():
            x = [c[keep] for c in x]
        acc += np.asarray(weights[s]) * direct_sum(x, kq)
    return acc


def direct_sum(x, kq):
    """FP64 direct type-1 sum of unit strengths at modes kq: per point either one exponential
    per mode or phase tables along each axis, whichever costs less."""
    import oracle
    span = (kq.max(axis=0) - kq.min(axis=0) + 1).sum()
    if 8 * len(kq) < span + 2 * len(kq):
        return oracle.dirft_modes(x[0], x[1], x[2], np.ones(len(x[0])), -1, kq)
    return oracle.dirft_modes_tab(x[0], x[1], x[2], np.ones(len(x[0])), -1, kq)


def map_metrics(got, want):
    """Relative l2 error of a map sample and the largest relative error over the samples above
    1e-3 of the sample maximum."""
    got = np.asarray(got, np.float64).ravel()
    want = np.asarray(want, np.float64).ravel()
    strong = want > 1e-3 * want.max()
    return {"rel_l2_S": float(np.linalg.norm(got - want) / np.linalg.norm(want)),
            "max_rel_S": float(np.max(np.abs(got[strong] - want[strong]) / want[strong]))}


def mode_index(grid, q):
    m0, m1, m2 = grid.n_q
    return np.stack([q % m0 - m0 // 2, (q // m0) % m1 - m1 // 2, q // (m0 * m1) - m2 // 2], 1)


def timed_steps(step, args, stream, L):
    """W untimed steps, then K timed steps bracketed by synchronisation; returns ms per step,
    the clock record and the number of this library's launches in the timed region."""
    import torch
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(env_int("LOCAL_RANK", 0))
    clocks.start()
    n0 = L.mpsq_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / args.steps, clocks.stop(), int(L.mpsq_launch_count() - n0)


def spread_roofline(job, pts_per_frame, kernel):
    """Stage times of one profiled transform pass; the spread kernel's algorithmic bytes
    (16 B per point + 8 or 16 B per fine-grid cell and grid) over its CUDA-event duration."""
    import torch
    info = job.info()
    job.profile(True)
    job.stage_ms(reset=True)
    job.transform()
    torch.cuda.synchronize()
    st, nfr = job.stage_ms()
    job.profile(False)
    stage = dict(zip(["bin", "spread", "fft", "deconv"], [v / max(nfr, 1) for v in st]))
    nf = info["fine_grid"]
    cell = 16 if job.precision == 1 else 8
    ngrid = job.n_grids()
    spread_bytes = pts_per_frame * 16 + ngrid * nf[0] * nf[1] * nf[2] * cell
    peak, peak_kind = measured_peaks()
    achieved = spread_bytes / (stage["spread"] / 1e3) / 1e9
    return {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "traffic": None,
            "algorithmic_bytes_per_launch": int(spread_bytes), "ms_per_launch": stage["spread"],
            "stages_ms_per_frame": stage, "width": info["width"], "fine_grid": list(nf),
            "pruned_fft": info["pruned"]}


def cpu_port_job(frames_np, counts, grid, weights_full, eps, n_frames):
    """The oracle's CPU port (FP64 ES NUFFT per species and frame + weighting + |F|^2) on
    n_frames frames; returns (seconds, points, threads)."""
    import oracle
    off = np.concatenate([[0], np.cumsum(counts)])
    cs = np.empty(grid.n_modes, np.complex128)
    s_q = np.zeros(grid.n_modes, np.float64)
    el, pts = 0.0, 0
    for t in range(n_frames):
        fr = frames_np[t % len(frames_np)]
        t0 = time.perf_counter()
        for s in range(len(counts)):
            r = np.asarray(fr[off[s]:off[s + 1], :3], np.float64)
            A = oracle.es_nufft(grid_coords(grid, r), np.ones(len(r)), -1, eps, grid.n_q)
            oracle.weight_accumulate(cs, weights_full[s], A, first=(s == 0))
        oracle.abs2_accumulate(s_q, cs)
        el += time.perf_counter() - t0
        pts += int(off[-1])
    return el, pts, oracle.num_threads()


def full_weights(grid, counts, b):
    return [np.full(grid.n_modes, float(b[s])) for s in range(len(counts))]


def run_config_job(name, metric, workload, args):
    """Shared driver of the job configurations.  workload() returns a dict with: frames (torch
    (F, N, 4) on cuda), counts, grid, job kwargs (`kw`), `maps(job, outs)` issuing the step's
    maps into the given output tensors, `outs` (device tensors), `accuracy(job, frames)`,
    `config` (dict), `pts_per_step`, and optional `fp64` / `cpu` callables."""
    import torch

    from mp_tools_gb300 import _lib
    from mp_tools_gb300.sqom import SqomJob
    torch.cuda.set_device(env_int("LOCAL_RANK", 0))
    L = _lib.load()
    wl = workload()
    stream = torch.cuda.current_stream()
    frames, grid = wl["frames"], wl["grid"]
    job = SqomJob(grid, species_counts=wl["counts"], n_frames=frames.shape[0],
                  stream=stream.cuda_stream, n_atoms_frame=frames.shape[1], **wl["kw"])
    job.set_frames(frames)
    outs = wl["outs"]

    def step():
        job.transform()
        wl["maps"](job, outs)

    ms, clk, launches = timed_steps(step, args, stream, L)
    value = wl["pts_per_step"] / (ms / 1e3)
    # e2e through the public API from pinned host memory
    host_frames, pin_f = host_buffer(frames.shape)
    host_frames.copy_(frames)
    host_outs = [host_buffer(o.shape) for o in outs]
    pinned = pin_f and all(p for _, p in host_outs)
    houts = [h for h, _ in host_outs]

    def step_e2e():
        job.transform_from_host(host_frames)
        wl["maps"](job, houts)

    step_e2e()
    job.sync()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step_e2e()
    job.wait_outputs()
    e1.record(stream)
    job.sync()
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1) / args.steps
    e2e = {"value": wl["pts_per_step"] / (ms_e2e / 1e3), "unit": UNIT,
           "h2d_bytes_per_step": int(host_frames.numel() * 4),
           "d2h_bytes_per_step": int(sum(h.numel() * 4 for h in houts)), "ms_per_step": ms_e2e,
           "host_memory": "pinned" if pinned else "pageable (pinning refused)"}
    roof = spread_roofline(job, int(sum(wl["counts"])), wl.get("kernel", "spread"))
    acc = None if args.no_accuracy else wl["accuracy"](job, frames, outs)
    fp64 = wl["fp64"](stream) if (wl.get("fp64") and not args.no_fp64) else None
    job.close()
    cpu = wl["cpu"]() if (wl.get("cpu") and not args.no_cpu) else None
    out = {"metric": metric, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": wl["dtype"], "data": wl["data"], "config": wl["config"],
           "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
           "clocks": clk, "accuracy": acc, "fp64_plain": fp64}
    print(json.dumps(out), flush=True)


def fp64_per_frame(frames, counts, grid, kw, stream, n=2):
    """The same frames through the FP64 plain path, one single-frame job per frame."""
    import torch

    from mp_tools_gb300 import _lib
    from mp_tools_gb300.sqom import SqomJob
    kw = dict(kw, precision=_lib.FP64)
    j64 = SqomJob(grid, species_counts=counts, n_frames=1, stream=stream.cuda_stream,
                  n_atoms_frame=frames.shape[1], no_pack=True, **kw)
    sq = torch.empty(grid.n_modes, dtype=torch.float32, device="cuda")
    j64.set_frames(frames[0:1])
    j64.transform()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for t in range(n):
        j64.set_frames(frames[t:t + 1])
        j64.transform()
        j64.sq_total(out=sq)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / n
    j64.close()
    return {"value": sum(counts) / (ms / 1e3), "unit": UNIT, "ms_per_frame": ms, "frames": n,
            "note": "per-frame FP64 plain job (no species packing)"}


def workload_c0():
    """ABO3 20^3 cells (40,000 atoms), Gaussian displacements, neutron weights, one frame, 160^3
    modes (8 zones per axis), FP64 at eps 1e-9; S(Q) checked on the central 32^3 sub-grid."""
    import torch

    from mp_tools_gb300 import _lib, synth
    from mp_tools_gb300.sqom import QGrid
    eps = EPS_CFG if EPS_CFG is not None else 1e-9
    rng = np.random.default_rng(CFG_SEED + 0)
    pos, _, counts = synth.abo3_static(20, ABO3_A, rng)
    grid = QGrid(_lib.CELL, (20, 20, 20), n_bz=8, a_par=(ABO3_A,) * 3, ndim=3)
    frames = torch.from_numpy(pos[None]).cuda()
    b = neutron_b()
    kw = dict(precision=_lib.FP64, eps=eps, weight_mode=_lib.WEIGHT_NEUTRON, b_coh=b)
    sq = torch.empty(grid.n_modes, dtype=torch.float32, device="cuda")

    def maps(job, outs):
        job.sq_total(out=outs[0])

    def accuracy(job, frames_dev, outs):
        k = np.arange(-16, 16)
        kz, ky, kx = np.meshgrid(k, k, k, indexing="ij")
        kq = np.stack([kx.ravel(), ky.ravel(), kz.ravel()], 1)
        m = np.array(grid.n_q)
        q = ((kq[:, 2] + m[2] // 2) * m[1] + kq[:, 1] + m[1] // 2) * m[0] + kq[:, 0] + m[0] // 2
        ref = oracle_amplitudes(pos, counts, grid, b, kq)
        out = error_metrics(job.amplitudes_at(q)[0], ref)
        out["sample"] = "central 32^3 sub-grid (32,768 modes), FP64 direct sum over all 40,000 atoms"
        return out

    def cpu():
        el, pts, thr = cpu_port_job(pos[None], counts, grid, full_weights(grid, counts, b), eps, 3)
        return {"value": pts / el, "unit": UNIT, "cores": thr, "kind": "port",
                "sample": f"the frame 3 times, 5 species, FP64 ES NUFFT eps {eps} + weights, {el:.1f} s"}

    return dict(frames=frames, counts=counts, grid=grid, kw=kw, maps=maps, outs=[sq],
                accuracy=accuracy, cpu=cpu, pts_per_step=int(sum(counts)), dtype="f64",
                kernel="spread_tile_kernel<double,3>",
                data="synthetic (seeded ABO3 supercell, Gaussian displacements)",
                config={"workload": "static S(Q) of ABO3 20^3 cells (40,000 atoms), 160^3 modes, "
                                    "FP64 eps %g, neutron weights" % eps,
                        "atoms": int(sum(counts)), "frames": 1, "species": 5,
                        "modes": list(grid.n_q), "eps": eps, "precision": "fp64",
                        "l2": "fine grid 320^3 complex128 (524 MB) larger than L2",
                        "parallelism": "single GPU"})


def workload_c1():
    """ABO3 64^3 cells (1,310,720 atoms) displaced by 48 seeded plane waves, 256 frames at
    10 fs, 256^3 modes (4 zones per axis), FP32 at eps 1e-6, neutron weights; Gaussian window
    (FWHM 128 frames) + 256-point transform per Q, 129 bins, and two E=const maps of the
    sliding Hann window (n_int 129, 128 start frames) at bins 5 and 17."""
    import torch

    from mp_tools_gb300 import _lib, synth
    from mp_tools_gb300.sqom import QGrid, TimeAxis
    from oracle import sqom_ref
    eps = EPS_CFG if EPS_CFG is not None else 1e-6
    F, n, dt = 256, 64, 0.01
    rng = np.random.default_rng(CFG_SEED + 1)
    frames, counts, _ = synth.abo3_planewave_frames(n, F, dt, ABO3_A, rng, device="cuda")
    grid = QGrid(_lib.CELL, (n, n, n), n_bz=4, a_par=(ABO3_A,) * 3, ndim=3)
    b = neutron_b()
    kw = dict(precision=_lib.FP32, eps=eps, weight_mode=_lib.WEIGHT_NEUTRON, b_coh=b)
    n_freq = F // 2 + 1
    fwhm = F / 2
    taxis = TimeAxis(F, dt, n_int=129)
    bins = (5, 17)
    outs = [torch.empty((n_freq, grid.n_modes), dtype=torch.float32, device="cuda"),
            torch.empty(grid.n_modes, dtype=torch.float32, device="cuda")] + \
           [torch.empty(grid.n_modes, dtype=torch.float32, device="cuda") for _ in bins]

    def maps(job, o):
        job.sqw_gauss(fwhm_frames=fwhm, n_freq=n_freq, t_step=dt, out=o[0])
        job.sq_total(out=o[1])
        for i, jf in enumerate(bins):
            job.sqw_econst(taxis, jf, out=o[2 + i])

    def accuracy(job, frames_dev, o):
        # 1,000 (Q, omega) points: 40 random Q x 25 random Gaussian-spectrum bins, and the same
        # 40 Q at the two E=const bins; the oracle forms F(Q, t) for all 256 frames by direct sum
        # and applies the same time transforms in FP64
        rq = np.random.default_rng(11)
        q = rq.choice(grid.n_modes, 40, replace=False)
        kq = mode_index(grid, q)
        ref = np.zeros((F, len(q)), np.complex128)
        for t in range(F):
            ref[t] = oracle_amplitudes(frames_dev[t].cpu().numpy(), counts, grid, b, kq)
        norm2 = job.norm2()
        g = sqom_ref.gauss_window(F, fwhm)
        sq_ref = sqom_ref.gauss_spectrum(ref, fwhm, n_freq, None, dt / g.sum() / norm2)
        wbin = rq.integers(0, n_freq, (len(q), 25))
        qt = torch.as_tensor(q, device="cuda")
        got_g = o[0][:, qt].cpu().numpy()                    # (n_freq, 40)
        cols = np.arange(len(q))[:, None]
        out = {"gauss": map_metrics(got_g[wbin, cols], sq_ref[wbin, cols])}
        tw = taxis.window().astype(np.float64)
        for i, jf in enumerate(bins):
            want = sqom_ref.econst(ref, taxis.n_int, tw, jf, None,
                                   dt / (0.5 * taxis.n_frame * taxis.n_int) / norm2)
            out[f"econst_bin{jf}"] = map_metrics(o[2 + i][qt].cpu().numpy(), want)
        cs = job.amplitudes_at(q)
        out["amplitudes"] = error_metrics(cs, ref)
        out["sample"] = ("40 random Q x 25 random bins of the Gaussian spectrum (1,000 (Q,w) "
                         "points) and the 40 Q at E=const bins 5 and 17; FP64 direct sum of all "
                         "256 frames over all 1,310,720 atoms, FP64 time transforms")
        return out

    def fp64(stream):
        return fp64_per_frame(frames, counts, grid, kw, stream, n=2)

    def cpu():
        fr = frames[0:1].cpu().numpy()
        el, pts, thr = cpu_port_job(fr, counts, grid, full_weights(grid, counts, b), eps, 1)
        return {"value": pts / el, "unit": UNIT, "cores": thr, "kind": "port",
                "sample": f"1 frame x 5 species (1,310,720 atoms, 256^3 modes), FP64 ES NUFFT "
                          f"eps {eps} + weights, {el:.1f} s"}

    return dict(frames=frames, counts=counts, grid=grid, kw=kw, maps=maps, outs=outs,
                accuracy=accuracy, fp64=fp64, cpu=cpu, pts_per_step=int(sum(counts)) * F,
                dtype="f32", kernel="spread3_pair_mma_kernel",
                data="synthetic (seeded ABO3 supercell, 48 plane-wave modes)",
                config={"workload": "inelastic S(Q,w) of ABO3 64^3 cells (1,310,720 atoms), "
                                    "256 frames, 256^3 modes, FP32 eps %g, neutron weights, "
                                    "Gaussian window + sliding Hann E=const maps" % eps,
                        "atoms": int(sum(counts)), "frames": F, "species": 5,
                        "modes": list(grid.n_q), "eps": eps, "precision": "fp32 split",
                        "time_transform": "Gaussian FWHM 128 frames, 256-point DFT, 129 bins; "
                                          "sliding Hann n_int 129 at bins 5, 17; total S(Q)",
                        "l2": "inputs larger than L2 (5.4 GB trajectory, 34 GB amplitude store)",
                        "parallelism": "single GPU"})


def workload_c4():
    """ABO3 136^3 cells (12,577,280 atoms), one frame: Gaussian displacements plus 90-degree
    domain walls (B sites +-0.1 A along z in alternating 17-cell slabs), 544^3 modes (4 zones),
    fine grid 1152^3, FP32 spreading with FP64-exact phase reduction at eps 1e-5; 4,096 random Q
    against the FP64 direct sum."""
    import torch

    from mp_tools_gb300 import _lib, synth
    from mp_tools_gb300.sqom import QGrid
    eps = EPS_CFG if EPS_CFG is not None else 1e-5
    n = 136
    rng = np.random.default_rng(CFG_SEED + 4)
    shift = synth.domain_wall_shift(n, ABO3_A, rng)
    pos, _, counts = synth.abo3_static(n, ABO3_A, rng, extra_b=shift)
    grid = QGrid(_lib.CELL, (n, n, n), n_bz=4, a_par=(ABO3_A,) * 3, ndim=3)
    frames = torch.from_numpy(pos[None]).cuda()
    b = neutron_b()
    kw = dict(precision=_lib.FP32, eps=eps, weight_mode=_lib.WEIGHT_NEUTRON, b_coh=b)
    sq = torch.empty(grid.n_modes, dtype=torch.float32, device="cuda")

    def maps(job, outs):
        job.sq_total(out=outs[0])

    def accuracy(job, frames_dev, outs):
        rq = np.random.default_rng(13)
        q = rq.choice(grid.n_modes, 4096, replace=False)
        ref = oracle_amplitudes(pos, counts, grid, b, mode_index(grid, q))
        out = error_metrics(job.amplitudes_at(q)[0], ref)
        out["sample"] = "4,096 random Q, FP64 direct sum over all 12,577,280 atoms"
        return out

    def cpu():
        import oracle
        off = np.concatenate([[0], np.cumsum(counts)])
        r = np.asarray(pos[off[1]:off[2], :3], np.float64)
        t0 = time.perf_counter()
        oracle.es_nufft(grid_coords(grid, r), np.ones(len(r)), -1, eps, grid.n_q)
        el = time.perf_counter() - t0
        return {"value": len(r) / el, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
                "sample": f"one species transform (B sites, 2,515,456 atoms, 544^3 modes, fine "
                          f"grid 1152^3 complex128), FP64 ES NUFFT eps {eps}, {el:.1f} s"}

    return dict(frames=frames, counts=counts, grid=grid, kw=kw, maps=maps, outs=[sq],
                accuracy=accuracy, cpu=cpu, pts_per_step=int(sum(counts)), dtype="f32",
                kernel="spread3_pair_mma_kernel",
                data="synthetic (seeded ABO3 supercell, Gaussian displacements, domain walls)",
                config={"workload": "large static S(Q) of ABO3 136^3 cells (12,577,280 atoms), "
                                    "544^3 modes, fine grid 1152^3, FP32 eps %g" % eps,
                        "atoms": int(sum(counts)), "frames": 1, "species": 5,
                        "modes": list(grid.n_q), "eps": eps, "precision": "fp32 split",
                        "l2": "fine grids of 12.2 GB each, larger than L2",
                        "parallelism": "single GPU"})


def run_dropin2d(args):
    """The reference's own call pattern through the drop-in boundary: an unmodified mp_sqom
    calls finufft2d1_ (Fortran convention, every argument by reference, host arrays, NULL
    opts) once per frame and species on the (hk0) plane (code/src/mp_sqom56.f90:1144-1156).
    Workload of the reference's BZO example log (examples/single_crystal_BZO/
    mp_sqom_cmd_log.txt): ABO3 32^3 cells (163,840 atoms, 5 species of 32,768), 160 x 160
    modes (5 zones, Q centre (2 2 0)), 20 frames x 5 species = 100 calls at eps 1e-6.  value: NU points per
    second of the calls, host arrays in and out (the e2e form is the only form this boundary
    has); the CPU port times the same calls."""
    import ctypes as C

    import torch

    import oracle
    from mp_tools_gb300 import _lib, synth
    torch.cuda.set_device(env_int("LOCAL_RANK", 0))
    L = _lib.load()
    eps = EPS_CFG if EPS_CFG is not None else 1e-6
    n, F, ms = 32, 20, 160
    rng = np.random.default_rng(CFG_SEED + 5)
    calls = []                     # (xf, yf, cf) per frame and species, as mp_sqom prepares them
    for t in range(F):
        pos, _, counts = synth.abo3_static(n, ABO3_A, rng)
        off = np.concatenate([[0], np.cumsum(counts)])
        for sp in range(5):
            r = pos[off[sp]:off[sp + 1], :3].astype(np.float32)
            tpe = np.float32(2 * np.pi / n)
            xf = np.ascontiguousarray((r[:, 0] * tpe).astype(np.float64))
            yf = np.ascontiguousarray((r[:, 1] * tpe).astype(np.float64))
            # Q centre (2 2 0) of the example: strengths exp(-2 pi i q_c . r) (:1101-1117)
            cf = np.exp(-2j * np.pi * (2.0 * r[:, 0].astype(np.float64) + 2.0 * r[:, 1]))
            calls.append((xf, yf, np.ascontiguousarray(cf)))
    fk = np.zeros(ms * ms, np.complex128)
    dp = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    m1, m2, iflag, epsc, ier = C.c_int64(ms), C.c_int64(ms), C.c_int(-1), C.c_double(eps), C.c_int(0)

    def one(xf, yf, cf):
        nj = C.c_int64(len(xf))
        L.finufft2d1_(C.byref(nj), dp(xf), dp(yf), dp(cf), C.byref(iflag), C.byref(epsc),
                      C.byref(m1), C.byref(m2), dp(fk), None, C.byref(ier))
        if ier.value != 0:
            raise RuntimeError(L.mpsq_last_error())

    def step():
        for c in calls:
            one(*c)

    for _ in range(args.warmup):
        step()
    clocks = ClockSampler(env_int("LOCAL_RANK", 0))
    clocks.start()
    n0 = L.mpsq_launch_count()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    el = (time.perf_counter() - t0) / args.steps
    launches = int(L.mpsq_launch_count() - n0)
    clk = clocks.stop()
    pts = sum(len(c[0]) for c in calls)
    # accuracy of one call against the FP64 direct sum (all 160 x 160 modes)
    xf, yf, cf = calls[1]
    one(xf, yf, cf)
    ref = oracle.dirft2d1(xf, yf, cf, -1, ms, ms).ravel()
    acc = error_metrics(fk.copy(), ref)
    acc["sample"] = "one call (B sites of frame 1, 32,768 points), all 160 x 160 modes, FP64 direct sum"
    cpu = None
    if not args.no_cpu:
        oracle.es_nufft([calls[0][0], calls[0][1]], calls[0][2], -1, eps, (ms, ms))
        t0 = time.perf_counter()
        for c in calls:
            oracle.es_nufft([c[0], c[1]], c[2], -1, eps, (ms, ms))
        el_cpu = time.perf_counter() - t0
        cpu = {"value": pts / el_cpu, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
               "sample": f"the same 100 calls (20 frames x 5 species, 32,768 points, 160 x 160 "
                         f"modes), FP64 ES NUFFT eps {eps}, {el_cpu:.2f} s"}
    out = {"metric": "NU pts/s finufft2d1_ drop-in calls (BZO 32^3 cells, 100 x 32,768 pts, 160^2 Q)",
           "value": pts / el, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * el, "ms_per_call": 1e3 * el / len(calls),
           "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded ABO3 32^3 supercells)",
           "config": {"workload": "mp_sqom's call pattern through finufft2d1_: 20 frames x 5 "
                                  "species, 32,768 points per call, 160 x 160 modes, eps %g, "
                                  "host arrays by reference" % eps,
                      "calls_per_step": len(calls), "points_per_call": 32768, "modes": [ms, ms],
                      "eps": eps, "precision": "fp64", "parallelism": "single GPU"},
           "reference_published": {"value": 100 * 32768 / 0.825, "unit": UNIT,
                                   "note": "the reference's own log: 0.825 s for 100 transforms "
                                           "of 32,768 points onto 160^2 (FINUFFT + OpenMP, its "
                                           "machine)"},
           "e2e": {"value": pts / el, "unit": UNIT,
                   "h2d_bytes_per_step": int(sum(32 * len(c[0]) for c in calls)),
                   "d2h_bytes_per_step": int(len(calls) * fk.nbytes), "ms_per_step": 1e3 * el},
           "cpu_baseline": cpu, "gpu_launches": launches, "clocks": clk, "accuracy": acc}
    print(json.dumps(out), flush=True)


EPS_CFG = None
CONFIGS = {
    "c0": ("NU pts/s static S(Q) FP64 plain (ABO3 20^3 cells, 40,000 atoms, 160^3 Q, eps 1e-9)",
           workload_c0),
    "c1": ("NU pts/s S(Q,w) FP32 batched (ABO3 64^3 cells, 1.31e6 atoms, 256 frames, 256^3 Q)",
           workload_c1),
    "c4": ("NU pts/s static S(Q) FP32 (ABO3 136^3 cells, 1.26e7 atoms, 544^3 Q)", workload_c4),
}


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
    ap.add_argument("--acc-q", type=int, default=1000, help="random Q modes of the accuracy sample")
    ap.add_argument("--acc-t", type=int, default=3, help="frames of the accuracy sample")
    ap.add_argument("--acc-map-q", type=int, default=40,
                    help="random Q of the S(Q) / S(Q,w) accuracy sample (all frames)")
    ap.add_argument("--eps", type=float, default=None, help="NUFFT tolerance (default: the config's)")
    ap.add_argument("--tune-cache", default="", help="autotuner cache file (default: none)")
    ap.add_argument("--config", default="c2", choices=["c0", "c1", "c2", "c4", "dropin2d"],
                    help="workload: c2 the batched amorphous alloy (default, the headline); c0 "
                         "static FP64 ABO3 20^3; c1 inelastic ABO3 64^3 x 256 frames; c4 static "
                         "ABO3 136^3; dropin2d mp_sqom's own finufft2d1_ call pattern")
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
    ap.add_argument("--serving-c3", action="store_true",
                    help="the serving configuration's own ranges (edge 16-100, 1-256 frames, "
                         "4-8 zones), trajectories made on the device")
    ap.add_argument("--serving-budget-frac", type=float, default=0.8,
                    help="device memory budget of the server, as a fraction of the free memory")
    ap.add_argument("--serving-capacity-jobs", type=int, default=0,
                    help="jobs of the capacity measurement (0: all)")
    args = ap.parse_args()
    if args.eps is not None:
        global EPS, EPS_CFG
        EPS = args.eps
        EPS_CFG = args.eps
    if args.config == "dropin2d" and args.impl != "reference":
        run_dropin2d(args)
        return
    if args.config != "c2" and args.impl != "reference" and not args.serving:
        metric, wl = CONFIGS[args.config]
        run_config_job(args.config, metric, wl, args)
        return
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
