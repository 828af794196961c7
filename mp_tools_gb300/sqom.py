"""Host-side mirror of mp_sqom's operator interface for the S(Q,omega) path.

``QGrid`` restates the Q-grid geometry of mp_sqom (code/src/mp_sqom56.f90:764-936): plane
vectors, phase scales tpe, pixel counts n_qx/n_qy (even), Q centre, the 1/|Q| table and the
physical-Q vectors the X-ray form factors use — in FP32 where the reference stores real(4).
The optional third axis (ndim=3) extends the plane to a volume along ev with the same rules.

``TimeAxis`` restates the time constants (:680-704) and windows (:941-948).

``SqomJob`` drives libmpsq's job API: trajectory upload, the frame loop on the GPU, and the
maps of plot_loop (total S(Q), E=const, E(Q) dispersion) plus the whole-run Gaussian spectrum,
normalised as the reference normalises them (:1527, :1573-1576).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import check, ptr

TWOPI = 2.0 * np.pi
f32 = np.float32


def _dot32(a, b):
    a = np.asarray(a, f32)
    b = np.asarray(b, f32)
    s = f32(0)
    for i in range(3):
        s = f32(s + f32(a[i] * b[i]))
    return s


def _norm32(a):
    return f32(np.sqrt(_dot32(a, a)))


def _matvec32(m, v):
    m = np.asarray(m, f32)
    return np.array([_dot32(m[i], v) for i in range(3)], f32)


@dataclass
class QGrid:
    """Q grid of one map (mp_sqom56.f90:764-936)."""
    input_method: int                 # _lib.CELL or _lib.BULK
    n_row: tuple                      # supercell (1,1,1 for BULK boxes)
    e1: tuple = (1, 0, 0)
    e2: tuple = (0, 1, 0)
    n_bz: float = 1.0                 # Brillouin zones (CELL) or Q-range in 1/A (BULK)
    q_center: tuple = (0.0, 0.0, 0.0)
    a_par: tuple = (1.0, 1.0, 1.0)
    a_cell_inv: np.ndarray | None = None
    ndim: int = 2
    at_pos_min: tuple | None = None
    at_pos_max: tuple | None = None
    at_pos_centre: tuple = (0.0, 0.0, 0.0)

    def __post_init__(self):
        n_row = np.asarray(self.n_row, np.int64)
        self.nsuper = int(np.prod(n_row))
        a_par = np.asarray(self.a_par, f32)
        if self.at_pos_min is None:
            if self.nsuper == 1:
                self.at_pos_min = tuple(-a_par / 2)
                self.at_pos_max = tuple(a_par / 2)
            else:
                self.at_pos_min = tuple((-n_row / 2.0).astype(f32))
                self.at_pos_max = tuple((n_row / 2.0).astype(f32))
        if self.a_cell_inv is None:
            # CELL: reciprocal of the orthogonal cell (:529-534 without data_header_3);
            # BULK boxes: the identity that BULK .dat headers carry (positions in Angstrom).
            self.a_cell_inv = (np.diag(1.0 / a_par) if self.nsuper > 1 else np.eye(3)).astype(f32)
        e1 = np.asarray(self.e1, f32)
        e2 = np.asarray(self.e2, f32)
        ev = np.array([e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                       e1[0] * e2[1] - e1[1] * e2[0]], f32)
        self.e1_norm, self.e2_norm, self.ev_norm = _norm32(e1), _norm32(e2), _norm32(ev)
        e1n = (e1 / self.e1_norm).astype(f32)
        e2n = (e2 / self.e2_norm).astype(f32)
        evn = (ev / self.ev_norm).astype(f32)
        self.axis = np.stack([e1n, e2n, evn])
        span = (np.asarray(self.at_pos_max, f32) - np.asarray(self.at_pos_min, f32)).astype(f32)
        # tpe = twopi (real 8) / real(4) dot product, stored as real(4) (:809-811); the plane
        # normal's scale is unused by a 2D map (the reference divides by zero there for
        # e.g. (hhl) planes of a cubic box)
        spans = [float(_dot32(a, span)) for a in self.axis]
        if any(s == 0.0 for s in spans[:self.ndim]):
            raise ValueError("box has zero extent along a Q axis: choose other plane vectors")
        self.tpe = np.array([f32(TWOPI / s) if s != 0.0 else f32(0.0) for s in spans], f32)
        scale = TWOPI if self.nsuper > 1 else 1.0
        self.ep = np.stack([(scale * _matvec32(self.a_cell_inv, a).astype(np.float64)).astype(f32)
                            for a in self.axis])
        e1p_n, e2p_n = _norm32(self.ep[0]), _norm32(self.ep[1])
        self.evp_norm = _norm32(self.ep[2])
        cos_ep = f32(_dot32(self.ep[0], self.ep[1]) / (e1p_n * e1p_n))
        bz_n = f32(self.n_bz)
        if self.nsuper > 1:
            bz_ny = max(bz_n, f32(bz_n * (e1p_n / (e2p_n * f32(np.sqrt(f32(1.0) - cos_ep ** 2))))))
            bz_nx = f32(bz_n + bz_ny * abs(cos_ep)) if abs(cos_ep) > 0 else bz_n
            bz_nz = bz_n
            n = [int(TWOPI * float(b) / float(t)) if t != 0 else 1
                 for b, t in zip((bz_nx, bz_ny, bz_nz), self.tpe)]
        else:
            bz_nx = bz_ny = bz_nz = bz_n
            n = [int(f32(b / t)) if t != 0 else 1 for b, t in zip((bz_nx, bz_ny, bz_nz), self.tpe)]
        n = [k + 1 if (k > 1 and k % 2) else k for k in n]
        n = [max(1, k) for k in n]
        if self.ndim == 2:
            n[2] = 1
        self.n_q = tuple(n)
        self.bz = np.array([bz_nx, bz_ny, bz_nz], f32)
        qc = np.asarray(self.q_center, f32)
        norms = (self.e1_norm, self.e2_norm, self.ev_norm)
        centre = np.array([f32(_dot32(self.axis[k], qc) / norms[k]) for k in range(3)], f32)
        self.q_min = np.array([centre[k] - f32(0.5) * self.bz[k] if self.n_q[k] > 1 else centre[k]
                               for k in range(3)], f32)
        self.dq = np.array([f32(self.bz[k] / self.n_q[k]) for k in range(3)], f32)
        self.q_v = (centre[2] * evn).astype(f32)  # out-of-plane part of q_center (:900)
        self.q_vp = (f32(_dot32(self.ep[2], qc) / self.evp_norm) * self.ep[2]).astype(f32)

    @property
    def shape(self):
        """Array shape of a map, slowest axis first: (n_qz, n_qy, n_qx)."""
        return (self.n_q[2], self.n_q[1], self.n_q[0])

    @property
    def n_modes(self) -> int:
        return int(np.prod(self.n_q))

    def axis_values(self, k):
        """Q coordinate along axis k of pixel i = 0..n-1 (r.l.u. or 1/A)."""
        return (self.q_min[k] + np.arange(self.n_q[k], dtype=f32) * self.dq[k]).astype(f32)

    def q2_norm(self) -> np.ndarray:
        """1/|Q| table (:904-917), Q in r.l.u. (CELL) or 1/A (BULK); flattened, x fastest."""
        qx, qy = self.axis_values(0), self.axis_values(1)
        q = (qx[None, None, :, None] * self.axis[0][None, None, None, :]
             + qy[None, :, None, None] * self.axis[1][None, None, None, :])
        if self.ndim == 3:
            qz = self.axis_values(2)
            q = q + qz[:, None, None, None] * self.axis[2][None, None, None, :]
            extra = f32(0)
        else:
            extra = _dot32(self.q_v, self.q_v)
        qsq = (q.astype(f32) ** 2).sum(-1).astype(f32) + extra
        out = np.where(qsq >= 1e-8, 1.0 / np.sqrt(np.maximum(qsq, 1e-30)), 1.0).astype(f32)
        return out.reshape(-1)

    def qphys(self):
        """(origin, steps[3], extra_sq) with Q_phys(k) = origin + sum_a k_a steps[a] for mode k
        (k_a = i_a - n_a/2) — the vector mp_sqom feeds to the form factors (:919-931)."""
        origin = np.zeros(3, np.float64)
        steps = np.zeros((3, 3), np.float64)
        for k in range(self.ndim):
            origin += float(self.q_min[k] + (self.n_q[k] // 2) * self.dq[k]) * self.ep[k].astype(np.float64)
            steps[k] = float(self.dq[k]) * self.ep[k].astype(np.float64)
        extra = float(_dot32(self.q_vp, self.q_vp)) if self.ndim == 2 else 0.0
        return origin, steps, extra


@dataclass
class TimeAxis:
    """Time constants and Hann window (mp_sqom56.f90:680-704, :941-948)."""
    nfile: int
    t_step: float
    n_int: int = 0
    j_sq: int = 1

    def __post_init__(self):
        if self.n_int == 0:
            self.n_int = self.nfile // 2
        if self.j_sq == 1 and self.n_int % 2 == 0:
            self.n_int += 1
        self.n_int = max(1, min(self.n_int, self.nfile))
        self.freq_step = 1.0 / ((self.n_int - 1) * self.t_step) if self.n_int > 1 else 0.0
        self.n_freq_max = (self.n_int - 1) // 2 + 1
        self.n_frame = self.nfile - self.n_int + 1

    def window(self) -> np.ndarray:
        if self.n_int <= 1:
            return np.ones(self.n_int, f32)
        i = np.arange(1, self.n_int + 1, dtype=np.float64)
        return (0.5 * (1.0 - np.cos(TWOPI * (i - 1) / (self.n_int - 1)))).astype(f32)


class SqomJob:
    """One S(Q,omega) job on the GPU (device-resident trajectory, amplitudes and grids)."""

    @staticmethod
    def describe(grid: QGrid, *, species_counts, n_frames: int, precision: int = _lib.FP32,
                 eps: float = 1e-6, weight_mode: int = _lib.WEIGHT_UNIT, b_coh=None, xff=None,
                 ff_convention: int = _lib.FF_MP_SQOM, mask=None, window: bool = False,
                 phase_rounding: bool = False, store_species: bool = False, no_pack: bool = False,
                 no_pruned_fft: bool = False, n_atoms_frame: int | None = None,
                 use_range: bool = False, eps_x: float = 0.1, stream_ordered: bool = False,
                 q_slab: int = 0):
        """The job descriptor (mpsq_job_desc) of these arguments, without creating the job
        (for estimate_bytes and admission control).  q_slab > 0 (3D): the amplitude store
        holds at most q_slab kz planes at a time (see set_q_slab)."""
        counts = [int(n) for n in species_counts]
        S = len(counts)
        if S < 1 or S > _lib.MAX_SPECIES:
            raise ValueError("1..16 species supported")
        d = _lib.JobDesc()
        d.ndim = grid.ndim
        d.precision = precision
        d.eps = eps
        for k in range(3):
            d.n_modes[k] = grid.n_q[k]
            d.tpe[k] = float(grid.tpe[k])
            d.centre[k] = float(grid.at_pos_centre[k])
            d.pos_min[k] = float(grid.at_pos_min[k])
            d.pos_max[k] = float(grid.at_pos_max[k])
            d.n_row[k] = int(grid.n_row[k])
            d.q_center[k] = float(grid.q_center[k])
            for b in range(3):
                d.axis[k][b] = float(grid.axis[k][b])
        d.input_method = grid.input_method
        d.phase_rounding = int(phase_rounding)
        d.use_range = int(use_range)
        d.eps_x = eps_x
        d.bulk_nsuper1 = int(grid.nsuper == 1)
        d.spatial_window = int(window)
        d.n_species = S
        off = np.concatenate([[0], np.cumsum(counts)])
        for s in range(S + 1):
            d.species_offset[s] = int(off[s])
        mask = [1] * S if mask is None else list(mask)
        for s in range(S):
            d.mask[s] = int(mask[s])
        d.weight_mode = weight_mode
        if b_coh is not None:
            for s in range(S):
                d.b_coh[s] = float(b_coh[s])
        if xff is not None:
            for s in range(S):
                for i in range(9):
                    d.xff[s][i] = float(xff[s][i])
        d.ff_convention = ff_convention
        origin, steps, extra = grid.qphys()
        for b in range(3):
            d.qphys_origin[b] = origin[b]
            for k in range(3):
                d.qphys_step[k][b] = steps[k][b]
        d.qphys_extra_sq = extra
        d.n_atoms_frame = int(n_atoms_frame if n_atoms_frame is not None else off[-1])
        d.n_frames = int(n_frames)
        d.store_species = int(store_species)
        d.no_pack = int(no_pack)
        d.no_pruned_fft = int(no_pruned_fft)
        # device memory from the stream-ordered pool: creating and closing the job never wait
        # for the device (many concurrent jobs, as in the request server)
        d.stream_ordered = int(stream_ordered)
        d.q_slab = int(q_slab)
        return d

    def __init__(self, grid: QGrid, *, species_counts, n_frames: int, precision: int = _lib.FP32,
                 eps: float = 1e-6, weight_mode: int = _lib.WEIGHT_UNIT, b_coh=None, xff=None,
                 ff_convention: int = _lib.FF_MP_SQOM, mask=None, window: bool = False,
                 phase_rounding: bool = False, store_species: bool = False, no_pack: bool = False,
                 no_pruned_fft: bool = False,
                 n_atoms_frame: int | None = None, use_range: bool = False, eps_x: float = 0.1,
                 stream: int | None = None, stream_ordered: bool = False, q_slab: int = 0):
        L = _lib.load()
        self.grid = grid
        self.species_counts = [int(n) for n in species_counts]
        d = SqomJob.describe(grid, species_counts=species_counts, n_frames=n_frames,
                             precision=precision, eps=eps, weight_mode=weight_mode, b_coh=b_coh,
                             xff=xff, ff_convention=ff_convention, mask=mask, window=window,
                             phase_rounding=phase_rounding, store_species=store_species,
                             no_pack=no_pack, no_pruned_fft=no_pruned_fft,
                             n_atoms_frame=n_atoms_frame, use_range=use_range, eps_x=eps_x,
                             stream_ordered=stream_ordered, q_slab=q_slab)
        self.desc = d
        self.q_slab = min(int(q_slab), grid.n_q[2]) if q_slab else 0
        self.slab_z0 = 0
        self.n_frames = int(n_frames)
        self.n_atoms_frame = d.n_atoms_frame
        self.precision = precision
        self._h = C.c_void_p()
        self._stream = int(stream or 0)
        self._copy_stream = None
        self._d2h_stream = None      # output copies to host torch tensors
        self._d2h_done = None
        self._pending_out = []       # (device buffer, host tensor, ready event) not yet issued
        self._stage = {}             # device staging buffers of those outputs
        check(L.mpsq_job_create(C.byref(d), C.c_void_p(stream or 0), C.byref(self._h)), "job_create")

    # ------------------------------------------------------------------ lifecycle
    def close(self):
        if self._h:
            if self._pending_out:            # owed copies of outputs to host tensors
                self._flush_outputs()
            if self._d2h_done is not None:
                self._d2h_done.synchronize()
            _lib.load().mpsq_job_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @staticmethod
    def estimate_bytes(desc) -> int:
        b = C.c_int64()
        check(_lib.load().mpsq_job_estimate_bytes(C.byref(desc), C.byref(b)), "estimate_bytes")
        return int(b.value)

    # ------------------------------------------------------------------ inputs
    def set_frames(self, pos, first: int = 0):
        """pos: (count, n_atoms_frame, 4) float32 — numpy array, torch CPU tensor (pinned memory
        is copied by DMA without staging) or torch CUDA tensor."""
        if hasattr(pos, "is_cuda"):          # torch tensor: use its own buffer, no host copy
            import torch
            if pos.dtype != torch.float32 or not pos.is_contiguous():
                pos = pos.to(torch.float32).contiguous()
            host = not pos.is_cuda
        else:
            host = True
            pos = np.ascontiguousarray(pos, dtype=np.float32)
        count = pos.shape[0] if pos.ndim == 3 else 1
        if pos.shape[-2] != self.n_atoms_frame or pos.shape[-1] != 4:
            raise ValueError("frames must be (count, n_atoms_frame, 4)")
        check(_lib.load().mpsq_job_set_frames(self._h, C.c_void_p(ptr(pos)), first, count, int(host)),
              "set_frames")
        self._keep = pos  # keep host memory alive until the copy is ordered

    def set_cell_index(self, at_ind):
        a = np.ascontiguousarray(at_ind, dtype=np.int32)
        check(_lib.load().mpsq_job_set_cell_index(self._h, C.c_void_p(ptr(a)), 1), "set_cell_index")
        self.sync()

    # ------------------------------------------------------------------ compute
    def transform_from_host(self, frames, chunk: int = 32, first_chunk: int = 4):
        """Uploads host frames (count = n_frames; a pinned torch CPU tensor copies by DMA) in
        chunks of `chunk` frames (the first one `first_chunk` frames, to start computing
        early) on a second CUDA stream and transforms every chunk on the job's stream as soon
        as it has arrived, so the upload of chunk c+1 overlaps the transform of chunk c.
        The first call's uploads start after all work already queued on the job's stream;
        a later call with the same chunking uploads each chunk as soon as the previous call has
        transformed that chunk, so it overlaps the previous call's remaining work."""
        import torch
        if hasattr(frames, "is_cuda"):
            if frames.is_cuda:
                raise ValueError("transform_from_host takes host frames")
            if frames.dtype != torch.float32 or not frames.is_contiguous():
                frames = frames.to(torch.float32).contiguous()
            base = frames.data_ptr()
        else:
            frames = np.ascontiguousarray(frames, dtype=np.float32)
            base = frames.ctypes.data
        F = frames.shape[0]
        if F != self.n_frames or frames.shape[1] != self.n_atoms_frame:
            raise ValueError("frames must be (n_frames, n_atoms_frame, 4)")
        L = _lib.load()
        job_stream = (torch.cuda.ExternalStream(self._stream) if self._stream
                      else torch.cuda.default_stream())
        if self._copy_stream is None:
            self._copy_stream = torch.cuda.Stream()
        cs = self._copy_stream
        frame_bytes = self.n_atoms_frame * 16
        bounds = [0] + list(range(min(max(1, first_chunk), F), F, chunk)) + [F]
        # A chunk's frames may be overwritten once the previous call has transformed them (the
        # transform reads positions only while binning; the maps read the amplitude store), so
        # with the same chunking each upload waits for that chunk's transform of the previous
        # call instead of for everything queued on the job's stream: the next call's uploads
        # run while this call still computes.
        prev = self._chunk_done if getattr(self, "_chunk_bounds", None) == bounds else None
        if prev is None:
            tail = torch.cuda.Event()
            tail.record(job_stream)
            cs.wait_event(tail)
        done = []
        for i, (c0, c1) in enumerate(zip(bounds[:-1], bounds[1:])):
            n = c1 - c0
            if prev is not None:
                cs.wait_event(prev[i])
            check(L.mpsq_job_set_frames_on(self._h, C.c_void_p(base + c0 * frame_bytes), c0, n, 1,
                                           C.c_void_p(cs.cuda_stream)), "set_frames_on")
            ev = torch.cuda.Event()
            ev.record(cs)
            job_stream.wait_event(ev)
            self.transform(c0, n)
            consumed = torch.cuda.Event()
            consumed.record(job_stream)
            done.append(consumed)
        self._chunk_bounds, self._chunk_done = bounds, done
        # copies of earlier outputs to the host go after the uploads, on the same stream
        self._flush_outputs(cs)
        # host memory stays alive until its copies are ordered: this call's and, as the next
        # call's uploads no longer wait for the whole stream, the previous call's
        self._keep_prev = getattr(self, "_keep", None)
        self._keep = frames

    def transform(self, first: int = 0, count: int | None = None):
        count = self.n_frames - first if count is None else count
        check(_lib.load().mpsq_job_transform(self._h, first, count), "transform")

    def transform_onephonon(self, j_plane: int, at_base, first: int = 0, count: int | None = None):
        """One-phonon amplitudes instead of the NUFFT (mp_sqom's j_oneph = 1,
        code/src/mp_sqom56.f90:1037-1098) for frames [first, first+count): j_plane 1 = (hk0),
        2 = (hhl); at_base (n_species, 3) basis positions in cells (the frame header's at_base).
        CELL input on a Q plane, cell indices set (set_cell_index)."""
        g = self.grid
        count = self.n_frames - first if count is None else count
        base = np.ascontiguousarray(np.asarray(at_base, f32).reshape(-1, 3))
        if base.shape[0] != len(self.species_counts):
            raise ValueError(f"at_base: {base.shape[0]} rows for {len(self.species_counts)} species")
        check(_lib.load().mpsq_job_transform_onephonon(
            self._h, first, count, int(j_plane), int(round(float(g.n_bz))), float(g.q_min[0]),
            float(g.q_min[1]), C.c_void_p(base.ctypes.data)), "transform_onephonon")

    def info(self) -> dict:
        """Spreading width, fine-grid lengths, number of fine grids per frame, whether the
        pruned three-pass transform runs, and the number of frame lanes."""
        w, ng, pr, ln = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        nf = (C.c_int64 * 3)()
        check(_lib.load().mpsq_job_info(self._h, C.byref(w), nf, C.byref(ng), C.byref(pr),
                                        C.byref(ln)), "info")
        return {"width": w.value, "fine_grid": tuple(nf), "n_grids": ng.value,
                "pruned": bool(pr.value), "lanes": ln.value}

    def n_grids(self) -> int:
        return self.info()["n_grids"]

    def set_option(self, option: int, value: int):
        """Run-time choice (_lib.OPT_GRAPH, OPT_SPREAD, OPT_XROWS, OPT_LANES, OPT_ZSLAB); see
        mpsq.h."""
        check(_lib.load().mpsq_job_set_option(self._h, int(option), int(value)), "set_option")

    def get_option(self, option: int) -> int:
        v = C.c_int()
        check(_lib.load().mpsq_job_get_option(self._h, int(option), C.byref(v)), "get_option")
        return v.value

    def autotune(self, first: int = 0, count: int | None = None, cache: str | None = None) -> dict:
        """Times the transform of frames [first, first + count) under every applicable
        combination of run-time choices, keeps the fastest (see mpsq_job_autotune); cache: a
        file of recorded choices per job shape."""
        count = min(self.n_frames - first, 8) if count is None else count
        ch = (C.c_int * 4)()
        ms = C.c_double()
        check(_lib.load().mpsq_job_autotune(self._h, int(first), int(count),
                                            cache.encode() if cache else None, ch, C.byref(ms)),
              "autotune")
        return {"graph": ch[0], "spread": ("tensor-core", "cuda-core")[ch[1]], "xrows": ch[2],
                "lanes": ch[3], "zslab": self.get_option(_lib.OPT_ZSLAB),
                "ms_per_call": ms.value, "frames_per_call": count}

    @property
    def slab_planes(self) -> int:
        """kz planes the amplitude store holds now (all of them without a q_slab)."""
        nz = self.grid.n_q[2]
        return min(self.q_slab, nz - self.slab_z0) if self.q_slab else nz

    @property
    def store_modes(self) -> int:
        """Q modes per frame in the amplitude store and in every map (the current slab's)."""
        return self.grid.n_q[0] * self.grid.n_q[1] * self.slab_planes

    def set_q_slab(self, z0: int):
        """Selects the kz planes [z0, z0 + q_slab) (clipped) for the next transforms and maps;
        their outputs cover Q indices z0 * n_qx * n_qy onward of the full grid."""
        check(_lib.load().mpsq_job_set_q_slab(self._h, int(z0)), "set_q_slab")
        self.slab_z0 = int(z0)

    def slabs(self):
        """(z0, planes, first flat Q index) of every slab, in order (one slab without q_slab)."""
        nz = self.grid.n_q[2]
        step = self.q_slab or nz
        plane = self.grid.n_q[0] * self.grid.n_q[1]
        return [(z0, min(step, nz - z0), z0 * plane) for z0 in range(0, nz, step)]

    def uses_pruned_fft(self) -> bool:
        return self.info()["pruned"]

    def sync(self):
        self._flush_outputs()
        check(_lib.load().mpsq_job_sync(self._h), "sync")
        if self._d2h_done is not None:
            self._d2h_done.synchronize()

    def _torch_stream(self):
        import torch
        return torch.cuda.ExternalStream(self._stream) if self._stream else torch.cuda.default_stream()

    def _target(self, out, key, shape):
        """Where an output is computed: (pointer, host flag for the C call, host torch tensor
        to copy to afterwards or None).  A host torch tensor (pinned for a real overlap) is
        filled from a device staging buffer by an asynchronous copy on another stream that
        overlaps whatever the job's stream runs next.  The copy is issued by the next
        transform_from_host after its uploads (so that the two directions do not share the
        host link while the transform waits for its frames), or by sync() / wait_outputs()."""
        if out is None or not hasattr(out, "is_cuda"):
            return out, 1, None
        if out.is_cuda:
            return out, 0, None
        import torch
        dev = self._stage.get(key)
        if dev is None or tuple(dev.shape) != tuple(shape):
            dev = torch.empty(shape, dtype=torch.float32, device="cuda")
            self._stage[key] = dev
        if any(p[0].data_ptr() == dev.data_ptr() for p in self._pending_out):
            self._flush_outputs()               # the buffer's earlier content is still owed
        if self._d2h_done is not None:          # the previous copy out of the buffer
            self._torch_stream().wait_event(self._d2h_done)
        return dev, 0, out

    def _copy_out(self, dev, host):
        import torch
        ready = torch.cuda.Event()
        ready.record(self._torch_stream())
        self._pending_out.append((dev, host, ready))

    def _flush_outputs(self, stream=None):
        """Issues the owed output copies on `stream` (default: the job's output stream)."""
        if not self._pending_out:
            return
        import torch
        if stream is None:
            if self._d2h_stream is None:
                self._d2h_stream = torch.cuda.Stream()
            stream = self._d2h_stream
        with torch.cuda.stream(stream):
            for dev, host, ready in self._pending_out:
                stream.wait_event(ready)
                host.copy_(dev.view(host.shape), non_blocking=True)
        self._pending_out = []
        self._d2h_done = torch.cuda.Event()
        self._d2h_done.record(stream)

    def wait_outputs(self):
        """Issues the owed copies of outputs to host tensors and makes the job's stream wait
        for them, on the device (no host synchronisation)."""
        self._flush_outputs()
        if self._d2h_done is not None:
            self._torch_stream().wait_event(self._d2h_done)

    def profile(self, enable: bool = True):
        check(_lib.load().mpsq_job_profile(self._h, int(enable)), "profile")

    def stage_ms(self, reset: bool = False):
        """Accumulated [bin, spread, fft, deconv] milliseconds and frames timed."""
        ms = (C.c_double * 4)()
        fr = C.c_int64()
        check(_lib.load().mpsq_job_stage_ms(self._h, ms, C.byref(fr), int(reset)), "stage_ms")
        return list(ms), int(fr.value)

    def radial_hist(self, a_cell_inv, d_q, q_step: float, q_range: float, n_hist: int,
                    amp_scale: float = 1.0) -> np.ndarray:
        """Sum over frames and modes of Re(A_a conj A_b) binned by nint(|Q|/q_step) with
        Q = a_cell_inv (k * d_q) (mp_sql's Gauss integration); returns
        (n_species, n_species, n_hist)."""
        S = len(self.species_counts) if self.desc.store_species else 1
        out = np.zeros(S * S * n_hist, np.float64)
        a = np.ascontiguousarray(np.asarray(a_cell_inv, np.float64).reshape(9))
        d = np.ascontiguousarray(np.asarray(d_q, np.float64).reshape(3))
        check(_lib.load().mpsq_job_radial_hist(self._h, C.c_void_p(ptr(a)), C.c_void_p(ptr(d)),
                                               float(q_step), float(q_range), int(n_hist),
                                               float(amp_scale), C.c_void_p(ptr(out)), 1),
              "radial_hist")
        return out.reshape(S, S, n_hist)

    def amplitudes_ptr(self) -> int:
        p = C.c_void_p()
        check(_lib.load().mpsq_job_amplitudes(self._h, C.byref(p)), "amplitudes")
        return int(p.value or 0)

    def amplitudes(self) -> np.ndarray:
        """cs(t,Q) copied to the host, shape (n_frames, n_Q), complex64/complex128."""
        import torch
        n = self.n_frames * self.store_modes
        dt = torch.complex128 if self.precision == _lib.FP64 else torch.complex64
        out = torch.empty(n, dtype=dt)
        self.sync()
        src = self.amplitudes_ptr()
        nbytes = out.element_size() * n
        cudart = _cudart()
        check_rt(cudart.cudaMemcpy(C.c_void_p(out.data_ptr()), C.c_void_p(src), C.c_size_t(nbytes), 2),
                 "cudaMemcpy")
        return out.numpy().reshape(self.n_frames, -1)

    def amplitudes_device(self):
        """cs(t,Q) as a torch tensor (n_frames, n_Q) viewing the job's device store (no copy;
        valid until the job is closed, rewritten by the next transform)."""
        import torch
        dt = "<c16" if self.precision == _lib.FP64 else "<c8"

        class _View:
            __cuda_array_interface__ = {"shape": (self.n_frames, self.store_modes), "typestr": dt,
                                        "data": (self.amplitudes_ptr(), False), "version": 3}

        self.sync()
        return torch.as_tensor(_View(), device="cuda")

    def amplitudes_at(self, q_index, frames=None) -> np.ndarray:
        """cs(t, Q) at the given flat Q indices (all frames, or the given frame indices), gathered
        on the device and copied to the host: (n_t, len(q_index))."""
        import torch
        cs = self.amplitudes_device()
        q = torch.as_tensor(np.asarray(q_index, np.int64), device="cuda")
        sel = cs if frames is None else cs[torch.as_tensor(np.asarray(frames, np.int64), device="cuda")]
        return sel[:, q].cpu().numpy()

    def norm2(self) -> float:
        return float(sum(self.species_counts)) ** 2

    def sq_total(self, normalize: bool = True, out=None, s_trig: float = 0.0) -> np.ndarray:
        """Total S(Q) = <|cs|^2>_t / (sum N_j)^2 (:1381-1387, :1573-1574); s_trig > 0 applies
        the speckle filter before the (sum N)^2 norm (:1531-1570, plane grids)."""
        n2 = self.norm2() if normalize else 1.0
        res, host, copy_to = self._target(out, "sq", (self.store_modes,))
        if res is None:
            res = np.empty(self.store_modes, f32)
        if s_trig > 0:
            self._plane_shape("speckle filter")
            check(_lib.load().mpsq_job_sq_total(self._h, 1.0, C.c_void_p(ptr(res)), int(host)), "sq_total")
            res = self._speckle(res, s_trig, False, 1.0 / n2, host)
        else:
            check(_lib.load().mpsq_job_sq_total(self._h, n2, C.c_void_p(ptr(res)), int(host)), "sq_total")
        if copy_to is not None:
            self._copy_out(res, copy_to)
            return copy_to
        return res

    def _plane_shape(self, what):
        if self.grid.n_q[2] != 1:
            raise ValueError(f"{what}: defined on plane (2D) Q grids only, got {self.grid.n_q}")
        return self.grid.n_q[1], self.grid.n_q[0]

    def _speckle(self, res, s_trig, dispersion, post_scale, host=True):
        """Speckle filter (:1531-1570) of a map in place, then the remaining normalisation."""
        n_slow, n_fast = res.shape if dispersion else self._plane_shape("speckle filter")
        check(_lib.load().mpsq_speckle_filter(C.c_void_p(ptr(res)), int(n_fast), int(n_slow),
                                              float(s_trig), int(not dispersion), float(post_scale),
                                              int(host), C.c_void_p(self._stream or None)),
              "speckle_filter")
        return res

    def sqw_econst(self, taxis: TimeAxis, j_freq: int, q2_norm=None, normalize=True,
                   t_wind=None, atom_pair=None, s_trig: float = 0.0, out=None) -> np.ndarray:
        """E=const map for 1-based bin j_freq (:1437-1478), normalised as :1527, :1575-1576.
        atom_pair=(a, b): the map of the raw amplitudes of species a + b (0-based; :1460-1464;
        needs store_species), where q2_norm does not apply.  s_trig > 0: speckle filter
        (:1531-1570) between the two normalisations, as the reference applies it.  out: a
        device tensor, or a host tensor filled asynchronously (see sq_total)."""
        w = np.ascontiguousarray(taxis.window() if t_wind is None else t_wind, f32)
        q2 = None if q2_norm is None else np.ascontiguousarray(q2_norm, f32)
        scale = 1.0 / (0.5 * taxis.n_frame * taxis.n_int)
        post = taxis.t_step / self.norm2() if normalize else 1.0
        if s_trig > 0:
            self._plane_shape("speckle filter")
        else:
            scale *= post
        res, host, copy_to = self._target(out, "econst", (self.store_modes,))
        if res is None:
            res = np.empty(self.store_modes, f32)
        L = _lib.load()
        if atom_pair is None:
            check(L.mpsq_job_sqw_econst(self._h, taxis.n_int, C.c_void_p(ptr(w)), j_freq,
                                        C.c_void_p(ptr(q2)), scale, C.c_void_p(ptr(res)), host),
                  "sqw_econst")
        else:
            check(L.mpsq_job_sqw_econst_pair(self._h, taxis.n_int, C.c_void_p(ptr(w)), j_freq,
                                             int(atom_pair[0]), int(atom_pair[1]), scale,
                                             C.c_void_p(ptr(res)), host), "sqw_econst_pair")
        if s_trig > 0:
            res = self._speckle(res, s_trig, False, post, bool(host))
        if copy_to is not None:
            self._copy_out(res, copy_to)
            return copy_to
        return res

    def sqw_dispersion(self, taxis: TimeAxis, q_index, n_freq=None, q2_norm=None,
                       normalize=True, t_wind=None, atom_pair=None, s_trig: float = 0.0) -> np.ndarray:
        """E(Q) cut along pixel indices q_index (:1480-1517); returns (n_path, n_freq).
        atom_pair=(a, b): the cut of the raw amplitudes of species a + b (:1494-1499).
        s_trig > 0: speckle filter along the frequencies (:1531-1548)."""
        w = np.ascontiguousarray(taxis.window() if t_wind is None else t_wind, f32)
        qi = np.ascontiguousarray(q_index, np.int64)
        n_freq = taxis.n_freq_max if n_freq is None else n_freq
        q2 = None if q2_norm is None else np.ascontiguousarray(q2_norm, f32)
        scale = 1.0 / (0.5 * taxis.n_frame * taxis.n_int)
        post = taxis.t_step / self.norm2() if normalize else 1.0
        if not s_trig > 0:
            scale *= post
        res = np.empty((len(qi), n_freq), f32)
        L = _lib.load()
        if atom_pair is None:
            check(L.mpsq_job_sqw_dispersion(self._h, taxis.n_int, C.c_void_p(ptr(w)), len(qi),
                                            C.c_void_p(ptr(qi)), n_freq, C.c_void_p(ptr(q2)),
                                            scale, C.c_void_p(ptr(res)), 1), "sqw_dispersion")
        else:
            check(L.mpsq_job_sqw_dispersion_pair(self._h, taxis.n_int, C.c_void_p(ptr(w)), len(qi),
                                                 C.c_void_p(ptr(qi)), n_freq, int(atom_pair[0]),
                                                 int(atom_pair[1]), scale, C.c_void_p(ptr(res)), 1),
                  "sqw_dispersion_pair")
        return self._speckle(res, s_trig, True, post) if s_trig > 0 else res

    def iqt(self, n_int: int, lag: int, q2_norm=None, normalize=True,
            s_trig: float = 0.0) -> np.ndarray:
        """I(Q,t) map at a time lag of `lag` frames (the j_sq /= 1 branch, :1467-1472),
        normalised by (sum N)^2 (:1573-1574); s_trig > 0: speckle filter before the norm."""
        q2 = None if q2_norm is None else np.ascontiguousarray(q2_norm, f32)
        post = 1.0 / self.norm2() if normalize else 1.0
        if s_trig > 0:
            self._plane_shape("speckle filter")
        scale = 1.0 if s_trig > 0 else post
        res = np.empty(self.store_modes, f32)
        check(_lib.load().mpsq_job_iqt(self._h, int(n_int), int(lag), C.c_void_p(ptr(q2)), scale,
                                       C.c_void_p(ptr(res)), 1), "iqt")
        return self._speckle(res, s_trig, False, post) if s_trig > 0 else res

    def iqt_dispersion(self, n_int: int, q_index, q2_norm=None, normalize=True,
                       s_trig: float = 0.0) -> np.ndarray:
        """I(Q,t) along pixel indices q_index for lags 0..n_frames-n_int (:1504-1510, :699);
        returns (n_path, n_frames - n_int + 1); s_trig > 0: speckle filter along the lags."""
        qi = np.ascontiguousarray(q_index, np.int64)
        q2 = None if q2_norm is None else np.ascontiguousarray(q2_norm, f32)
        post = 1.0 / self.norm2() if normalize else 1.0
        scale = 1.0 if s_trig > 0 else post
        res = np.empty((len(qi), self.n_frames - int(n_int) + 1), f32)
        check(_lib.load().mpsq_job_iqt_dispersion(self._h, int(n_int), len(qi), C.c_void_p(ptr(qi)),
                                                  C.c_void_p(ptr(q2)), scale, C.c_void_p(ptr(res)), 1),
              "iqt_dispersion")
        return self._speckle(res, s_trig, True, post) if s_trig > 0 else res

    def sqw_gauss(self, fwhm_frames=None, n_freq=None, t_step=1.0, q2_norm=None, normalize=True,
                  out=None) -> np.ndarray:
        """Whole-run Gaussian-window spectrum, (n_freq, n_Q); normalised by sum(g) * t_step /
        (sum N)^2 like the sliding-window maps."""
        F = self.n_frames
        fwhm = F / 2 if fwhm_frames is None else fwhm_frames
        n_freq = F // 2 + 1 if n_freq is None else n_freq
        g = np.exp(-4.0 * np.log(2.0) * ((np.arange(F) - 0.5 * (F - 1)) / fwhm) ** 2)
        scale = 1.0 / g.sum()
        if normalize:
            scale *= t_step / self.norm2()
        q2 = None if q2_norm is None else np.ascontiguousarray(q2_norm, f32)
        res, host, copy_to = self._target(out, "sqw", (n_freq, self.store_modes))
        if res is None:
            res = np.empty((n_freq, self.store_modes), f32)
        check(_lib.load().mpsq_job_sqw_gauss(self._h, float(fwhm), n_freq, C.c_void_p(ptr(q2)),
                                             scale, C.c_void_p(ptr(res)), int(host)), "sqw_gauss")
        if copy_to is not None:
            self._copy_out(res, copy_to)
            return copy_to
        return res


def speckle_filter(cs_plot, s_trig: float, dispersion: bool = False,
                   post_scale: float = 1.0) -> np.ndarray:
    """mp_sqom's speckle filter (code/src/mp_sqom56.f90:1531-1570) on the GPU, for a finished
    host map: a plane map as (n_qy, n_qx) (qx contiguous; two walks, the second over the
    transposed map) or an E(Q) / I(Q,t) cut as (n_path, n_freq) (dispersion=True; one walk
    along the frequencies).  Returns a new float32 array times post_scale."""
    m = np.array(cs_plot, dtype=f32, copy=True, order="C")
    if m.ndim != 2:
        raise ValueError(f"speckle filter: a 2D map is needed, got shape {m.shape}")
    check(_lib.load().mpsq_speckle_filter(C.c_void_p(m.ctypes.data), m.shape[1], m.shape[0],
                                          float(s_trig), int(not dispersion), float(post_scale),
                                          1, None), "speckle_filter")
    return m


_rt = None


def _cudart():
    global _rt
    if _rt is None:
        import glob
        import os
        cands = sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*"))
        _rt = C.CDLL(cands[0] if cands else "libcudart.so")
        _rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    return _rt


def check_rt(code, where):
    if code != 0:
        raise RuntimeError(f"{where}: cuda error {code}")
