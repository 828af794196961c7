"""Spherically averaged scattering of MP_TOOLS mp_sql on the GPU NUFFT.

mp_sql builds the full 3D transform of each species (there as a stack of finufft2d1 slices
with z-phased strengths, code/src/mp_sql56.f90:1096-1135; here one 3D transform per species),
bins Re(A_a conj A_b) by |Q| (Gauss integration, :1224-1254), normalises the histogram
(:1264-1282), smooths it with a Gaussian (:1366-1414) and forms the output modes
(:1416-1503): S(Q) (mode 4), Faber-Ziman partials Z(Q) (5), I(Q) (6), unscaled I(Q) (7).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _lib
from .sqom import SqomJob

f32 = np.float32
TWOPI = 2.0 * np.pi
MODE_NAMES = {4: "S(Q)", 5: "Z(Q)", 6: "I(Q)", 7: "I(Q)"}


def _nint(x) -> int:
    """Fortran NINT (round half away from zero)."""
    return int(np.floor(abs(x) + 0.5)) * (1 if x >= 0 else -1)


@dataclass
class SqlGrid:
    """Q cube of mp_sql (code/src/mp_sql56.f90:975-1044): odd pixel counts n_qq, centred modes,
    phase steps d_q = 2 pi / box, |Q| = |a_cell_inv (k d_q)|."""
    q_range: float
    a_par: tuple
    n_row: tuple = (1, 1, 1)
    a_cell_inv: np.ndarray | None = None
    input_method: int = _lib.BULK

    def __post_init__(self):
        n_row = np.asarray(self.n_row, np.int64)
        a_par = np.asarray(self.a_par, f32)
        self.nsuper = int(np.prod(n_row))
        if self.nsuper == 1:
            span = a_par                                   # at_pos_max - at_pos_min (:955-958)
        else:
            span = n_row.astype(f32)
        if self.a_cell_inv is None:
            self.a_cell_inv = np.eye(3, dtype=f32) if self.nsuper == 1 else np.diag(1.0 / a_par).astype(f32)
        ai = np.asarray(self.a_cell_inv, f32)
        bz_n = f32(2.0 * self.q_range)
        e_r = [ai[:, k] for k in range(3)]
        cross = lambda u, v: np.array([u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2],
                                       u[0] * v[1] - u[1] * v[0]], f32)  # noqa: E731
        ev = [cross(e_r[1], e_r[2]), cross(e_r[2], e_r[0]), cross(e_r[0], e_r[1])]
        bz = [f32(bz_n / f32(np.dot(e_r[k], ev[k]) / np.linalg.norm(ev[k]))) for k in range(3)]
        self.d_q = (f32(TWOPI) / span).astype(f32)
        self.n_q = tuple(2 * _nint(float(f32(0.5 * bz[k]) / self.d_q[k])) + 1 for k in range(3))
        # attributes the job builder reads (identity axes, phase x = r * d_q, no centring)
        self.ndim = 3
        self.axis = np.eye(3, dtype=f32)
        self.tpe = self.d_q
        self.at_pos_centre = (0.0, 0.0, 0.0)
        self.at_pos_min = (-1e30,) * 3   # mp_sql transforms every atom
        self.at_pos_max = (1e30,) * 3
        self.q_center = (0.0, 0.0, 0.0)

    @property
    def n_modes(self) -> int:
        return int(np.prod(self.n_q))

    def qphys(self):
        return np.zeros(3), np.zeros((3, 3)), 0.0


def transform_histogram(frames, counts, grid: SqlGrid, q_step: float, *, precision=_lib.FP32,
                        eps=1e-6, stream=None) -> np.ndarray:
    """Runs the per-species 3D NUFFT of all frames on the GPU and returns the raw |Q|
    histogram sq_hist(a, b, bin) = sum_frames sum_{|Q| in bin} Re(A_a conj A_b), amplitudes
    divided by the total atom count (Gauss integration, :1224-1254)."""
    frames = np.asarray(frames, np.float32)
    F = frames.shape[0]
    n_hist = 1 + int(f32(grid.q_range) / f32(q_step))
    job = SqomJob(grid, species_counts=counts, n_frames=F, precision=precision, eps=eps,
                  store_species=True, n_atoms_frame=frames.shape[1], stream=stream)
    try:
        job.set_frames(frames)
        job.transform()
        job.sync()
        return job.radial_hist(grid.a_cell_inv, grid.d_q, q_step, grid.q_range, n_hist,
                               amp_scale=1.0 / float(sum(counts)))
    finally:
        job.close()


def xray_ff_hist(xff, q_hist):
    """Cromer-Mann f at the histogram bins, s = Q/(4 pi) (mp_sql56.f90:1046-1058)."""
    q_sq = (0.25 * (np.asarray(q_hist, np.float64) / TWOPI) ** 2)
    xff = np.asarray(xff, np.float64)
    f = np.full_like(q_sq, xff[8])
    for i in range(4):
        f = f + xff[2 * i] * np.exp(-xff[2 * i + 1] * q_sq)
    return f


def scattering_functions(sq_hist, *, q_step, nfile, at_volume, occ, mode, weight="xray",
                         xff=None, b_coh=None, mask=None, scf=None, n_smooth_fwhm=1,
                         indistinguishable=True):
    """Normalisation, smoothing and output mode of mp_sql.  Returns (q, total, partials) with
    partials[(a, b)] for a >= b (the off-diagonal ones symmetrised), rows from
    i_start = int(.5/q_step) + n_smooth/2 (1-based) as in the text output (:1760-1775)."""
    sq = np.array(sq_hist, np.float64, copy=True)
    S, _, n_hist = sq.shape
    occ = np.asarray(occ, np.float64)
    occ = occ / occ.sum()
    mask = np.ones(S) if mask is None else np.asarray(mask, np.float64)
    scf = np.ones(S) if scf is None else np.asarray(scf, np.float64)
    q_hist = np.arange(n_hist) * float(f32(q_step))
    # Gauss integral normalisation (:1276-1281), bins 2..n_hist
    sq[:, :, 1:] /= (q_step * q_hist[1:] ** 2)
    sq[:, :, 1:] *= 2.0 * np.pi ** 2 / (nfile * at_volume)
    # Gaussian smoothing (:1370-1414)
    ns = 1 if n_smooth_fwhm == 1 else (5 * n_smooth_fwhm) // 2 + 1
    j = np.arange(1, ns + 1)
    fs = 2.0 ** (-(((j - ns // 2 - 1) / (0.5 * n_smooth_fwhm)) ** 2))
    fs /= fs.sum()
    i0 = int(0.5 / q_step)            # first smoothed bin (1-based)
    plot = np.zeros_like(sq)
    for i in range(i0, n_hist + 1):   # 1-based bin
        if ns == 1:
            plot[:, :, i - 1] = sq[:, :, i - 1]
            continue
        for jj in range(1, ns + 1):
            idx = i - ns // 2 + jj - 1
            if idx <= 2:
                continue
            if idx >= n_hist:
                plot[:, :, i - 1] += sq[:, :, n_hist - jj - 1] * fs[jj - 1]
            else:
                plot[:, :, i - 1] += sq[:, :, idx - 1] * fs[jj - 1]
    plot[:, :, :i0] = 0.0
    if weight == "xray":
        X = np.stack([xray_ff_hist(xff[s], q_hist) for s in range(S)])  # (S, n_hist)
        if mode != 5:
            for i in range(i0, n_hist + 1):
                x = X[:, i - 1]
                w_av_sq = np.sum(occ * scf * x) ** 2
                w_sq_av = np.sum(occ * (scf * x ** 2))
                mw = mask * scf * x
                plot[:, :, i - 1] *= np.outer(mw, mw)
                if mode == 6:
                    plot[:, :, i - 1] /= w_sq_av
                if indistinguishable and mode < 5:
                    for a in range(S):
                        plot[a, a, i - 1] -= occ[a] * mask[a] * (scf[a] * x[a]) ** 2
                    if mode == 4:
                        plot[:, :, i - 1] += np.outer(occ * mask * scf * x, occ * mask * scf * x)
                    plot[:, :, i - 1] /= w_av_sq
        elif indistinguishable:
            for a in range(S):
                plot[a, a, :] -= occ[a]
            plot /= np.outer(occ, occ)[:, :, None]
    else:
        w = np.ones(S) if weight == "unit" else np.asarray(b_coh, np.float64)
        # averaged weights for mixed occupancies (:1350-1353); all atoms indistinguishable
        if indistinguishable:
            w = np.full(S, np.sum(w * occ) / np.sum(occ))
        w_sq_av = np.sum(occ * (scf * w) ** 2)
        w_av_sq = np.sum(occ * scf * w) ** 2
        if mode != 5:
            plot[:, :, i0 - 1:] *= (np.outer(w, w) * np.outer(mask * scf, mask * scf))[:, :, None]
            if mode == 6:
                plot /= w_sq_av
            if indistinguishable and mode < 5:
                for a in range(S):
                    plot[a, a, 1:] -= occ[a] * mask[a] * (scf[a] * w[a]) ** 2
                if mode == 4:
                    plot += (np.outer(occ * w, occ * w) * np.outer(mask * scf, mask * scf))[:, :, None]
                plot /= w_av_sq
        elif indistinguishable:
            for a in range(S):
                plot[a, a, :] -= occ[a]
            plot /= np.outer(occ, occ)[:, :, None]
    total = plot.sum(axis=(0, 1)) if mode != 5 else None
    parts = {}
    for a in range(S):
        for b in range(a + 1):
            # off-diagonal partials are symmetrised except for Z(Q) (:1505-1521)
            parts[(a, b)] = plot[a, b] + (plot[b, a] if (a != b and mode != 5) else 0.0)
    i_start = i0 + ns // 2
    rows = slice(i_start - 1, n_hist)
    return (q_hist[rows], None if total is None else total[rows],
            {k: v[rows] for k, v in parts.items()})
