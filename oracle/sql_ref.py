"""ORACLE — test infrastructure only (see oracle/__init__.py).

numpy restatement of MP_TOOLS mp_sql's spherical average, statement by statement, for the
golden-file check on the Al-U example:
  q-cube and d_q           code/src/mp_sql56.f90:975-1019
  |Q| of each mode         code/src/mp_sql56.f90:1041 (FP32, NORM2 scaled sum of squares)
  |Q| histogram (Gauss)    code/src/mp_sql56.f90:1224-1254  (amplitudes / sum(n_sup))
  normalisation            code/src/mp_sql56.f90:1276-1281
  smoothing                code/src/mp_sql56.f90:1366-1414
  X-ray output modes       code/src/mp_sql56.f90:1458-1503 (j_weight = 3)
  total and partials       code/src/mp_sql56.f90:1505-1521
"""
from __future__ import annotations

import numpy as np

import oracle

TWOPI = 2 * np.pi


def cube(q_range, box):
    """(n_qq, d_q) for a cubic BULK box with a_cell_inv = identity."""
    d_q = np.float32(TWOPI) / np.float32(box)
    bz = np.float32(2 * q_range)
    half = float(np.float32(0.5 * bz)) / float(d_q)
    n = 2 * int(np.floor(half + 0.5)) + 1
    return n, float(d_q)


def amplitudes(frame, lo, hi, n, d_q, eps=1e-9):
    """A(k) = sum_j exp(-i k . r_j d_q) for k in [-(n-1)/2, (n-1)/2]^3 (CPU ES NUFFT, FP64)."""
    r = np.asarray(frame[lo:hi, :3], np.float64)
    x = [r[:, a] * d_q for a in range(3)]
    return oracle.es_nufft(x, np.ones(len(r)), -1, eps, (n, n, n))


def norm2_scaled(x, y, z):
    """Fortran NORM2 of FP32 3-vectors as the scaled sum of squares (BLAS snrm2 recurrence),
    every operation rounded to FP32 (the q_norm of code/src/mp_sql56.f90:1041).  Bins of
    modes whose |Q|/q_step falls on a half-integer follow this rounding, not sqrt(x²+y²+z²)."""
    f32 = np.float32
    scale = np.zeros(np.shape(x), f32)
    ssq = np.ones(np.shape(x), f32)
    for c in (x, y, z):
        a = np.abs(np.asarray(c, f32))
        nz = a != 0
        up = nz & (scale < a)
        with np.errstate(divide="ignore", invalid="ignore"):
            r_up = (scale / np.where(up, a, f32(1))).astype(f32)
            r_dn = (a / np.where(scale > 0, scale, f32(1))).astype(f32)
            s_up = (f32(1) + (ssq * (r_up * r_up).astype(f32)).astype(f32)).astype(f32)
            s_dn = (ssq + (r_dn * r_dn).astype(f32)).astype(f32)
        ssq = np.where(up, s_up, np.where(nz, s_dn, ssq)).astype(f32)
        scale = np.where(up, a, scale).astype(f32)
    return (scale * np.sqrt(ssq)).astype(f32)


def q_norm(n, d_q, a_cell_inv=None):
    """|Q| of every mode of an n^3 cube, FP32 as code/src/mp_sql56.f90:1041:
    v = k * d_q, Q = a_cell_inv v (left-to-right sums), NORM2(Q)."""
    f32 = np.float32
    A = np.eye(3, dtype=f32) if a_cell_inv is None else np.asarray(a_cell_inv, f32)
    d = np.broadcast_to(np.asarray(d_q, f32), (3,))
    k = (np.arange(n) - n // 2).astype(f32)
    v = [np.broadcast_to((k * d[a]).astype(f32).reshape([n if b == a else 1 for b in range(3)]),
                         (n, n, n)) for a in range(3)]
    Q = []
    for r in range(3):
        acc = (A[r, 0] * v[0]).astype(f32)
        acc = (acc + (A[r, 1] * v[1]).astype(f32)).astype(f32)
        acc = (acc + (A[r, 2] * v[2]).astype(f32)).astype(f32)
        Q.append(acc)
    return norm2_scaled(*Q)


def histogram(amps, n, d_q, q_step, q_range, a_cell_inv=None):
    """sq_hist(a,b,bin) = sum over modes with |Q| <= q_range of Re(A_a conj A_b),
    bin = nint(|Q|/q_step) in FP32 (code/src/mp_sql56.f90:1236-1241); amps is a list of
    (n,n,n) arrays already divided by the total atom count."""
    f32 = np.float32
    qn = q_norm(n, d_q, a_cell_inv)
    sel = qn <= f32(q_range)
    ratio = (qn[sel] / f32(q_step)).astype(f32).astype(np.float64)
    bins = np.floor(ratio + 0.5).astype(np.int64)   # NINT of a positive FP32 value
    n_hist = 1 + int(f32(q_range) / f32(q_step))
    S = len(amps)
    out = np.zeros((S, S, n_hist))
    for a in range(S):
        for b in range(S):
            v = (amps[a][sel] * np.conj(amps[b][sel])).real
            out[a, b] = np.bincount(bins, weights=v, minlength=n_hist)[:n_hist]
    return out


def xray_total_and_partials(sq_hist, *, q_step, nfile, at_volume, occ, xff, mode, fwhm):
    """Modes 4 (S), 5 (Z), 6 (I), 7 (unscaled I) for X-ray weights and indistinguishable atoms
    (BULK boxes); returns (q, total, {(a,b): partial}) for the printed rows."""
    S, _, n_hist = sq_hist.shape
    occ = np.asarray(occ, float) / np.sum(occ)
    q = np.arange(n_hist) * float(np.float32(q_step))
    h = sq_hist.copy()
    for i in range(1, n_hist):
        h[:, :, i] = h[:, :, i] / (q_step * q[i] ** 2) * (2 * np.pi ** 2 / (nfile * at_volume))
    ns = 1 if fwhm == 1 else 5 * fwhm // 2 + 1
    f = np.array([2.0 ** (-((j - ns // 2 - 1) / (0.5 * fwhm)) ** 2) for j in range(1, ns + 1)])
    f = f / f.sum()
    start = int(0.5 / q_step)
    p = np.zeros_like(h)
    for i in range(start, n_hist + 1):
        if ns == 1:
            p[:, :, i - 1] = h[:, :, i - 1]
        else:
            for j in range(1, ns + 1):
                src = i - ns // 2 + j - 1
                if src <= 2:
                    continue
                p[:, :, i - 1] += (h[:, :, n_hist - j - 1] if src >= n_hist else h[:, :, src - 1]) * f[j - 1]
    p[:, :, :start] = 0.0
    x = np.zeros((S, n_hist))
    for s in range(S):
        qs = 0.25 * (q / TWOPI) ** 2
        x[s] = xff[s][8] + sum(xff[s][2 * m] * np.exp(-xff[s][2 * m + 1] * qs) for m in range(4))
    if mode == 5:
        for a in range(S):
            p[a, a] -= occ[a]
        for a in range(S):
            for b in range(S):
                p[a, b] /= occ[a] * occ[b]
    else:
        for i in range(start, n_hist + 1):
            xi = x[:, i - 1]
            av_sq = np.sum(occ * xi) ** 2
            sq_av = np.sum(occ * xi ** 2)
            for a in range(S):
                for b in range(S):
                    p[a, b, i - 1] *= xi[a] * xi[b]
            if mode == 6:
                p[:, :, i - 1] /= sq_av
            if mode < 5:
                for a in range(S):
                    p[a, a, i - 1] -= occ[a] * xi[a] ** 2
                    if mode == 4:
                        for b in range(S):
                            p[a, b, i - 1] += occ[a] * xi[a] * occ[b] * xi[b]
                p[:, :, i - 1] /= av_sq
    total = p.sum(axis=(0, 1)) if mode != 5 else None
    parts = {}
    for a in range(S):
        for b in range(a + 1):
            # off-diagonal partials are symmetrised except for Z(Q) (:1505-1521)
            parts[(a, b)] = p[a, b] + (p[b, a] if (a != b and mode != 5) else 0)
    first = start + ns // 2
    rows = slice(first - 1, n_hist)
    return q[rows], (None if total is None else total[rows]), {k: v[rows] for k, v in parts.items()}
