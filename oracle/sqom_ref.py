"""ORACLE — test infrastructure only (see oracle/__init__.py).

numpy restatement of the loops of MP_TOOLS mp_sqom around the NUFFT call, each function citing
the reference lines it follows (paths relative to the MP_TOOLS tree):

  prep_points      code/src/mp_sqom56.f90:1100-1143  selection, phases x,y(,z), strengths
  weighted_sum     code/src/mp_sqom56.f90:1338-1377  species weights, elastic mean, 1/|Q|
  sq_total         code/src/mp_sqom56.f90:1381-1387  S(Q) = <|cs|^2>_t
  hann_window      code/src/mp_sqom56.f90:941-948    t_wind
  econst           code/src/mp_sqom56.f90:1437-1478  sliding-window E=const map
  dispersion       code/src/mp_sqom56.f90:1480-1517  E(Q) cut, FFT per start frame
  gauss_spectrum   whole-run Gaussian window + one DFT per Q (the benchmark's time transform)
  speckle_filter   code/src/mp_sqom56.f90:1531-1570  sequential speckle walk on a finished map
  one_phonon       code/src/mp_sqom56.f90:1037-1098  displacement-field (one-phonon) amplitudes
  xray_ff          code/src/mp_sqom56.f90:919-936 (and mp_sql56.f90:1048-1058 convention)
"""
from __future__ import annotations

import numpy as np


def prep_points(frame, lo, hi, *, input_method, ndim, axis, tpe, centre, q_center,
                window=False, phase_rounding=False, use_range=False, at_ind=None,
                n_row=(1, 1, 1), pos_min=None, pos_max=None, tol=0.1):
    """Points of one species (atoms lo..hi of frame, float32 (N,4)).  Returns the list of
    coordinate arrays (radians, FP64) and complex128 strengths, after the reference's
    selection: CELL skips atoms at exactly (0,0,0) (:1107) and, with use_range, cells outside
    [pos_min, pos_max] (:1108-1111); BULK keeps atoms within the box +- tol (:1121-1128)."""
    r = np.asarray(frame[lo:hi, :3], dtype=np.float32)
    keep = np.ones(len(r), bool)
    if input_method == 0:
        keep &= ~((r[:, 0] == 0) & (r[:, 1] == 0) & (r[:, 2] == 0))
        if use_range and at_ind is not None:
            ci = np.asarray(at_ind[lo:hi, :3]) - (np.asarray(n_row) // 2) - 1
            keep &= np.all((ci >= np.asarray(pos_min)) & (ci <= np.asarray(pos_max)), axis=1)
    else:
        pmin = np.asarray(pos_min, np.float32)
        pmax = np.asarray(pos_max, np.float32)
        t = np.float32(tol)
        keep &= np.all((r >= pmin - t) & (r < pmax + t), axis=1)
    r = r[keep]
    coords = []
    for k in range(ndim):
        if phase_rounding:
            ax = np.asarray(axis[k], np.float32)
            d = (r - np.asarray(centre, np.float32)).astype(np.float32)
            pr = np.float32(0.0) * d[:, 0]
            for b in range(3):
                pr = (pr + (ax[b] * d[:, b]).astype(np.float32)).astype(np.float32)
            coords.append((pr * np.float32(tpe[k])).astype(np.float32).astype(np.float64))
        else:
            d = r.astype(np.float64) - np.asarray(centre, np.float64)
            coords.append((d @ np.asarray(axis[k], np.float64)) * float(tpe[k]))
    qc = np.asarray(q_center, np.float64)
    if np.any(qc != 0):
        if phase_rounding:
            tq = (np.float32(2 * np.pi) * qc.astype(np.float32)).astype(np.float32)
            arg = np.zeros(len(r), np.float32)
            for b in range(3):
                arg = (arg + (tq[b] * r[:, b]).astype(np.float32)).astype(np.float32)
            c = np.exp(-1j * arg.astype(np.float64))
        else:
            turns = r.astype(np.float64) @ qc
            c = np.exp(-2j * np.pi * (turns - np.floor(turns)))
    else:
        c = np.ones(len(r), np.complex128)
    if window:
        nw = 2 if ndim == 2 else 3
        for k in range(nw):
            c = c * (1.0 + np.cos(coords[k]))
    return coords, c


def xray_ff(xff, qsq_kappa):
    """f = c + sum_i a_i exp(-b_i * s2) with s2 = kappa |Q|^2, xff = (a1 b1 .. a4 b4 c)."""
    xff = np.asarray(xff, np.float64)
    f = np.full_like(qsq_kappa, xff[8], dtype=np.float64)
    for i in range(4):
        f = f + xff[2 * i] * np.exp(-xff[2 * i + 1] * qsq_kappa)
    return f


def weighted_sum(amps, weights, mask=None, wnorm=1.0):
    """cs(t,Q) = sum_j mask_j w_j(Q) A_j(t,Q) (:1338-1356).  amps (F, S, nQ), weights (S, nQ)
    or (S,)."""
    amps = np.asarray(amps)
    S = amps.shape[1]
    mask = np.ones(S) if mask is None else np.asarray(mask)
    w = np.asarray(weights, np.float64)
    if w.ndim == 1:
        w = w[:, None]
    cs = np.zeros((amps.shape[0], amps.shape[2]), np.complex128)
    for j in range(S):
        if mask[j]:
            cs += w[j][None, :] * amps[:, j, :]
    return cs * wnorm


def centered(cs, q2_norm=None):
    """cs - <cs>_t (mean over frames, :1177-1185), times 1/|Q| if given (:1373)."""
    x = cs - cs.mean(axis=0, keepdims=True)
    if q2_norm is not None:
        x = x * np.asarray(q2_norm)[None, :]
    return x


def sq_total(cs, norm2=1.0):
    """S(Q) = sum_t |cs|^2 / nfile / norm2 (:1381-1387, :1573-1574)."""
    return (np.abs(cs) ** 2).sum(axis=0) / cs.shape[0] / norm2


def hann_window(n_int, variant="symmetric"):
    """t_wind of :941-948 ('symmetric', denominator n_int-1) or of :2429-2431 ('options')."""
    i = np.arange(1, n_int + 1, dtype=np.float64)
    if n_int <= 1:
        return np.ones(n_int)
    if variant == "symmetric":
        return 0.5 * (1.0 - np.cos(2 * np.pi * (i - 1) / (n_int - 1)))
    return 0.5 * (1.0 - np.cos(2 * np.pi * i / (n_int + 1)))


def econst(cs, n_int, t_wind, j_freq, q2_norm=None, scale=1.0, center=True):
    """E=const map for 1-based bin j_freq (:1437-1478): sum over start frames of
    |sum_i om_phase_i x(t0+i)|^2, om_phase_i = t_wind_i exp(-2 pi i (j_freq-1)(i-n_int/2-1)/n_int).
    center=False takes cs as is: the atom-pair form (:1460-1464), where cs is the sum of two
    species' raw amplitudes."""
    x = centered(cs, q2_norm) if center else np.asarray(cs)
    F = x.shape[0]
    i = np.arange(1, n_int + 1)
    ph = np.asarray(t_wind) * np.exp(-2j * np.pi * (j_freq - 1) * (i - n_int // 2 - 1) / n_int)
    n0 = F - n_int + 1
    out = np.zeros(x.shape[1])
    for t0 in range(n0):
        X = ph @ x[t0:t0 + n_int]
        out += np.abs(X) ** 2
    return out * scale


def dispersion(cs, n_int, t_wind, q_index, n_freq, q2_norm=None, scale=1.0, center=True):
    """E(Q) cut (:1480-1517): for each path index, sum over start frames of
    |FFT(t_wind * x(t0 : t0+n_int))[0:n_freq]|^2 (forward, unscaled).  Returns (n_path, n_freq).
    center=False: the atom-pair form (:1494-1499) on the raw sum of two species."""
    x = (centered(cs, q2_norm) if center else np.asarray(cs))[:, np.asarray(q_index)]
    F = x.shape[0]
    n0 = F - n_int + 1
    out = np.zeros((x.shape[1], n_freq))
    w = np.asarray(t_wind)[:, None]
    for t0 in range(n0):
        X = np.fft.fft(w * x[t0:t0 + n_int], axis=0)[:n_freq]
        out += (np.abs(X) ** 2).T
    return out * scale


def iqt_map(cs, n_int, lag, q2_norm=None, scale=1.0):
    """I(Q,t) map at time lag `lag` (frames), the j_sq /= 1 branch of :1467-1472: the real
    part of sum_{i<n_int} x(i+lag) conj(x(i)) / n_int, x = centred (1/|Q|-scaled) amplitudes."""
    x = centered(cs, q2_norm)
    v = (x[lag:lag + n_int] * np.conj(x[:n_int])).sum(axis=0) / n_int
    return v.real * scale


def iqt_dispersion(cs, n_int, q_index, q2_norm=None, scale=1.0):
    """I(Q,t) along a path (:1504-1510, n_freq_max = nfile - n_int + 1 at :699): out[p, t] =
    Re sum_{i<n_int} x(t+i, q_p) conj(x(i, q_p)) for t = 0..nfile-n_int."""
    x = centered(cs, q2_norm)[:, np.asarray(q_index)]
    F = x.shape[0]
    n_lag = F - n_int + 1
    out = np.zeros((x.shape[1], n_lag))
    for t in range(n_lag):
        out[:, t] = (x[t:t + n_int] * np.conj(x[:n_int])).sum(axis=0).real
    return out * scale


def gauss_window(n_frames, fwhm):
    t = np.arange(n_frames)
    tc = 0.5 * (n_frames - 1)
    return np.exp(-4.0 * np.log(2.0) * ((t - tc) / fwhm) ** 2)


def gauss_spectrum(cs, fwhm, n_freq, q2_norm=None, scale=1.0):
    """|sum_t g_t (cs_t - <cs>) exp(-2 pi i k t / F)|^2 for k < n_freq; returns (n_freq, nQ)."""
    x = centered(cs, q2_norm)
    g = gauss_window(x.shape[0], fwhm)[:, None]
    X = np.fft.fft(g * x, axis=0)[:n_freq]
    return np.abs(X) ** 2 * scale


def _speckle_walk(csp, s_trig):
    """One walk of :1541-1548 over a flat float32 array, in place and in the reference's
    order: the left neighbour is already filtered, the right one not (except that the last
    value's right neighbour is the filtered first value); wrap-around at both ends."""
    s = np.float32(s_trig)
    n = csp.size
    for i2 in range(n):
        a = csp[i2 - 1]                    # i1 = i2 - 1, wrapping to the last value
        b = csp[(i2 + 1) % n]              # i3 = i2 + 1, wrapping to the (filtered) first
        lo, hi = min(a, b), max(a, b)
        if csp[i2] < np.float32(lo / s):
            csp[i2] = lo
        if csp[i2] > np.float32(s * hi):
            csp[i2] = hi


def speckle_filter(cs_plot, s_trig, dispersion=False):
    """The speckle filter of :1531-1570 on a finished map (float32).

    Plane maps (dispersion False) are given as an (n_qy, n_qx) array, i.e. the reference's
    cs_plot(n_qx, n_qy) with qx contiguous: a walk over the flattened map, then a walk over
    the transposed map.  E(Q) cuts (dispersion True) are given as (n_qdisp, n_freq) with the
    frequency contiguous, the reference's cs_plot(n_freq_max, n_qdisp) after :1538: one walk."""
    m = np.array(cs_plot, dtype=np.float32, copy=True)
    shape = m.shape
    flat = m.reshape(-1)
    _speckle_walk(flat, s_trig)
    if not dispersion:
        t = np.ascontiguousarray(flat.reshape(shape).T)
        tf = t.reshape(-1)
        _speckle_walk(tf, s_trig)
        return np.ascontiguousarray(tf.reshape(t.shape).T)
    return flat.reshape(shape)


def one_phonon(frame, at_ind, counts, at_base, n_row, n_bz, qx_min, qy_min, plane, n_q):
    """Per-species one-phonon amplitudes of one frame (:1037-1098), shape (S, n_qy, n_qx),
    complex128; pixels beyond the n_bz x n_bz zones are 0 (the reference leaves them unset).
    Displacements in FP32 in the reference's order, sums and transforms in FP64."""
    f = np.float32
    n1, n2 = int(n_row[0]), int(n_row[1])
    nqx, nqy = int(n_q[0]), int(n_q[1])
    off = np.concatenate([[0], np.cumsum(counts)])
    S = len(counts)
    out = np.zeros((S, nqy, nqx), np.complex128)
    qx_min, qy_min = f(qx_min), f(qy_min)
    nqx_min = int(f(f(n1) * f(qx_min - np.floor(qx_min))))        # :1039-1040, truncation
    nqy_min = int(f(f(n2) * f(qy_min - np.floor(qy_min))))
    for j in range(S):
        r = frame[off[j]:off[j + 1], :3].astype(f)
        c = at_ind[off[j]:off[j + 1], :3].astype(np.int64)
        b = np.asarray(at_base[j], f)
        keep = ~((r[:, 0] == 0) & (r[:, 1] == 0) & (r[:, 2] == 0))   # vacancies (:1049)
        r, c = r[keep], c[keep]
        if plane == 1:                                                # :1046-1057
            k, l = c[:, 0], c[:, 1]
            dx = ((r[:, 0] - b[0]) - c[:, 0].astype(f)) + f(n_row[0] // 2)
            dy = ((r[:, 1] - b[1]) - c[:, 1].astype(f)) + f(n_row[1] // 2)
        else:                                                         # :1059-1071
            k = np.mod(c[:, 0] - 1 + c[:, 1] - 1, (n_row[0] + n_row[1]) // 2) + 1
            l = c[:, 2]
            t = (((r[:, 0] - b[0]) - c[:, 0].astype(f)) + f(n_row[0] // 2)) + f(1)
            t = ((((t + r[:, 1]) - b[1]) - c[:, 1].astype(f)) + f(n_row[1] // 2)) + f(1)
            dx = (t / f(np.sqrt(f(2.0)))).astype(f)
            dy = ((((r[:, 2] - b[2]) - c[:, 2].astype(f)) + f(n_row[2] // 2)) + f(1)).astype(f)
        ux = np.zeros((n2, n1))
        uy = np.zeros((n2, n1))
        np.add.at(ux, (l - 1, k - 1), dx.astype(np.float64))
        np.add.at(uy, (l - 1, k - 1), dy.astype(np.float64))
        uqx = np.fft.fft2(ux) / n1                                    # forward exp(-i), :1075
        uqy = np.fft.fft2(uy) / n2
        for jj in range(int(n_bz)):
            for ii in range(int(n_bz)):
                kk = np.arange(1, n1 + 1)
                ll = np.arange(1, n2 + 1)
                qx = (f(qx_min + f(ii)) + (f(1) * (kk - 1).astype(f)) / f(n1)).astype(f)
                qy = (f(qy_min + f(jj)) + (f(1) * (ll - 1).astype(f)) / f(n2)).astype(f)
                ik = np.mod(nqx_min + kk, n1)
                ik[ik == 0] = n1
                il = np.mod(nqy_min + ll, n2)
                il[il == 0] = n2
                QX, QY = np.meshgrid(qx.astype(np.float64), qy.astype(np.float64))
                IK, IL = np.meshgrid(ik - 1, il - 1)
                if plane == 1:
                    dot = f(qx[None, :] * b[0]) + f(qy[:, None] * b[1])
                else:
                    dot = f(qx[None, :] * f(b[0] + b[1])) + f(qy[:, None] * b[2])
                arg = (f(2.0 * np.pi) * dot.astype(f)).astype(np.float64)
                val = np.exp(-1j * arg) * (QX * uqx[IL, IK] + QY * uqy[IL, IK])
                out[j, jj * n2:(jj + 1) * n2, ii * n1:(ii + 1) * n1] = val
    return out
