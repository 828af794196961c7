"""One-phonon mode (mp_sqom's j_oneph = 1, code/src/mp_sqom56.f90:1037-1098).

The reference ships no output of this mode, so the oracle's restatement is pinned on physics
(CPU): on the (hk0) plane the one-phonon amplitude is the first-order term of the exact
transform, A_exact(Q) = +-2 pi i n_row A_1ph(Q) + O((Q.u)^2) at every non-Bragg pixel
(the sign alternates with the pixel parity through the centred cell origin), checked against
the oracle's FP64 direct sum; and a single displaced atom gives the closed form.  On (hhl)
the reference places the one-phonon pixels at steps of 1/n_row along [hh0], which is not the
Q grid of its NUFFT path there (n_qx = n_bz n_row sqrt 2), so only the restatement applies.
GPU: the job's one-phonon amplitudes (both planes, FP32 and FP64, neutron and X-ray weights,
a vacancy) equal the oracle's weighted per-species amplitudes to FP32 / FP64 rounding and feed
the usual time-axis maps."""
import numpy as np
import pytest

import oracle
from helpers import abo3_cell, rel_l2
from mp_tools_gb300 import _lib
from mp_tools_gb300.sqom import QGrid
from oracle import sqom_ref

BASE = np.array([[0, 0, 0], [0.5, 0.5, 0.5], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]],
                np.float32)


def _exact_plane_amplitudes(pos, counts, grid):
    off = np.concatenate([[0], np.cumsum(counts)])
    out = []
    for s in range(len(counts)):
        coords, c = sqom_ref.prep_points(
            pos, off[s], off[s + 1], input_method=grid.input_method, ndim=2, axis=grid.axis,
            tpe=grid.tpe, centre=grid.at_pos_centre, q_center=grid.q_center, window=False,
            phase_rounding=False, pos_min=grid.at_pos_min, pos_max=grid.at_pos_max, tol=0.1)
        f = oracle.dirft2d1(coords[0], coords[1], c, -1, grid.n_q[0], grid.n_q[1])
        out.append(f.reshape(grid.n_q[1], grid.n_q[0]))
    return np.stack(out)


@pytest.mark.parametrize("n,q_center", [(6, (0, 0, 0)), (4, (0.5, 0.25, 0)), (5, (0, 0, 0))])
def test_oracle_is_first_order_of_exact_transform(n, q_center):
    """Small displacements (0.004 A): at the non-Bragg pixels of a commensurate plane (n_row q on
    integers), A_exact = -2 pi i n_row exp(2 pi i (n_row//2)(q_x + q_y)) A_1ph to second order
    (the phase factor is the centred cell origin); the reference's truncated nqx_min puts the
    one-phonon pixels off their Q when n_row q_min is not an integer."""
    pos, ind, counts = abo3_cell(n, np.random.default_rng(3), sigma=(0.004, 0.004, 0.004))
    grid = QGrid(_lib.CELL, (n, n, n), n_bz=2, q_center=q_center, a_par=(4.19,) * 3)
    a1 = sqom_ref.one_phonon(pos, ind, counts, BASE, (n, n, n), 2, grid.q_min[0], grid.q_min[1],
                             1, grid.n_q)
    ex = _exact_plane_amplitudes(pos, counts, grid)
    qx, qy = np.meshgrid(grid.axis_values(0).astype(float), grid.axis_values(1).astype(float))
    bragg = (np.abs(qx - np.round(qx)) < 1e-6) & (np.abs(qy - np.round(qy)) < 1e-6)
    assert (~bragg).sum() > 0.9 * bragg.size
    pattern = -2j * np.pi * n * np.exp(2j * np.pi * (n // 2) * (qx + qy))
    for s in range(len(counts)):
        assert rel_l2(ex[s][~bragg], (pattern * a1[s])[~bragg]) < 1e-2, s


def test_oracle_single_displaced_atom_closed_form():
    n = 4
    pos, ind, counts = abo3_cell(n, np.random.default_rng(0), sigma=(0, 0, 0))
    # every atom sits at cell + base - n/2 (d = -1 on (hk0)); displace one atom of species 1
    pos = pos.copy()
    a = counts[0] + 9
    delta = np.float32(0.03)
    pos[a, 0] += delta
    k0, l0 = int(ind[a, 0]), int(ind[a, 1])
    grid = QGrid(_lib.CELL, (n, n, n), n_bz=1, q_center=(0.25, 0, 0), a_par=(4.19,) * 3)
    out = sqom_ref.one_phonon(pos, ind, counts, BASE, (n, n, n), 1, grid.q_min[0], grid.q_min[1],
                              1, grid.n_q)
    f32 = np.float32
    nqx_min = int(f32(n * (grid.q_min[0] - np.floor(grid.q_min[0]))))
    nqy_min = int(f32(n * (grid.q_min[1] - np.floor(grid.q_min[1]))))
    b = BASE[1]
    for (x, y) in ((1, 0), (2, 3), (3, 1)):     # pixels away from the zone centre
        qx = float(f32(grid.q_min[0]) + f32(x) / f32(n))
        qy = float(f32(grid.q_min[1]) + f32(y) / f32(n))
        kk = (nqx_min + x + 1) % n or n
        ll = (nqy_min + y + 1) % n or n
        # u_x = delta at (k0, l0) plus the constant -1 per atom (only at kk = ll = 1)
        uqx = (delta * np.exp(-2j * np.pi * ((kk - 1) * (k0 - 1) + (ll - 1) * (l0 - 1)) / n)
               + (-(n ** 3) if (kk, ll) == (1, 1) else 0)) / n
        uqy = (-(n ** 3) if (kk, ll) == (1, 1) else 0) / n
        want = np.exp(-2j * np.pi * (qx * b[0] + qy * b[1])) * (qx * uqx + qy * uqy)
        assert abs(out[1, y, x] - want) < 1e-6 * max(1.0, abs(want)), (x, y)


def _cell_frames(n, F, seed, sigma=0.01):
    rng = np.random.default_rng(seed)
    base, ind, counts = abo3_cell(n, rng)
    frames = np.repeat(base[None], F, axis=0).copy()
    frames[:, :, :3] += rng.normal(0, sigma, size=frames[:, :, :3].shape).astype(np.float32)
    return frames, ind, counts


def _xray_weights(grid, xff, kappa=1 / 16.0):
    """Cromer-Mann f_s(Q) per pixel as the job evaluates them (mp_sqom's s^2 = kappa |Q|^2)."""
    origin, steps, extra = grid.qphys()
    k = [np.arange(n) - n // 2 for n in grid.n_q]
    kz, ky, kx = np.meshgrid(k[2], k[1], k[0], indexing="ij")
    Q = (origin[None, :] + kx.reshape(-1, 1) * steps[0] + ky.reshape(-1, 1) * steps[1]
         + kz.reshape(-1, 1) * steps[2])
    s2 = kappa * ((Q ** 2).sum(1) + extra)
    return np.stack([sqom_ref.xray_ff(x, s2) for x in xff])


@pytest.mark.gpu
@pytest.mark.parametrize("plane", [1, 2])
@pytest.mark.parametrize("prec,tol", [(_lib.FP32, 2e-5), (_lib.FP64, 1e-9)])
@pytest.mark.parametrize("weight", ["neutron", "xray"])
def test_gpu_one_phonon_equals_oracle(cuda, plane, prec, tol, weight):
    from mp_tools_gb300.sqom import SqomJob, TimeAxis
    n, F = 6, 6
    frames, ind, counts = _cell_frames(n, F, seed=plane)
    frames[:, 3, :3] = 0.0                          # a vacancy
    if plane == 1:
        grid = QGrid(_lib.CELL, (n, n, n), n_bz=3, q_center=(0.5, 0, 0), a_par=(4.19,) * 3)
    else:
        grid = QGrid(_lib.CELL, (n, n, n), e1=(1, 1, 0), e2=(0, 0, 1), n_bz=2, a_par=(4.19,) * 3)
    S = len(counts)
    if weight == "neutron":
        b = [0.507, 0.716, 0.5803, 0.5803, 0.5803]
        kw = dict(weight_mode=_lib.WEIGHT_NEUTRON, b_coh=b)
        w = np.repeat(np.asarray(b)[:, None], grid.n_modes, axis=1)
    else:
        xff = [[6.4202, 3.0387, 1.9002, 0.7426, 1.5936, 31.5472, 1.9646, 85.0886, 1.1151],
               [36.0228, 0.5293, 23.4128, 3.3253, 14.9491, 16.0927, 4.1880, 100.6130, 13.3966]]
        xff = [xff[s % 2] for s in range(S)]
        kw = dict(weight_mode=_lib.WEIGHT_XRAY, xff=xff)
        w = _xray_weights(grid, xff)
    job = SqomJob(grid, species_counts=counts, n_frames=F, precision=prec, eps=1e-6,
                  n_atoms_frame=frames.shape[1], **kw)
    try:
        job.set_cell_index(ind)
        job.set_frames(frames)
        job.transform_onephonon(plane, BASE)
        job.sync()
        amps = job.amplitudes()
        want = np.empty((F, grid.n_modes), np.complex128)
        for t in range(F):
            a = sqom_ref.one_phonon(frames[t], ind, counts, BASE, (n, n, n), grid.n_bz,
                                    grid.q_min[0], grid.q_min[1], plane, grid.n_q)
            want[t] = (w * a.reshape(S, -1)).sum(0)
        assert rel_l2(amps, want) < tol
        # the usual time-axis maps run on these amplitudes
        ta = TimeAxis(nfile=F, t_step=0.01)
        got = job.sqw_econst(ta, 1, normalize=False)
        ref = sqom_ref.econst(want, ta.n_int, ta.window(), 1, None,
                              1.0 / (0.5 * ta.n_frame * ta.n_int))
        assert rel_l2(got, ref) < max(tol, 1e-6) * 10
    finally:
        job.close()


@pytest.mark.gpu
def test_gpu_one_phonon_rejects_unsupported_input(cuda):
    from mp_tools_gb300.sqom import SqomJob
    frames, ind, counts = _cell_frames(4, 2, seed=0)
    grid = QGrid(_lib.CELL, (4, 4, 4), n_bz=2, a_par=(4.19,) * 3)
    job = SqomJob(grid, species_counts=counts, n_frames=2, precision=_lib.FP32, eps=1e-6,
                  n_atoms_frame=frames.shape[1])
    try:
        job.set_frames(frames)
        with pytest.raises(RuntimeError, match="cell indices"):
            job.transform_onephonon(1, BASE)
        job.set_cell_index(ind)
        with pytest.raises(RuntimeError, match="plane"):
            job.transform_onephonon(3, BASE)
    finally:
        job.close()
